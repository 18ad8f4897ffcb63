// The batched radiation-field launch: the kernel instantiated over (model,
// node) work items of many models (the batch of batch.cu).  Compiled apart
// from rf.cu so the two sets of instantiations build in parallel.
#include "rf_kernel.cuh"

namespace {

// the batched kernel for a channel layout and line group
template <int NS, int RT>
const void *batch_kernel_ns(bool dust, int nlg) {
    if (RT) return (const void *)k_radiation_field<NS, 5, false, true, RT>;
    if (nlg == 10)
        return dust ? (const void *)k_radiation_field<NS, 10, true, true, 0>
                    : (const void *)k_radiation_field<NS, 10, false, true, 0>;
    return dust ? (const void *)k_radiation_field<NS, 5, true, true, 0>
                : (const void *)k_radiation_field<NS, 5, false, true, 0>;
}
const void *batch_kernel(int nch, bool dust, int nlg, int max_lines) {
    const ChanLayout cl = chan_layout(nch, dust, max_lines);
    if (cl.rt) {
        switch (cl.ns) {
        case 1: return batch_kernel_ns<1, 1>(dust, nlg);
        case 2: return batch_kernel_ns<2, 1>(dust, nlg);
        case 4: return batch_kernel_ns<4, 1>(dust, nlg);
        default: return batch_kernel_ns<8, 1>(dust, nlg);
        }
    }
    switch (cl.ns) {
    case 1: return batch_kernel_ns<1, 0>(dust, nlg);
    case 2: return batch_kernel_ns<2, 0>(dust, nlg);
    case 3: return batch_kernel_ns<3, 0>(dust, nlg);
    case 5: return batch_kernel_ns<5, 0>(dust, nlg);
    default: return batch_kernel_ns<9, 0>(dust, nlg);
    }
}

}  // namespace

namespace portal {

const void *rf_batch_kernel_ptr(int nch, bool dust, int nlg, int max_lines) {
    return batch_kernel(nch, dust, nlg, max_lines);
}

// dynamic shared memory of a 256-thread block: the remainder channel's
// (cell, line) table of each of its 8 warps, rows for the largest model
static size_t batch_dyn_smem(int nch, bool dust, int max_lines) {
    return chan_layout(nch, dust, max_lines).rt ? (size_t)8 * 32 * rem_row_stride(max_lines) * sizeof(float2) : 0;
}

// Also raises the kernel's dynamic shared-memory limit: called for every
// candidate before the pass is captured.
int rf_batch_blocks_per_sm(int nch, bool dust, int nlg, int max_lines, int *blocks) {
    const void *k = batch_kernel(nch, dust, nlg, max_lines);
    const size_t dyn = batch_dyn_smem(nch, dust, max_lines);
    *blocks = 0;
    if (dyn && cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn) != cudaSuccess)
        return PORTAL_ERR_CUDA;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k, 256, dyn);
    return e == cudaSuccess ? PORTAL_OK : PORTAL_ERR_CUDA;
}

int rf_batch_launch(cudaStream_t s, int grid, int nch, bool dust, int nlg, int max_lines, const RFBatch &bw) {
    const void *k = batch_kernel(nch, dust, nlg, max_lines);
    RFArgs a0{};
    RFBatch b = bw;
    b.rem_lines = max_lines;
    void *args[] = {&a0, &b};
    cudaError_t e = cudaLaunchKernel(k, dim3(grid), dim3(256), args, batch_dyn_smem(nch, dust, max_lines), s);
    return e == cudaSuccess ? PORTAL_OK : PORTAL_ERR_CUDA;
}

}  // namespace portal
