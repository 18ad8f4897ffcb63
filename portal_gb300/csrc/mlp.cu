// Learned warm start for the Lambda iteration: a small MLP trained on the
// GPU with the library's own kernels (no reference counterpart).
//
// Network: n_in -> width (SiLU) -> ... (depth hidden layers) -> n_out
// (linear).  Parameters are FP32 master copies; every GEMM rounds its
// operands to BF16 (weights and activations) and accumulates in FP32 on the
// tensor cores: the forward GEMMs (inference and training) with tcgen05
// (k_gemm_tc, accumulator in tensor memory), the backward GEMMs, whose
// operands are transposed, with mma.sync m16n8k16 (k_gemm).  Inputs and
// targets are standardised with statistics stored in the model.
//
// GEMM kernel: C(M,N) = A(M,K) B(K,N) with 64x64 block tiles, 4 warps of
// 32x32, K steps of 32 staged in shared memory as BF16 (K-contiguous rows,
// padded), and fused epilogues:
//   forward hidden   Z = C + b, H = silu(Z)     (Z kept for the backward)
//   forward output   Y = C + b
//   backward dX      dZ_prev = C * silu'(Z_prev)
//   backward dW      G = C
// The operand layouts are template flags: A K-contiguous (row-major M x K)
// or M-contiguous; B K-contiguous (stored N x K) or N-contiguous.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "common.cuh"
#include "umma.cuh"

using namespace portal;

namespace {

enum Epi { EPI_STORE = 0, EPI_BIAS = 1, EPI_BIAS_SILU = 2, EPI_DSILU = 3 };

struct EpiArgs {
    int kind, ldc;
    float *C;          // output (G, Y, H or dZ)
    float *Z;          // pre-activation out (EPI_BIAS_SILU) or in (EPI_DSILU)
    const float *bias;
};

__device__ __forceinline__ float sigm(float z) { return 1.f / (1.f + __expf(-z)); }

template <bool AK, bool BK>
__global__ void __launch_bounds__(128) k_gemm(int M, int N, int K, const float *__restrict__ A, int lda,
                                              const float *__restrict__ B, int ldb, EpiArgs e) {
    __shared__ __align__(16) __nv_bfloat16 As[64][40];
    __shared__ __align__(16) __nv_bfloat16 Bs[64][40];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int wm = w >> 1, wn = w & 1, g = lane >> 2, t = lane & 3;
    const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int q = 0; q < 4; q++) acc[i][j][q] = 0.f;
    for (int k0 = 0; k0 < K; k0 += 32) {
        for (int i = tid; i < 64 * 32; i += 128) {
            int r, kk;
            if (AK) { r = i >> 5; kk = i & 31; } else { kk = i >> 6; r = i & 63; }
            const int gm = m0 + r, gk = k0 + kk;
            float v = 0.f;
            if (gm < M && gk < K) v = AK ? A[(size_t)gm * lda + gk] : A[(size_t)gk * lda + gm];
            As[r][kk] = __float2bfloat16(v);
        }
        for (int i = tid; i < 64 * 32; i += 128) {
            int c, kk;
            if (BK) { c = i >> 5; kk = i & 31; } else { kk = i >> 6; c = i & 63; }
            const int gn = n0 + c, gk = k0 + kk;
            float v = 0.f;
            if (gn < N && gk < K) v = BK ? B[(size_t)gn * ldb + gk] : B[(size_t)gk * ldb + gn];
            Bs[c][kk] = __float2bfloat16(v);
        }
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < 32; ks += 16) {
            uint32_t af[2][4], bfr[4][2];
#pragma unroll
            for (int mi = 0; mi < 2; mi++) {
                const int rb = wm * 32 + mi * 16;
                af[mi][0] = *(const uint32_t *)&As[rb + g][ks + 2 * t];
                af[mi][1] = *(const uint32_t *)&As[rb + g + 8][ks + 2 * t];
                af[mi][2] = *(const uint32_t *)&As[rb + g][ks + 2 * t + 8];
                af[mi][3] = *(const uint32_t *)&As[rb + g + 8][ks + 2 * t + 8];
            }
#pragma unroll
            for (int ni = 0; ni < 4; ni++) {
                const int cb = wn * 32 + ni * 8;
                bfr[ni][0] = *(const uint32_t *)&Bs[cb + g][ks + 2 * t];
                bfr[ni][1] = *(const uint32_t *)&Bs[cb + g][ks + 2 * t + 8];
            }
#pragma unroll
            for (int mi = 0; mi < 2; mi++)
#pragma unroll
                for (int ni = 0; ni < 4; ni++)
                    asm volatile(
                        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
                        "{%8,%9}, {%0,%1,%2,%3};\n"
                        : "+f"(acc[mi][ni][0]), "+f"(acc[mi][ni][1]), "+f"(acc[mi][ni][2]), "+f"(acc[mi][ni][3])
                        : "r"(af[mi][0]), "r"(af[mi][1]), "r"(af[mi][2]), "r"(af[mi][3]), "r"(bfr[ni][0]),
                          "r"(bfr[ni][1]));
        }
        __syncthreads();
    }
#pragma unroll
    for (int mi = 0; mi < 2; mi++)
#pragma unroll
        for (int ni = 0; ni < 4; ni++)
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int r = m0 + wm * 32 + mi * 16 + g + ((q & 2) ? 8 : 0);
                const int c = n0 + wn * 32 + ni * 8 + 2 * t + (q & 1);
                if (r >= M || c >= N) continue;
                const float v = acc[mi][ni][q];
                const size_t o = (size_t)r * e.ldc + c;
                switch (e.kind) {
                case EPI_STORE: e.C[o] = v; break;
                case EPI_BIAS: e.C[o] = v + e.bias[c]; break;
                case EPI_BIAS_SILU: {
                    const float z = v + e.bias[c];
                    e.Z[o] = z;
                    e.C[o] = z * sigm(z);
                    break;
                }
                case EPI_DSILU: {
                    const float z = e.Z[o], s = sigm(z);
                    e.C[o] = v * s * (1.f + z * (1.f - s));
                    break;
                }
                }
            }
}

// ---- the forward GEMMs on the 5th-generation tensor cores ------------------
// C(M, N) = A(M, K) W(N, K)^T with the fused epilogues above, for K, N <= 256.
// Persistent CTAs of 4 warps (one per SM, the grid at most the SM count):
// each converts all of W to BF16 in shared memory once, then for each of its
// 128-row tiles of A converts the rows to BF16 beside it, one thread issues
// the Kp/16 MMAs of shape 128 x Np x 16 into an FP32 accumulator in tensor
// memory and commits them to an mbarrier, and each warp reads its 32 rows
// back with tcgen05.ld for the epilogue.  Shared-memory operands use the
// canonical no-swizzle K-major layout: 8-row x 16-byte core matrices,
// K-adjacent ones 128 B apart, row groups Kp/8 x 128 B apart (K and N
// zero-padded to multiples of 16).  Waits are bounded: a timeout sets *err,
// the CTA stops and still frees its tensor memory.
constexpr int TC_M = 128;

// the A tile's region doubles as the epilogue's transpose buffer (4 KB per
// warp of 512 threads) once a tile's MMAs are complete
constexpr int TC_EPI_BYTES = 16 * 32 * 32 * 4;
__host__ __device__ inline size_t tc_a_bytes(int Kp) {
    return (size_t)TC_M * Kp * 2 > (size_t)TC_EPI_BYTES ? (size_t)TC_M * Kp * 2 : (size_t)TC_EPI_BYTES;
}
__host__ __device__ inline size_t tc_smem_bytes(int Np, int Kp) {
    return tc_a_bytes(Kp) + (size_t)Np * Kp * 2 + 16;
}

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t *>(&h);
}

// rows [r0, r0 + rows) of the row-major src (ld floats per row, K valid
// columns, nrow_valid valid rows) into the canonical BF16 tile; each thread
// first loads TC_U chunks (two float4 each) and then converts them, so that
// many loads are in flight per thread
constexpr int TC_THREADS = 512;
constexpr int TC_U = 4;

__device__ __forceinline__ void tc_load8(const float *p, bool valid, int nk, float *v) {
    if (valid && nk >= 8 && ((reinterpret_cast<uintptr_t>(p) & 15) == 0)) {
        const float4 x = __ldg(reinterpret_cast<const float4 *>(p));
        const float4 y = __ldg(reinterpret_cast<const float4 *>(p) + 1);
        v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
        v[4] = y.x; v[5] = y.y; v[6] = y.z; v[7] = y.w;
    } else {
#pragma unroll
        for (int j = 0; j < 8; j++) v[j] = (valid && j < nk) ? p[j] : 0.f;
    }
}

__device__ __forceinline__ void tc_stage(unsigned char *tile, int rows, int Kp, const float *__restrict__ src,
                                         int r0, int nrow_valid, int K, int ld, int tid) {
    const int kc = Kp / 8;
    const uint32_t sbo = (uint32_t)kc * 128;
    const int total = rows * kc;
    for (int base = tid; base < total; base += TC_THREADS * TC_U) {
        float v[TC_U][8];
#pragma unroll
        for (int u = 0; u < TC_U; u++) {
            const int i = base + u * TC_THREADS;
            const int r = i / kc, c = i - r * kc;
            tc_load8(src + (size_t)(r0 + r) * ld + c * 8, i < total && r < nrow_valid, K - c * 8, v[u]);
        }
#pragma unroll
        for (int u = 0; u < TC_U; u++) {
            const int i = base + u * TC_THREADS;
            if (i >= total) break;
            const int r = i / kc, c = i - r * kc;
            uint4 q;
            q.x = pack_bf16x2(v[u][0], v[u][1]);
            q.y = pack_bf16x2(v[u][2], v[u][3]);
            q.z = pack_bf16x2(v[u][4], v[u][5]);
            q.w = pack_bf16x2(v[u][6], v[u][7]);
            *reinterpret_cast<uint4 *>(tile + (size_t)(r >> 3) * sbo + (size_t)c * 128 + (size_t)(r & 7) * 16) = q;
        }
    }
}

__global__ void __launch_bounds__(TC_THREADS, 1) k_gemm_tc(int M, int N, int K, int Np, int Kp, uint32_t tcols,
                                                           const float *__restrict__ A, const float *__restrict__ W,
                                                           EpiArgs e, int *err) {
    extern __shared__ __align__(1024) unsigned char tsm[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    unsigned char *As = tsm;
    unsigned char *Bs = tsm + tc_a_bytes(Kp);
    uint64_t *bar = reinterpret_cast<uint64_t *>(Bs + (size_t)Np * Kp * 2);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(bar + 1);
    float *T = reinterpret_cast<float *>(As) + (size_t)warp * 32 * 32;  // this warp's 32 x 32 transpose buffer
    tc_stage(Bs, Np, Kp, W, 0, N, K, K, tid);
    if (warp == 0) umma::tmem_alloc(tslot, tcols);
    if (tid == 0) {
        umma::mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t taddr = *tslot;
    const uint32_t idesc = umma::idesc_bf16_f32(TC_M, Np);
    const uint32_t sbo = (uint32_t)(Kp / 8) * 128;
    const int ntiles = (M + TC_M - 1) / TC_M;
    // epilogue split: warp w reads the lane quarter w % 4 (tcgen05.ld's rule)
    // and every (TC_THREADS / 128)-th 32-column chunk from chunk w / 4
    const int quarter = warp & 3, cgroup = warp >> 2, ngroups = TC_THREADS / 128;
    int iter = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, iter++) {
        const int m0 = t * TC_M;
        tc_stage(As, TC_M, Kp, A, m0, min(TC_M, M - m0), K, K, tid);
        umma::fence_proxy_async();
        umma::fence_before_sync();
        __syncthreads();   // A staged; the previous tile's accumulator reads are done
        umma::fence_after_sync();
        if (tid == 0) {
            const uint32_t a0 = umma::smem_addr(As), b0 = umma::smem_addr(Bs);
            for (int ks = 0; ks < Kp / 16; ks++)
                umma::mma_bf16(taddr, umma::smem_desc(a0 + ks * 256, 128, sbo),
                               umma::smem_desc(b0 + ks * 256, 128, sbo), idesc, ks > 0);
            umma::mma_commit(bar);
        }
        bool done = false;
        for (int it = 0; it < (1 << 24) && !done; it++) done = umma::mbar_try_wait(bar, (uint32_t)(iter & 1));
        ok = __syncthreads_and(done);
        umma::fence_after_sync();
        if (!ok) {
            if (tid == 0) atomicExch(err, 1);
            break;
        }
        // epilogue: thread t of the warp holds row (rbase + t), columns c0..c0+31;
        // through the warp's transpose buffer (XOR-swizzled, no bank
        // conflicts) each store instruction then writes 32 consecutive
        // columns of one row
        const int rbase = m0 + quarter * 32;
        for (int c0 = cgroup * 32; c0 < Np; c0 += 32 * ngroups) {
            float v[32];
            umma::tmem_ld32(taddr + ((uint32_t)(quarter * 32) << 16) + (uint32_t)c0, v);
            const int cl = c0 + lane;                  // the column this lane stores
            const float bl = (e.kind != EPI_STORE && cl < N) ? e.bias[cl] : 0.f;
            __syncwarp();
#pragma unroll
            for (int j = 0; j < 32; j++) T[lane * 32 + (j ^ lane)] = v[j];
            __syncwarp();
            for (int pass = 0; pass < (e.kind == EPI_BIAS_SILU ? 2 : 1); pass++) {
                float *dst = (pass == 0 && e.kind == EPI_BIAS_SILU) ? e.Z : e.C;
                for (int r = 0; r < 32; r++) {
                    const int row = rbase + r;
                    if (row >= M) break;
                    if (cl < N) {
                        const float z = T[r * 32 + (lane ^ r)] + bl;
                        dst[(size_t)row * e.ldc + cl] = (e.kind == EPI_BIAS_SILU && pass == 1) ? z * sigm(z) : z;
                    }
                }
            }
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(taddr, tcols);
}

// column sums of dZ (B x n) -> db (n): deterministic, one thread per column
__global__ void k_colsum(int B, int n, const float *__restrict__ dZ, float *__restrict__ db) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    float s = 0.f;
    for (int r = 0; r < B; r++) s += dZ[(size_t)r * n + c];
    db[c] = s;
}

// gather a minibatch and standardise: Xb = (X[idx] - mx)/sx, Tb = (Y[idx] - my)/sy
__global__ void k_gather(int B, int nin, int nout, const int *__restrict__ idx, const float *__restrict__ X,
                         const float *__restrict__ Y, const float *__restrict__ st, float *__restrict__ Xb,
                         float *__restrict__ Tb) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B) return;
    const int s = idx[i];
    const float *mx = st, *sx = st + nin, *my = st + 2 * nin, *sy = st + 2 * nin + nout;
    for (int k = 0; k < nin; k++) Xb[(size_t)i * nin + k] = (X[(size_t)s * nin + k] - mx[k]) / sx[k];
    if (Y)
        for (int k = 0; k < nout; k++) Tb[(size_t)i * nout + k] = (Y[(size_t)s * nout + k] - my[k]) / sy[k];
}

// MSE loss and its gradient on standardised targets; loss partials per block
__global__ void k_mse(int n, const float *__restrict__ Yp, const float *__restrict__ T, float scale,
                      float *__restrict__ dY, float *__restrict__ part) {
    __shared__ float red[256];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.f;
    if (i < n) {
        const float d = Yp[i] - T[i];
        dY[i] = 2.f * d * scale;
        l = d * d * scale;
    }
    red[threadIdx.x] = l;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// the epoch's loss on the device: one minibatch's block partial sums added,
// in block order, to a running FP64 total (read once per epoch instead of a
// stream synchronisation per minibatch)
__global__ void k_loss_accum(int nb, const float *__restrict__ part, double *__restrict__ acc) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double s = 0.0;
        for (int b = 0; b < nb; b++) s += part[b];
        *acc += s;
    }
}

__global__ void k_adam(int n, float *__restrict__ p, const float *__restrict__ gr, float *__restrict__ m,
                       float *__restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = gr[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// de-standardise predictions
__global__ void k_unstd(int B, int nout, const float *__restrict__ st_y, float *__restrict__ Y) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B * nout) return;
    const int k = i % nout;
    Y[i] = Y[i] * st_y[nout + k] + st_y[k];
}

}  // namespace

struct portal_mlp {
    int device = 0;
    cudaStream_t stream = nullptr;
    int n_in = 0, width = 0, depth = 0, n_out = 0, n_layers = 0;
    std::vector<int> fin, fout;
    std::vector<size_t> woff, boff;
    size_t n_params = 0;
    DevBuf<float> params, grads, adam_m, adam_v, stats;
    DevBuf<float> act;   // activations / pre-activations for one batch
    DevBuf<float> xbuf, ybuf, part;
    DevBuf<double> lossacc;  // the running loss of a training epoch
    DevBuf<int> idx;
    DevBuf<int> tc_err;  // set by a tensor-core GEMM whose completion wait timed out
    int cap_batch = 0;
    long long step = 0;
    std::string err;
};

namespace {

int mlp_fail(portal_mlp *m, int code, const std::string &msg) {
    if (m) m->err = msg;
    return code;
}

#define MCHECK(m, call)                                                                  \
    do {                                                                                 \
        cudaError_t _e = (call);                                                         \
        if (_e != cudaSuccess) return mlp_fail((m), PORTAL_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
    } while (0)

// after a stream synchronize: did a tensor-core GEMM give up waiting?
int tc_status(portal_mlp *m) {
    int e = 0;
    if (cudaMemcpy(&e, m->tc_err.p, sizeof e, cudaMemcpyDeviceToHost) != cudaSuccess)
        return mlp_fail(m, PORTAL_ERR_CUDA, "tensor-core status read");
    if (e) return mlp_fail(m, PORTAL_ERR_CUDA, "a tensor-core GEMM timed out waiting for its MMAs");
    return PORTAL_OK;
}

template <bool AK, bool BK>
void gemm(cudaStream_t s, int M, int N, int K, const float *A, int lda, const float *B, int ldb, EpiArgs e) {
    dim3 grid((N + 63) / 64, (M + 63) / 64);
    k_gemm<AK, BK><<<grid, 128, 0, s>>>(M, N, K, A, lda, B, ldb, e);
}

// A(M,K) row-major times W(N,K)^T on the tensor cores (N, K <= 256)
bool gemm_tc_fits(int N, int K) { return N >= 1 && K >= 1 && N <= 256 && K <= 256; }
void gemm_tc(cudaStream_t s, int M, int N, int K, const float *A, const float *W, EpiArgs e, int *err) {
    const int Np = (N + 15) / 16 * 16, Kp = (K + 15) / 16 * 16;
    uint32_t tcols = 32;
    while ((int)tcols < Np) tcols <<= 1;
    const size_t smem = tc_smem_bytes(Np, Kp);
    static size_t raised = 0;
    if (smem > raised) {
        cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc_smem_bytes(256, 256));
        raised = tc_smem_bytes(256, 256);
    }
    static int nsm = 0;
    if (!nsm) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (nsm < 1) nsm = 1;
    }
    const int ntiles = (M + TC_M - 1) / TC_M;
    k_gemm_tc<<<std::min(ntiles, nsm), TC_THREADS, smem, s>>>(M, N, K, Np, Kp, tcols, A, W, e, err);
}

// activation workspace layout for a batch of B rows:
//   X (B x n_in) | per layer l: Z_l, H_l (B x fout[l]) | dA, dB (B x max width)
struct Work {
    float *X, *dA, *dB;
    std::vector<float *> Z, H;
};

size_t work_floats(const portal_mlp *m, int B) {
    size_t n = (size_t)B * m->n_in;
    for (int l = 0; l < m->n_layers; l++) n += 2 * (size_t)B * m->fout[l];
    int wmax = std::max(m->width, m->n_out);
    n += 2 * (size_t)B * wmax;
    return n;
}

int ensure_batch(portal_mlp *m, int B) {
    if (B <= m->cap_batch) return PORTAL_OK;
    if (m->act.reserve(work_floats(m, B)) || m->xbuf.reserve((size_t)B * m->n_in) ||
        m->ybuf.reserve((size_t)B * m->n_out) || m->idx.reserve(B) || m->part.reserve((size_t)B * m->n_out / 256 + 2))
        return mlp_fail(m, PORTAL_ERR_NOMEM, "MLP workspace");
    m->cap_batch = B;
    return PORTAL_OK;
}

Work layout(portal_mlp *m, int B) {
    Work w;
    float *p = m->act.p;
    w.X = p;
    p += (size_t)B * m->n_in;
    for (int l = 0; l < m->n_layers; l++) {
        w.Z.push_back(p);
        p += (size_t)B * m->fout[l];
        w.H.push_back(p);
        p += (size_t)B * m->fout[l];
    }
    const int wmax = std::max(m->width, m->n_out);
    w.dA = p;
    p += (size_t)B * wmax;
    w.dB = p;
    return w;
}

// forward of standardised inputs already in w.X; the output layer's result
// goes to w.H.back()
void forward(portal_mlp *m, int B, Work &w) {
    const float *in = w.X;
    int nin = m->n_in;
    for (int l = 0; l < m->n_layers; l++) {
        const bool last = (l == m->n_layers - 1);
        EpiArgs e{last ? EPI_BIAS : EPI_BIAS_SILU, m->fout[l], w.H[l], w.Z[l], m->params.p + m->boff[l]};
        if (gemm_tc_fits(m->fout[l], nin))
            gemm_tc(m->stream, B, m->fout[l], nin, in, m->params.p + m->woff[l], e, m->tc_err.p);
        else
            gemm<true, true>(m->stream, B, m->fout[l], nin, in, nin, m->params.p + m->woff[l], nin, e);
        in = w.H[l];
        nin = m->fout[l];
    }
}

// backward from dY in w.dA (B x n_out); gradients into m->grads
void backward(portal_mlp *m, int B, Work &w) {
    float *dZ = w.dA, *dPrev = w.dB;
    for (int l = m->n_layers - 1; l >= 0; l--) {
        const int nin = m->fin[l], nout = m->fout[l];
        const float *Hin = (l == 0) ? w.X : w.H[l - 1];
        // dW = dZ^T Hin : (nout x B)(B x nin)
        EpiArgs eg{EPI_STORE, nin, m->grads.p + m->woff[l], nullptr, nullptr};
        gemm<false, false>(m->stream, nout, nin, B, dZ, nout, Hin, nin, eg);
        k_colsum<<<(nout + 127) / 128, 128, 0, m->stream>>>(B, nout, dZ, m->grads.p + m->boff[l]);
        if (l > 0) {
            // dZ_prev = (dZ W) * silu'(Z_prev)
            EpiArgs ed{EPI_DSILU, nin, dPrev, w.Z[l - 1], nullptr};
            gemm<true, false>(m->stream, B, nin, nout, dZ, nout, m->params.p + m->woff[l], nin, ed);
            std::swap(dZ, dPrev);
        }
    }
}

}  // namespace

extern "C" int portal_mlp_create(portal_mlp **out, int device, int n_in, int width, int depth, int n_out,
                                 unsigned long long seed) {
    if (!out || n_in < 1 || width < 1 || depth < 1 || n_out < 1 || width > 4096 || depth > 16)
        return PORTAL_ERR_ARG;
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess) return PORTAL_ERR_NODEVICE;
    portal_mlp *m = new portal_mlp();
    m->device = device;
    m->n_in = n_in; m->width = width; m->depth = depth; m->n_out = n_out;
    m->n_layers = depth + 1;
    size_t off = 0;
    for (int l = 0; l < m->n_layers; l++) {
        const int fi = (l == 0) ? n_in : width, fo = (l == m->n_layers - 1) ? n_out : width;
        m->fin.push_back(fi);
        m->fout.push_back(fo);
        m->woff.push_back(off);
        off += (size_t)fi * fo;
        m->boff.push_back(off);
        off += fo;
    }
    m->n_params = off;
    if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess ||
        m->params.reserve(off) || m->grads.reserve(off) || m->adam_m.reserve(off) || m->adam_v.reserve(off) ||
        m->stats.reserve(2 * (size_t)(n_in + n_out)) || m->tc_err.reserve(1)) {
        delete m;
        return PORTAL_ERR_NOMEM;
    }
    cudaMemset(m->tc_err.p, 0, sizeof(int));
    // He-uniform weights, zero biases, identity standardisation
    std::mt19937_64 rng(seed);
    std::vector<float> h(off, 0.f);
    for (int l = 0; l < m->n_layers; l++) {
        const float bound = std::sqrt(6.f / (float)m->fin[l]);
        std::uniform_real_distribution<float> u(-bound, bound);
        for (size_t i = 0; i < (size_t)m->fin[l] * m->fout[l]; i++) h[m->woff[l] + i] = u(rng);
    }
    std::vector<float> st(2 * (size_t)(n_in + n_out), 0.f);
    for (int k = 0; k < n_in; k++) st[n_in + k] = 1.f;
    for (int k = 0; k < n_out; k++) st[2 * n_in + n_out + k] = 1.f;
    cudaMemcpy(m->params.p, h.data(), off * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(m->stats.p, st.data(), st.size() * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemset(m->adam_m.p, 0, off * sizeof(float));
    cudaMemset(m->adam_v.p, 0, off * sizeof(float));
    *out = m;
    return PORTAL_OK;
}

extern "C" int portal_mlp_destroy(portal_mlp *m) {
    if (!m) return PORTAL_OK;
    cudaSetDevice(m->device);
    if (m->stream) {
        cudaStreamSynchronize(m->stream);
        cudaStreamDestroy(m->stream);
    }
    delete m;
    return PORTAL_OK;
}

extern "C" const char *portal_mlp_last_error(const portal_mlp *m) { return m ? m->err.c_str() : ""; }

extern "C" long long portal_mlp_num_params(const portal_mlp *m) { return m ? (long long)m->n_params : 0; }

extern "C" int portal_mlp_get_params(const portal_mlp *m, float *params, float *stats) {
    if (!m) return PORTAL_ERR_ARG;
    cudaSetDevice(m->device);
    if (params && cudaMemcpy(params, m->params.p, m->n_params * sizeof(float), cudaMemcpyDeviceToHost)) return PORTAL_ERR_CUDA;
    if (stats && cudaMemcpy(stats, m->stats.p, 2 * (size_t)(m->n_in + m->n_out) * sizeof(float),
                            cudaMemcpyDeviceToHost)) return PORTAL_ERR_CUDA;
    return PORTAL_OK;
}

extern "C" int portal_mlp_set_params(portal_mlp *m, const float *params, const float *stats) {
    if (!m) return PORTAL_ERR_ARG;
    cudaSetDevice(m->device);
    if (params && cudaMemcpy(m->params.p, params, m->n_params * sizeof(float), cudaMemcpyHostToDevice)) return PORTAL_ERR_CUDA;
    if (stats && cudaMemcpy(m->stats.p, stats, 2 * (size_t)(m->n_in + m->n_out) * sizeof(float),
                            cudaMemcpyHostToDevice)) return PORTAL_ERR_CUDA;
    return PORTAL_OK;
}

// one forward + backward on standardised (X, T) given on the host: loss and
// the flat gradient (same layout as the parameters)
extern "C" int portal_mlp_gradients(portal_mlp *m, const float *X, const float *T, int B, float *grads,
                                    float *loss) {
    if (!m || !X || !T || B < 1) return PORTAL_ERR_ARG;
    cudaSetDevice(m->device);
    int rc = ensure_batch(m, B);
    if (rc) return rc;
    Work w = layout(m, B);
    MCHECK(m, cudaMemcpyAsync(w.X, X, (size_t)B * m->n_in * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    MCHECK(m, cudaMemcpyAsync(m->ybuf.p, T, (size_t)B * m->n_out * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    forward(m, B, w);
    const int n = B * m->n_out, nb = (n + 255) / 256;
    k_mse<<<nb, 256, 0, m->stream>>>(n, w.H.back(), m->ybuf.p, 1.f / (float)n, w.dA, m->part.p);
    backward(m, B, w);
    MCHECK(m, cudaGetLastError());
    std::vector<float> parts(nb);
    MCHECK(m, cudaMemcpyAsync(parts.data(), m->part.p, nb * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    if (grads)
        MCHECK(m, cudaMemcpyAsync(grads, m->grads.p, m->n_params * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    MCHECK(m, cudaStreamSynchronize(m->stream));
    if (int rc2 = tc_status(m)) return rc2;
    if (loss) {
        double s = 0.0;
        for (float p : parts) s += p;
        *loss = (float)s;
    }
    return PORTAL_OK;
}

// Train on (X, Y) (host, raw units): the standardisation statistics are taken
// from this data set, then `epochs` passes of shuffled minibatches with Adam.
extern "C" int portal_mlp_train(portal_mlp *m, const float *X, const float *Y, int M, int epochs, int batch,
                                float lr, unsigned long long seed, float *loss_per_epoch) {
    if (!m || !X || !Y || M < 1 || epochs < 1 || batch < 1) return PORTAL_ERR_ARG;
    cudaSetDevice(m->device);
    const int nin = m->n_in, nout = m->n_out;
    // statistics (FP64 on the host)
    std::vector<float> st(2 * (size_t)(nin + nout));
    for (int k = 0; k < nin; k++) {
        double s = 0, s2 = 0;
        for (int i = 0; i < M; i++) { double v = X[(size_t)i * nin + k]; s += v; s2 += v * v; }
        const double mu = s / M, sd = std::sqrt(std::max(s2 / M - mu * mu, 1e-12));
        st[k] = (float)mu; st[nin + k] = (float)sd;
    }
    for (int k = 0; k < nout; k++) {
        double s = 0, s2 = 0;
        for (int i = 0; i < M; i++) { double v = Y[(size_t)i * nout + k]; s += v; s2 += v * v; }
        const double mu = s / M, sd = std::sqrt(std::max(s2 / M - mu * mu, 1e-12));
        st[2 * nin + k] = (float)mu; st[2 * nin + nout + k] = (float)sd;
    }
    MCHECK(m, cudaMemcpyAsync(m->stats.p, st.data(), st.size() * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    DevBuf<float> dX, dY;
    if (dX.reserve((size_t)M * nin) || dY.reserve((size_t)M * nout)) return mlp_fail(m, PORTAL_ERR_NOMEM, "MLP data");
    MCHECK(m, cudaMemcpyAsync(dX.p, X, (size_t)M * nin * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    MCHECK(m, cudaMemcpyAsync(dY.p, Y, (size_t)M * nout * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    const int B = std::min(batch, M);
    int rc = ensure_batch(m, B);
    if (rc) return rc;
    Work w = layout(m, B);
    std::mt19937_64 rng(seed);
    std::vector<int> perm(M);
    for (int i = 0; i < M; i++) perm[i] = i;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    DevBuf<int> pidx;
    if (pidx.reserve(M)) return mlp_fail(m, PORTAL_ERR_NOMEM, "MLP permutation");
    for (int ep = 0; ep < epochs; ep++) {
        std::shuffle(perm.begin(), perm.end(), rng);
        int nbatch = 0;
        MCHECK(m, cudaMemcpyAsync(pidx.p, perm.data(), (size_t)M * sizeof(int), cudaMemcpyHostToDevice, m->stream));
        if (loss_per_epoch) {
            if (m->lossacc.reserve(1)) return mlp_fail(m, PORTAL_ERR_NOMEM, "loss accumulator");
            MCHECK(m, cudaMemsetAsync(m->lossacc.p, 0, sizeof(double), m->stream));
        }
        MCHECK(m, cudaStreamSynchronize(m->stream));  // perm is rewritten next epoch
        for (int b0 = 0; b0 + B <= M; b0 += B) {
            k_gather<<<(B + 127) / 128, 128, 0, m->stream>>>(B, nin, nout, pidx.p + b0, dX.p, dY.p, m->stats.p, w.X,
                                                             m->ybuf.p);
            forward(m, B, w);
            const int n = B * nout, nb = (n + 255) / 256;
            k_mse<<<nb, 256, 0, m->stream>>>(n, w.H.back(), m->ybuf.p, 1.f / (float)n, w.dA, m->part.p);
            backward(m, B, w);
            m->step++;
            const float c1 = 1.f - std::pow(b1, (float)m->step), c2 = 1.f - std::pow(b2, (float)m->step);
            k_adam<<<(int)((m->n_params + 255) / 256), 256, 0, m->stream>>>((int)m->n_params, m->params.p, m->grads.p,
                                                                          m->adam_m.p, m->adam_v.p, lr, b1, b2,
                                                                          eps, c1, c2);
            if (loss_per_epoch) k_loss_accum<<<1, 32, 0, m->stream>>>(nb, m->part.p, m->lossacc.p);
            nbatch++;
        }
        MCHECK(m, cudaGetLastError());
        if (loss_per_epoch) {
            double eloss = 0.0;
            MCHECK(m, cudaMemcpyAsync(&eloss, m->lossacc.p, sizeof(double), cudaMemcpyDeviceToHost, m->stream));
            MCHECK(m, cudaStreamSynchronize(m->stream));
            loss_per_epoch[ep] = (float)(eloss / std::max(nbatch, 1));
        }
    }
    MCHECK(m, cudaStreamSynchronize(m->stream));
    return tc_status(m);
}

// Predict raw-unit outputs for raw inputs X (host or device pointers as
// flagged).  B rows.
extern "C" int portal_mlp_predict(portal_mlp *m, const float *X, int B, float *Y) {
    if (!m || !X || !Y || B < 1) return PORTAL_ERR_ARG;
    cudaSetDevice(m->device);
    const int chunk = 65536;
    int rc = ensure_batch(m, std::min(B, chunk));
    if (rc) return rc;
    DevBuf<float> dXr;
    if (dXr.reserve((size_t)std::min(B, chunk) * m->n_in)) return mlp_fail(m, PORTAL_ERR_NOMEM, "MLP predict");
    DevBuf<int> iota;
    std::vector<int> h(std::min(B, chunk));
    for (size_t i = 0; i < h.size(); i++) h[i] = (int)i;
    if (iota.reserve(h.size())) return mlp_fail(m, PORTAL_ERR_NOMEM, "MLP predict");
    MCHECK(m, cudaMemcpyAsync(iota.p, h.data(), h.size() * sizeof(int), cudaMemcpyHostToDevice, m->stream));
    for (int b0 = 0; b0 < B; b0 += chunk) {
        const int nb = std::min(chunk, B - b0);
        Work w = layout(m, nb);
        MCHECK(m, cudaMemcpyAsync(dXr.p, X + (size_t)b0 * m->n_in, (size_t)nb * m->n_in * sizeof(float),
                                  cudaMemcpyHostToDevice, m->stream));
        k_gather<<<(nb + 127) / 128, 128, 0, m->stream>>>(nb, m->n_in, m->n_out, iota.p, dXr.p, nullptr, m->stats.p,
                                                          w.X, nullptr);
        forward(m, nb, w);
        k_unstd<<<(nb * m->n_out + 255) / 256, 256, 0, m->stream>>>(nb, m->n_out, m->stats.p + 2 * m->n_in,
                                                                   w.H.back());
        MCHECK(m, cudaMemcpyAsync(Y + (size_t)b0 * m->n_out, w.H.back(), (size_t)nb * m->n_out * sizeof(float),
                                  cudaMemcpyDeviceToHost, m->stream));
        MCHECK(m, cudaStreamSynchronize(m->stream));
    }
    MCHECK(m, cudaGetLastError());
    return tc_status(m);
}
