// Delaunay neighbour lists on the device: adj_list_no_delaunay
// (miscellaneous.f90:910-1015) with SortUnique's per-node sort and
// de-duplication (unique.f90:43-59).
//
// The reference reads the tetrahedra of grid.vtk one by one, appends to each
// vertex's list the other three vertices, then sorts every list and keeps
// each id once.  Here the same lists are built from the tetrahedra in device
// memory:
//   k_adj_count   one thread per tetrahedron: 3 entries for each of its 4
//                 vertices (atomic counts per node);
//   k_scan_*      exclusive scan of the counts (block scan, block sums, add);
//   k_adj_fill    one thread per tetrahedron: the other three vertices into
//                 each vertex's segment (slot from an atomic cursor -- the
//                 order inside a segment does not matter, it is sorted next);
//   k_adj_unique  one warp per node: each entry is kept when no earlier
//                 entry holds the same id, and goes to the position given by
//                 the number of kept ids below it -- the ascending, duplicate-
//                 free list of SortUnique, written at the start of the node's
//                 segment, with its length;
//   k_adj_scatter the lists into the reference's del_ne(node_num, max_ne)
//                 layout (column-major, 1-based ids, 0 in unused slots).
// The result does not depend on the order of the atomics, so it is the
// same on every run and equal to the host construction.
#include <algorithm>
#include <string>
#include <vector>

#include "common.cuh"

namespace {

constexpr int SCAN_BLOCK = 1024;

__global__ void k_adj_count(long long ntet, const int *__restrict__ tet, int N, int *__restrict__ cnt,
                            int *__restrict__ bad) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntet) return;
    for (int v = 0; v < 4; v++) {
        const int n = tet[4 * t + v];
        if (n < 0 || n >= N) { atomicExch(bad, 1); return; }
    }
    for (int v = 0; v < 4; v++) atomicAdd(&cnt[tet[4 * t + v]], 3);
}

// inclusive scan of one block of SCAN_BLOCK counts (Hillis-Steele in shared
// memory), written exclusive; the block total goes to sums[blockIdx]
__global__ void k_scan_block(int n, const int *__restrict__ in, long long *__restrict__ out,
                             long long *__restrict__ sums) {
    __shared__ long long s[SCAN_BLOCK];
    const int i = blockIdx.x * SCAN_BLOCK + threadIdx.x;
    const long long v = (i < n) ? in[i] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < SCAN_BLOCK; o <<= 1) {
        const long long a = (threadIdx.x >= o) ? s[threadIdx.x - o] : 0;
        __syncthreads();
        s[threadIdx.x] += a;
        __syncthreads();
    }
    if (i < n) out[i] = s[threadIdx.x] - v;
    if (threadIdx.x == SCAN_BLOCK - 1) sums[blockIdx.x] = s[threadIdx.x];
}

// exclusive scan of the block sums in one thread (a few thousand at most)
__global__ void k_scan_sums(int nb, long long *__restrict__ sums, long long *__restrict__ total) {
    long long run = 0;
    for (int b = 0; b < nb; b++) {
        const long long v = sums[b];
        sums[b] = run;
        run += v;
    }
    *total = run;
}

__global__ void k_scan_add(int n, long long *__restrict__ off, const long long *__restrict__ sums) {
    const int i = blockIdx.x * SCAN_BLOCK + threadIdx.x;
    if (i < n) off[i] += sums[blockIdx.x];
}

__global__ void k_adj_fill(long long ntet, const int *__restrict__ tet, const long long *__restrict__ off,
                           int *__restrict__ cur, int *__restrict__ raw) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntet) return;
    int q[4];
    for (int v = 0; v < 4; v++) q[v] = tet[4 * t + v];
    for (int v = 0; v < 4; v++) {
        const int n = q[v];
        const long long p = off[n] + atomicAdd(&cur[n], 3);
        int k = 0;
        for (int w = 0; w < 4; w++)
            if (w != v) raw[p + k++] = q[w];
    }
}

// One warp per node: the node's raw segment raw[off .. off+cnt) becomes its
// sorted unique list at uniq[off ..): an entry is kept when no earlier entry
// holds the same id, and goes to the position given by the number of kept
// ids below it.  The segment and its flags are staged in shared memory when
// they fit (a Delaunay node has about 80 raw entries), else read from global
// memory with the flags recomputed.
__global__ void k_adj_unique(int N, const long long *__restrict__ off, const int *__restrict__ cnt,
                             const int *__restrict__ raw, int *__restrict__ uniq, int *__restrict__ num,
                             int *__restrict__ maxne) {
    constexpr int CAP = 512;
    __shared__ int sv[8][CAP];
    __shared__ unsigned char sf[8][CAP];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int node = blockIdx.x * 8 + wib;
    if (node >= N) return;
    const long long o = off[node];
    const int n = cnt[node];
    const int *g = raw + o;
    auto first_at = [&](const int *v, int i) {
        const int x = v[i];
        for (int j = 0; j < i; j++)
            if (v[j] == x) return false;
        return true;
    };
    int kept = 0;
    if (n <= CAP) {
        int *v = sv[wib];
        unsigned char *f = sf[wib];
        for (int i = lane; i < n; i += 32) v[i] = g[i];
        __syncwarp();
        for (int i = lane; i < n; i += 32) f[i] = first_at(v, i);
        __syncwarp();
        for (int i = lane; i < n; i += 32) {
            if (!f[i]) continue;
            const int x = v[i];
            int r = 0;
            for (int j = 0; j < n; j++) r += (f[j] && v[j] < x);
            uniq[o + r] = x;
            kept++;
        }
    } else {
        for (int i = lane; i < n; i += 32) {
            if (!first_at(g, i)) continue;
            const int x = g[i];
            int r = 0;
            for (int j = 0; j < n; j++) r += (g[j] < x && first_at(g, j));
            uniq[o + r] = x;
            kept++;
        }
    }
    for (int s = 16; s >= 1; s >>= 1) kept += __shfl_xor_sync(0xffffffffu, kept, s);
    if (lane == 0) {
        num[node] = kept;
        atomicMax(maxne, kept);
    }
}

// del_ne(node_num, max_ne) column-major, 1-based, zero-padded
__global__ void k_adj_scatter(int N, int max_ne, const long long *__restrict__ off, const int *__restrict__ num,
                              const int *__restrict__ uniq, int *__restrict__ del_ne) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)N * max_ne) return;
    const int node = (int)(t % N), slot = (int)(t / N);
    del_ne[t] = (slot < num[node]) ? uniq[off[node] + slot] + 1 : 0;
}

}  // namespace

using namespace portal;

extern "C" int portal_adj_list(portal_ctx *c, int node_num, long long del_num, const int *del_tri, int max_ne_temp,
                               int *del_ne, int *del_num_ne, int *max_ne, double *ms) {
    if (!c) return PORTAL_ERR_ARG;
    if (node_num < 1 || del_num < 0 || !del_tri || max_ne_temp < 1 || !del_num_ne || !max_ne)
        return set_err(c, PORTAL_ERR_ARG, "portal_adj_list: bad arguments");
    cudaSetDevice(c->device);
    cudaStream_t s = c->stream;
    const int N = node_num;
    const long long M = del_num;
    DevBuf<int> tet, cnt, cur, raw, uniq, num, flags, dne;
    DevBuf<long long> off, sums;
    const int nb_scan = (N + SCAN_BLOCK - 1) / SCAN_BLOCK;
    if (tet.reserve((size_t)4 * (M > 0 ? M : 1)) || cnt.reserve(N) || cur.reserve(N) || num.reserve(N) ||
        flags.reserve(2) || off.reserve(N) || sums.reserve((size_t)nb_scan + 1))
        return set_err(c, PORTAL_ERR_NOMEM, "portal_adj_list: buffers");
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    PCHECK(c, cudaMemcpyAsync(tet.p, del_tri, (size_t)4 * M * sizeof(int), cudaMemcpyHostToDevice, s));
    cudaEventRecord(e0, s);
    PCHECK(c, cudaMemsetAsync(cnt.p, 0, (size_t)N * sizeof(int), s));
    PCHECK(c, cudaMemsetAsync(cur.p, 0, (size_t)N * sizeof(int), s));
    PCHECK(c, cudaMemsetAsync(flags.p, 0, 2 * sizeof(int), s));
    const int tb = 256;
    const unsigned gt = (unsigned)((M + tb - 1) / tb);
    if (M > 0) k_adj_count<<<gt, tb, 0, s>>>(M, tet.p, N, cnt.p, flags.p);
    k_scan_block<<<nb_scan, SCAN_BLOCK, 0, s>>>(N, cnt.p, off.p, sums.p);
    k_scan_sums<<<1, 1, 0, s>>>(nb_scan, sums.p, sums.p + nb_scan);
    k_scan_add<<<nb_scan, SCAN_BLOCK, 0, s>>>(N, off.p, sums.p);
    PCHECK(c, cudaGetLastError());
    int hflags[2] = {0, 0};
    long long total = 0;
    PCHECK(c, cudaMemcpyAsync(hflags, flags.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    PCHECK(c, cudaMemcpyAsync(&total, sums.p + nb_scan, sizeof(long long), cudaMemcpyDeviceToHost, s));
    PCHECK(c, cudaStreamSynchronize(s));
    if (hflags[0]) return set_err(c, PORTAL_ERR_ARG, "portal_adj_list: a tetrahedron names a node outside 0..node_num-1");
    // the reference stops when a node's unsorted list exceeds max_ne_temp
    // (miscellaneous.f90:995-1000)
    {
        std::vector<int> hc((size_t)N);
        PCHECK(c, cudaMemcpyAsync(hc.data(), cnt.p, (size_t)N * sizeof(int), cudaMemcpyDeviceToHost, s));
        PCHECK(c, cudaStreamSynchronize(s));
        for (int i = 0; i < N; i++)
            if (hc[i] > max_ne_temp)
                return set_err(c, PORTAL_ERR_ARG, "count_ne=" + std::to_string(hc[i]) + " while max_ne_temp=" +
                                                      std::to_string(max_ne_temp) + " (node " + std::to_string(i + 1) +
                                                      "): adjust max_ne_temp");
    }
    if (raw.reserve((size_t)(total > 0 ? total : 1)) || uniq.reserve((size_t)(total > 0 ? total : 1)))
        return set_err(c, PORTAL_ERR_NOMEM, "portal_adj_list: lists");
    if (M > 0) k_adj_fill<<<gt, tb, 0, s>>>(M, tet.p, off.p, cur.p, raw.p);
    k_adj_unique<<<(N + 7) / 8, 256, 0, s>>>(N, off.p, cnt.p, raw.p, uniq.p, num.p, flags.p + 1);
    PCHECK(c, cudaGetLastError());
    int mx = 0;
    PCHECK(c, cudaMemcpyAsync(&mx, flags.p + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
    PCHECK(c, cudaStreamSynchronize(s));
    *max_ne = mx;
    if (del_ne && mx > 0) {
        // the first max_ne columns of del_ne(node_num, max_ne_temp) -- column-
        // major, so they are its first node_num * max_ne entries
        if (dne.reserve((size_t)N * mx)) return set_err(c, PORTAL_ERR_NOMEM, "portal_adj_list: del_ne");
        const long long tot = (long long)N * mx;
        k_adj_scatter<<<(unsigned)((tot + tb - 1) / tb), tb, 0, s>>>(N, mx, off.p, num.p, uniq.p, dne.p);
        PCHECK(c, cudaGetLastError());
    }
    cudaEventRecord(e1, s);
    if (del_ne && mx > 0)
        PCHECK(c, cudaMemcpyAsync(del_ne, dne.p, (size_t)N * mx * sizeof(int), cudaMemcpyDeviceToHost, s));
    PCHECK(c, cudaMemcpyAsync(del_num_ne, num.p, (size_t)N * sizeof(int), cudaMemcpyDeviceToHost, s));
    PCHECK(c, cudaStreamSynchronize(s));
    if (del_ne)  // the unused columns are 0, as the reference leaves them (del_ne(i,:) = 0)
        std::fill(del_ne + (size_t)N * mx, del_ne + (size_t)N * max_ne_temp, 0);
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    if (ms) *ms = t;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return PORTAL_OK;
}
