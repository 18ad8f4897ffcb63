// Kernel argument blocks and the internal entry points shared by the
// single-model calls (rf.cu, se.cu) and the batched launch (batch.cu).
#pragma once

#include "common.cuh"

namespace portal {

// Everything the radiation-field kernel reads or writes for one model.
struct RFArgs {
    int N, bulk, L, nvel, nch, ndir, n_depth;
    float dx32;
    const double *__restrict__ pos;
    const double *__restrict__ bvec;
    const double *__restrict__ ab;
    const float4 *__restrict__ cellv;
    const int *__restrict__ off;
    const int *__restrict__ idx;
    const float4 *__restrict__ edge;
    const float4 *__restrict__ ltab;
    const double *__restrict__ dirs;  // (ndir, 6): mu, sin th, cos ph, sin ph, w, w*c_in/sqrt2
    const float *__restrict__ chq;    // (nch) 2 nv / nvel
    const float *__restrict__ chw;    // (nch) exp(-q0^2) * 2/(sqrt(pi) nvel)
    const float *__restrict__ bb;     // (L) black_body(2.73 K) per line: the incoming intensity
    double gx, gy, gz;
    // star mode: each node's ray set from star_all (nth x nph bands around the
    // star direction), star rays end on the star and start from B(T_star)
    int star, nth, nph;
    double xs, ys, zs, Rs;
    const float *__restrict__ bbs;    // (L) black_body(T_star) per line
    double *J0, *J2;
    double *JE, *LS;                  // split field (accelerated Lambda iteration) or null
    int *status;
    int *segs;                        // (N) ray segments of each node (sum of node_count) or null
    float *kmom;                      // (6, N) second moment sum w I n n of line 1 (xx yy zz xy xz yz) or null
    int2 *walk;
    unsigned long long *counters;
};

// Everything the SE kernel reads or writes for one model.
struct SEArgs {
    int N, bulk, c_dim, n_trans, nlev, L, c_temp, c_num, c_par, nent;
    int n_feat;                         // features per node: NF per transition + depolarisation
    int n_dep, depol;                   // (level, K >= 2) depolarisation rates, mode (0 off)
    const double *__restrict__ dep_tab; // (c_temp, n_dep) D^(K) coefficients [cm^3/s] or null
    const double *__restrict__ J0;
    const double *__restrict__ J2;
    const double *__restrict__ JE;      // J0_eff (r_num, N) or null
    const double *__restrict__ LS;      // L* (r_num, N) or null
    const double *__restrict__ h2;
    const double *__restrict__ tkin;
    const double *__restrict__ ab;
    // per transition
    const int *__restrict__ tr_rad;
    const int *__restrict__ tr_col;
    const double *__restrict__ tr_nu;
    const double *__restrict__ tr_A;
    const double *__restrict__ tr_B21;
    const double *__restrict__ col_temps;
    const double *__restrict__ Cji;
    // program over the matrix entries
    const int *__restrict__ ent_off;
    const int *__restrict__ ent_pos;
    const int *__restrict__ term_f;
    const double *__restrict__ term_c;
    const int *__restrict__ norm_col;   // (nlev) count_array
    const double *__restrict__ norm_val;
    const int *__restrict__ pack;       // (2 nlev) rho index or -1
    const int *__restrict__ row_off;    // (c_dim + 1) entries of each matrix row,
    const int *__restrict__ row_ent;    // ascending column (the rates' summation order)
    const int4 *__restrict__ asm_rec;   // the entries with terms: (pos, first term, end, 0)
    int n_asm;
    double *pops;                       // (N, 2 nlev) column-major
    double *jj20;                       // (N, L) or null
    double *rates;                      // (N, 3, 2 nlev) column-major or null
    int *status;
    int *nfail;
    double *a64;                        // FP64 matrices, one slot of a64_stride doubles per team
    size_t a64_stride;
    int fp64_only;                      // factorise every system in FP64 (no FP32 LU)
};

// A batched launch: work items (model, node) over many models, the models'
// argument blocks in device memory.
struct RFBatch {
    const RFArgs *models;
    const int2 *items;
    long long n_items;
    unsigned long long *queue;   // [0] next item, [1] segments walked
    int2 *walk;                  // per warp: 32 rays x n_depth
    int n_depth;
    int rem_lines;               // lines of the remainder channel's shared table (largest model)
};
struct SEBatch {
    const SEArgs *models;
    const int2 *items;
    long long n_items;
    size_t warp_bytes;           // dynamic shared memory per warp (largest model)
    double *a64;                 // FP64 matrices, one slot of a64_stride doubles per warp
    size_t a64_stride;           // largest model's c_dim^2
};

// rf.cu
int rf_prepare(portal_ctx *c, int nth, int nph, int nvel, const double *gvec, double dx, int n_depth,
               bool split, RFArgs *a);
int rf_pass(portal_ctx *c, const RFArgs &a, cudaStream_t s);
int rf_batch_blocks_per_sm(int nch, bool dust, int nlg, int max_lines, int *blocks);
const void *rf_batch_kernel_ptr(int nch, bool dust, int nlg, int max_lines);  // identity of the variant
int rf_batch_launch(cudaStream_t s, int grid, int nch, bool dust, int nlg, int max_lines, const RFBatch &bw);
// se.cu
int se_prepare(portal_ctx *c, int kmax, SEArgs *a, size_t *warp_bytes);
int se_pass(portal_ctx *c, cudaStream_t s);
int se_batch_launch(cudaStream_t s, int grid, int warps_per_block, const SEBatch &bw);
int se_batch_blocks_per_sm(int warps_per_block, size_t warp_bytes, size_t a64_stride, int *blocks);
size_t se_matrix_doubles(const portal_ctx *c);  // c_dim^2 of the prepared SE program

}  // namespace portal
