// Shared definitions of the PORTAL GB300 library: the context, device
// buffers, error plumbing and the small numerics both kernels families use.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "portal_gb300.h"

namespace portal {

// --------------------------------------------------------------------------
// device buffer (RAII, grows on demand, never shrinks)
// --------------------------------------------------------------------------
template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    // returns cudaSuccess or the allocation error
    cudaError_t reserve(size_t count) {
        if (count <= n && p) return cudaSuccess;
        release();
        if (count == 0) count = 1;
        cudaError_t e = cudaMalloc(&p, count * sizeof(T));
        if (e != cudaSuccess) { p = nullptr; n = 0; return e; }
        n = count;
        return cudaSuccess;
    }
};

enum TimerSlot { T_LINETAB = 0, T_RF = 1, T_SE = 2, T_EMCOEF = 3, T_IMWALK = 4, T_IMRT = 5, T_NSLOT = 6 };

}  // namespace portal

struct portal_ctx {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;       // the stream all work runs on
    cudaStream_t own_stream = nullptr;   // created by portal_create
    std::string err;

    // ---- molecule (host copies, FP64) ----
    bool have_mol = false;
    int nlev = 0, r_num = 0, c_num = 0, c_temp = 0, c_par = 0;
    std::vector<int> j_lev, r_trans, c_trans;
    std::vector<double> e_levs, A, nu, Bij, kd_v, col_temps, Cji;

    // ---- cloud ----
    bool have_cloud = false;
    int N = 0, bulk = 0, nnz = 0, maxdeg = 0;
    double tx = 0.0;
    portal::DevBuf<double> pos64;     // (3,N) FP64 positions
    portal::DevBuf<double> bvec64;    // (3,N)
    portal::DevBuf<double> vel64;     // (3,N) FP64 velocities (image rotation)
    portal::DevBuf<float4> cellv;     // (vx,vy,vz,b) per node
    portal::DevBuf<int> nb_off;       // N+1
    portal::DevBuf<int> nb_idx;       // nnz, 0-based
    portal::DevBuf<float4> edge;      // nnz: (ex,ey,ez,|e|^2/2) from FP64
    portal::DevBuf<double> levp;      // (nlev,N)
    portal::DevBuf<double> nmol;      // per node total molecule density (sum lev_p)
    portal::DevBuf<double> b64, tkin, tdust, dustp, h2, ab;
    bool has_dust = false;

    // ---- star mode (star_mod = 1, main_para.f90:75, :122, :216-246) ----
    int star_mode = 0;
    double T_star = 0.0, R_star_m = 0.0;  // R_star as the input file gives it, metres
    double X_star[3] = {0.0, 0.0, 0.0};   // used unscaled, as the reference does
    portal::DevBuf<double> ab_star;       // ab, 0 for the nodes inside the star (skipped)
    portal::DevBuf<float> bbstar;         // (r_num) black_body(T_star) per line
    portal::DevBuf<unsigned char> star_model;  // the RFArgs of a star-mode pass (batched kernel)
    portal::DevBuf<int2> star_items;      // its work items (0, node)
    int star_items_n = 0;
    // the abundances the node loop runs on: nodes with ab <= 0 (and, in star
    // mode, inside the star) are skipped by the radiation field and the SE
    const double *active_ab() const { return star_mode ? ab_star.p : ab.p; }
    double R_star() const { return R_star_m / tx; }  // main_para.f90:122

    // ---- derived / results ----
    portal::DevBuf<float4> ltab;      // (r_num,N) line table
    portal::DevBuf<unsigned char> linebuf;  // per-line constants of the molecule (rf.cu)
    portal::DevBuf<float> bbcmb;      // (r_num) black_body(2.73 K) per line
    portal::DevBuf<double> J0, J2;    // (r_num,N)
    portal::DevBuf<double> JE, LS;    // (r_num,N) J0 without the node's own emission, local operator L*
    bool ali_valid = false;           // JE / LS belong to the current J0 (the SE splits the field)
    portal::DevBuf<int> status;       // N
    portal::DevBuf<int> nodeseg;      // N: ray segments of each node in the last radiation field
    portal::DevBuf<float> kmom;       // (6, N): second moment of line 1's field per node
    portal::DevBuf<int2> walk;        // per-warp walk scratch
    portal::DevBuf<unsigned long long> counters;  // [0] work, [1] segments, [2..] misc
    portal::DevBuf<double> dirtab;    // direction table
    portal::DevBuf<float> chtab;      // channel tables
    bool j_valid = false;
    double rf_dxp = 0.0;              // r_max * trace step of the last radiation-field set-up

    // SE program (device) -- built per (molecule, kmax, depolarisation mode)
    int se_kmax = -1, c_dim = 0, n_trans = 0;
    int depol = 0;                    // depolarising collisions (portal_set_depolarization)
    int n_dep = 0, n_feat = 0;
    portal::DevBuf<int> se_ints;
    portal::DevBuf<double> se_dbls;
    std::vector<int> count_array;
    portal::DevBuf<double> se_a64;    // FP64 SE matrices, one per resident warp
    portal::DevBuf<double> pops;      // (N, 2*nlev) column-major result
    portal::DevBuf<double> rates;     // (N,3,2*nlev)
    portal::DevBuf<double> jj20;      // (N, r_num)
    int se_ni = 0;
    int se_nasm = 0;                  // entries with terms (the assembly's list)
    size_t se_offs[20] = {};

    // ---- timing ----
    cudaEvent_t ev[2 * portal::T_NSLOT] = {};
    double t_ms[portal::T_NSLOT] = {};
    int t_launch[portal::T_NSLOT] = {};
    bool ev_ready = false;
};

namespace portal {

inline int set_err(portal_ctx *c, int code, const std::string &msg) {
    if (c) c->err = msg;
    return code;
}

inline int cuda_fail(portal_ctx *c, cudaError_t e, const char *what) {
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    if (c) c->err = m;
    return (e == cudaErrorMemoryAllocation) ? PORTAL_ERR_NOMEM : PORTAL_ERR_CUDA;
}

#define PCHECK(ctx, call)                                                  \
    do {                                                                   \
        cudaError_t _e = (call);                                           \
        if (_e != cudaSuccess) return portal::cuda_fail((ctx), _e, #call); \
    } while (0)

// timers: record start/stop around one kernel launch on the ctx stream
inline void timer_start(portal_ctx *c, int slot) { cudaEventRecord(c->ev[2 * slot], c->stream); }
inline void timer_stop(portal_ctx *c, int slot) { cudaEventRecord(c->ev[2 * slot + 1], c->stream); }
// after a stream synchronize: fold the slot's event pair into the totals
inline void timer_collect(portal_ctx *c, int slot) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c->ev[2 * slot], c->ev[2 * slot + 1]) == cudaSuccess) {
        c->t_ms[slot] += ms;
        c->t_launch[slot] += 1;
    }
}
inline void timers_reset(portal_ctx *c) {
    for (int i = 0; i < T_NSLOT; i++) { c->t_ms[i] = 0.0; c->t_launch[i] = 0; }
}

// FP64 without FMA contraction, in the operation order of the oracle (the
// reference's expressions evaluated left to right)
__device__ __forceinline__ double dsum3sq(double x, double y, double z) {
    return __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
}
__device__ __forceinline__ double ddot3(double ax, double ay, double az, double bx, double by, double bz) {
    return __dadd_rn(__dadd_rn(__dmul_rn(ax, bx), __dmul_rn(ay, by)), __dmul_rn(az, bz));
}

// Distance from node position p to the unit sphere along d: pos_quadratic
// (miscellaneous.f90:1078-1098) with the arguments check_neigh_fast forms
// for trace_out's first step (:1033), norm2(d)**2, 2 p.d, norm2(p)**2 - 1.
// Evaluated without contraction so that the sign of |p|^2 - 1 -- which, for
// the outermost node of a cloud (|p| = 1 to the last bit after the
// normalisation by r_max), decides whether its inward rays leave the sphere
// at once -- is the same as in the FP64 restatement.  0 where the
// discriminant is not positive (the reference leaves delta_x unset there).
__device__ __forceinline__ double sphere_exit(double px, double py, double pz, double dx, double dy,
                                              double dz) {
    const double nd = __dsqrt_rn(dsum3sq(dx, dy, dz));
    const double a = __dmul_rn(nd, nd);
    const double b = __dmul_rn(2.0, ddot3(px, py, pz, dx, dy, dz));
    const double np = __dsqrt_rn(dsum3sq(px, py, pz));
    const double c = __dsub_rn(__dmul_rn(np, np), 1.0);
    const double dis = __dsub_rn(__dmul_rn(b, b), __dmul_rn(__dmul_rn(4.0, a), c));
    if (!(dis > 0.0)) return 0.0;
    const double sq = __dsqrt_rn(dis);
    const double x1 = __ddiv_rn(__dadd_rn(-b, sq), __dmul_rn(2.0, a));
    const double x2 = __ddiv_rn(__dsub_rn(-b, sq), __dmul_rn(2.0, a));
    return (x2 > 0.0) ? x2 : x1;
}

// 1 - e^-tau of a cell's optical depth tau = x ln 2, given e = 2^-x from
// ex2: the weight of the transfer update I' = I + (1 - e^-tau) (S - I).
//   - 1 - e alone loses the small-tau regime (e rounds to 1 below tau ~ 6e-8
//     and keeps only ~1.5e-7/tau of relative accuracy above), where an
//     optically thin line's emission S tau can be all there is (a high line
//     whose source function exceeds the background by 1e14); below
//     |tau| = 0.0435 the cubic Taylor form tau (1 - tau/2 + tau^2/6) is used
//     (relative error <= 3.5e-6 on both sides of the switch).
//   - The reference forms 1 - exp(-tau) in FP64, which rounds it to a
//     multiple of 2^-53 (exp(-tau) lies on the 2^-53 grid below 1) and drops
//     tau below 2^-54 altogether; its results for such lines depend on that
//     rounding.  The Taylor value is rounded the same way: adding and
//     removing 1.5 * 2^-30 rounds anything below 2^-31 to a multiple of 2^-53
//     (the FP32 grid spacing at that magnitude) and changes larger values by
//     at most an FP32 rounding.
constexpr float OM_TAYLOR_X = 0.0628f;                 // |x| below which the Taylor form is used
constexpr float OM_MAGIC = 1.3969838619232178e-09f;    // 1.5 * 2^-30
__device__ __forceinline__ float om_taylor(float x) {
    constexpr float C1 = 0.693147181f;   // ln 2
    constexpr float C2 = -0.240226507f;  // -(ln 2)^2 / 2
    constexpr float C3 = 0.0555041087f;  // (ln 2)^3 / 6
    const float h = fmaf(x, fmaf(x, C3, C2), C1);
    return __fsub_rn(fmaf(x, h, OM_MAGIC), OM_MAGIC);
}
__device__ __forceinline__ float one_minus_exp(float x, float e) {
    return (fabsf(x) < OM_TAYLOR_X) ? om_taylor(x) : 1.f - e;
}
// The same for two optical depths at once on the packed FP32x2 pipe (the
// same operations and roundings per element as om_taylor / one_minus_exp).
__device__ __forceinline__ float2 om_taylor2(float2 x) {
    const float2 h = __ffma2_rn(x, __ffma2_rn(x, make_float2(0.0555041087f, 0.0555041087f),
                                              make_float2(-0.240226507f, -0.240226507f)),
                                make_float2(0.693147181f, 0.693147181f));
    return __fadd2_rn(__ffma2_rn(x, h, make_float2(OM_MAGIC, OM_MAGIC)), make_float2(-OM_MAGIC, -OM_MAGIC));
}
__device__ __forceinline__ float2 one_minus_exp2(float2 x, float e0, float e1) {
    const float2 t = om_taylor2(x);
    const float2 b = __ffma2_rn(make_float2(e0, e1), make_float2(-1.f, -1.f), make_float2(1.f, 1.f));
    return make_float2((fabsf(x.x) < OM_TAYLOR_X) ? t.x : b.x, (fabsf(x.y) < OM_TAYLOR_X) ? t.y : b.y);
}

// host: Gauss-Legendre rule on (-1,1), ascending knots (Newton iteration on
// the three-term recurrence, long double)
void gauss_legendre(int n, double *x, double *w);
// host: the direction set of legendre_all (miscellaneous.f90:1100-1137);
// returns rows (mu, phi, w) packed as 3 doubles per direction
int legendre_all(int nth, int nph, std::vector<double> &xth);

}  // namespace portal
