// Polarized statistical equilibrium of every node: make_AC + get_rhovec +
// the packing of trace_node.
//
// Reference: trace_node main_sub.f90:93-137, make_AC miscellaneous.f90:288-392,
// all_transitions :394-460, setup_count_array :206-239, get_rhovec
// em_coefs.f90:115-201, setup_stateq pop_eqs.f90:361-653 and the coupling
// constants pop_eqs.f90:1-359.
//
// Every entry of the SE matrix is a linear combination of seven per-node,
// per-transition quantities
//     f0 = B21 J0,  f1 = B21 J2,  f2 = A21,  f3 = C21 (n_H2, T),
//     f4 = C21 exp(-h nu / k T),  f5 = B21 J0_eff,  f6 = A21 (1 - L*)
// with node-independent coefficients built from the Wigner coupling
// constants.  f5 and f6 serve the couplings between K = 0 components
// (populations) only.  Without a local operator J0_eff = J0 and L* = 0, so
// they equal f0 and f2 exactly and the matrix is setup_stateq's.  With one
// (the accelerated Lambda iteration) J0 = J0_eff + L* S is split into the
// field of everything but the node's own emission and the node's own
// contribution L* S, and the net radiative rates of the K = 0 equations,
// (B_lu n_l - B_ul n_u) J0 - A n_u, become (B_lu n_l - B_ul n_u) J0_eff -
// A (1 - L*) n_u (Rybicki & Hummer 1991, A&A 245, 171: the preconditioned
// rate equations), still linear in the populations.  At the fixed point
// (S unchanged) both forms are the same equations.  The host turns setup_stateq's loops into that program once per
// (molecule, kmax): a CSR list over matrix entries of (feature, coefficient)
// terms.  The kernel (one warp per node, or a team of four warps for
// systems of 48 or more unknowns) evaluates the features, assembles the
// matrix (FP64, in an L2-resident slot per team), replaces row 1 by the normalisation
// sum sqrt(2J+1) rho^0_0 = 1, factorises a row-scaled FP32 copy with partial
// pivoting and refines the solution of A rho = e_1 with FP64 residuals.
// Should the refinement stall (FP32 LU too inaccurate for the matrix's
// condition) the node is refactorised in FP64 on the device and flagged.
//
// Depolarising collisions (portal_set_depolarization; off by default, as
// main_sub.f90:96 passes D0 = 0): setup_stateq's col_dep slot
// (pop_eqs.f90:642-648) holds D^(K)(level) = n_H2 1e-6 times the
// coefficient de_polarization tabulates (depol.f90:242-317), interpolated in
// T as make_depolarization_temp does (depol.f90:319-360).  Each (level, K >=
// 2) rate is one more per-node feature after the transitions' ones; mode 2
// keeps a second copy that stands for col_dep read where the reference does
// not assign it (its last assigned value, carried through the loop), which
// the extra_info rates leave out as the reference's C_mat does.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <map>

#include "internal.cuh"

namespace portal {
void coupling_constants(int which, int j, int k, int j2, int k2, double *c0, double *c2);
double wigner3j(int tj1, int tj2, int tj3, int tm1, int tm2, int tm3);
double wigner6j(int tj1, int tj2, int tj3, int tj4, int tj5, int tj6);
}
using namespace portal;

namespace {

constexpr double A_TO_B = 6.781962e49;  // pop_eqs.f90:419
constexpr double HK = 4.79924e-11;      // pop_eqs.f90:535

__device__ __forceinline__ double warp_max(double v) {
    for (int o = 16; o >= 1; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// In-place LU with partial pivoting of the n x n column-major matrix M
// (pivot: the first row of largest modulus, as LAPACK's IDAMAX picks).
// Returns false if a pivot is zero.
template <typename T>
__device__ bool warp_lu(int n, T *M, int *piv, int lane) {
    bool ok = true;
    for (int k = 0; k < n; k++) {
        T best = (T)-1;
        int bi = n;
        for (int i = k + lane; i < n; i += 32) {
            T v = fabs(M[i + (size_t)n * k]);
            if (v > best) { best = v; bi = i; }
        }
        for (int o = 16; o >= 1; o >>= 1) {
            T ob = __shfl_xor_sync(0xffffffffu, best, o);
            int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        if (bi >= n) bi = k;  // NaN column: no row qualified; keep the diagonal
        if (lane == 0) piv[k] = bi;
        if (!(best > (T)0)) { ok = false; }
        if (bi != k)
            for (int j = lane; j < n; j += 32) {
                T t = M[k + (size_t)n * j];
                M[k + (size_t)n * j] = M[bi + (size_t)n * j];
                M[bi + (size_t)n * j] = t;
            }
        __syncwarp();
        const T d = M[k + (size_t)n * k];
        const T r = (d != (T)0) ? (T)1 / d : (T)0;
        for (int i = k + 1 + lane; i < n; i += 32) M[i + (size_t)n * k] *= r;
        __syncwarp();
        for (int i = k + 1 + lane; i < n; i += 32) {
            const T lik = M[i + (size_t)n * k];
            if (lik != (T)0)
                for (int j = k + 1; j < n; j++) M[i + (size_t)n * j] -= lik * M[k + (size_t)n * j];
        }
        __syncwarp();
    }
    return ok;
}

// Solve (LU) x = P b in place in b (length n, shared memory), one warp.
// The pivots are applied in shared memory; then lane l holds b[l + 32 m] in
// register br[m], and step k broadcasts b[k] = br[k / 32] of lane k % 32
// with a shuffle.  The steps run in blocks of 32 under an unrolled loop over
// the register index, so every register is named at compile time (a
// run-time index would put br in local memory).  The per-element operations
// are those of the plain forward and back substitution (b[i] -= M[i,k] b[k];
// b[k] /= M[k,k]).  MR rows per lane: n <= 32 MR.
template <typename T, typename V, int MR>
__device__ void warp_lu_solve(int n, const T *M, const int *piv, V *b, int lane) {
    if (lane == 0)
        for (int k = 0; k < n; k++)
            if (piv[k] != k) { V t = b[k]; b[k] = b[piv[k]]; b[piv[k]] = t; }
    __syncwarp();
    V br[MR];
#pragma unroll
    for (int m = 0; m < MR; m++) br[m] = (lane + 32 * m < n) ? b[lane + 32 * m] : (V)0;
#pragma unroll
    for (int kb = 0; kb < MR; kb++) {
        if (32 * kb >= n) break;
        const int kend = min(32, n - 32 * kb);
        for (int kk = 0; kk < kend; kk++) {
            const int k = 32 * kb + kk;
            const V bk = __shfl_sync(0xffffffffu, br[kb], kk);
#pragma unroll
            for (int m = kb; m < MR; m++) {
                const int i = lane + 32 * m;
                if (i > k && i < n) br[m] -= (V)M[i + (size_t)n * k] * bk;
            }
        }
    }
#pragma unroll
    for (int kb = MR - 1; kb >= 0; kb--) {
        if (32 * kb >= n) continue;
        const int kend = min(32, n - 32 * kb);
        for (int kk = kend - 1; kk >= 0; kk--) {
            const int k = 32 * kb + kk;
            if (lane == kk) br[kb] /= (V)M[k + (size_t)n * k];
            const V bk = __shfl_sync(0xffffffffu, br[kb], kk);
#pragma unroll
            for (int m = 0; m <= kb; m++) {
                const int i = lane + 32 * m;
                if (i < k) br[m] -= (V)M[i + (size_t)n * k] * bk;
            }
        }
    }
#pragma unroll
    for (int m = 0; m < MR; m++)
        if (lane + 32 * m < n) b[lane + 32 * m] = br[m];
    __syncwarp();
}

// The same factorisation by a team of TW warps (TW = 1: warp_lu itself).
// Warp w owns the columns j = w (mod TW): it swaps their rows, applies the
// trailing update to them and, for its own column k, runs the pivot search
// (the first row of largest modulus, as before) and forms the multipliers.
// Two barriers per step: the pivot row is published, the multipliers are.
// Every element sees the operations of warp_lu in the same order, so the
// factors are the same.  Rows are spread over the lanes (at most MR per
// lane, the multipliers held in registers: n <= 32 MR).
constexpr int SE_MAX_ROWS = 8;   // c_dim <= 256
template <typename T, int TW, int MR>
__device__ bool team_lu(int n, T *M, int *piv, int tid, double *red_v, int *red_i) {
    if constexpr (TW == 1) {
        return warp_lu<T>(n, M, piv, tid);
    } else {
        const int lane = tid & 31, w = tid >> 5;
        bool ok = true;
        for (int k = 0; k < n; k++) {
            const bool own_k = (k % TW) == w;
            if (own_k) {
                T best = (T)-1;
                int bi = n;
                for (int i = k + lane; i < n; i += 32) {
                    T v = fabs(M[i + (size_t)n * k]);
                    if (v > best) { best = v; bi = i; }
                }
                for (int o = 16; o >= 1; o >>= 1) {
                    T ob = __shfl_xor_sync(0xffffffffu, best, o);
                    int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                    if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
                }
                if (bi >= n) bi = k;  // NaN column: keep the diagonal
                if (lane == 0) {
                    red_v[0] = (double)best;
                    red_i[0] = bi;
                    piv[k] = bi;
                }
            }
            __syncthreads();   // the pivot row is published (and the last step's updates are done)
            const T best = (T)red_v[0];
            const int bi = red_i[0];
            if (!(best > (T)0)) ok = false;
            if (bi != k)
                for (int j = w + TW * lane; j < n; j += 32 * TW) {
                    T t = M[k + (size_t)n * j];
                    M[k + (size_t)n * j] = M[bi + (size_t)n * j];
                    M[bi + (size_t)n * j] = t;
                }
            if (own_k) {
                __syncwarp();
                const T d = M[k + (size_t)n * k];
                const T r = (d != (T)0) ? (T)1 / d : (T)0;
                for (int i = k + 1 + lane; i < n; i += 32) M[i + (size_t)n * k] *= r;
            }
            __syncthreads();   // the multipliers are published
            T l[MR];
#pragma unroll
            for (int m = 0; m < MR; m++) {
                const int i = k + 1 + lane + 32 * m;
                l[m] = (i < n) ? M[i + (size_t)n * k] : (T)0;
            }
            int j = k + 1 + ((w - (k + 1)) % TW + TW) % TW;   // this warp's first column after k
            for (; j < n; j += TW) {
                const T mkj = M[k + (size_t)n * j];
#pragma unroll
                for (int m = 0; m < MR; m++) {
                    const int i = k + 1 + lane + 32 * m;
                    if (i < n && l[m] != (T)0) M[i + (size_t)n * j] -= l[m] * mkj;
                }
            }
        }
        __syncthreads();
        return ok;
    }
}

// Dynamic shared memory per team (one warp, or the block's team of warps):
//   feat [n_feat] double | x, r [n] double | LU32 [n*n] float | d32 [n] float
//   | scale [n] float | piv [n] int
// The FP64 matrix A64 [n*n] (assembly, residuals, the FP64 fallback) sits in
// a per-team slot of global memory instead (L2-resident: the grid's teams x
// n^2 doubles); kept out of shared memory it lets 3x more warps share an SM,
// and the kernel is latency-bound.
constexpr int NF = 7;  // features per transition

__host__ __device__ inline size_t se_warp_bytes(int n, int n_feat) {
    size_t b = 0;
    b += sizeof(double) * ((size_t)n_feat + 2 * (size_t)n);
    b += sizeof(float) * ((size_t)n * n + 2 * (size_t)n);
    b += sizeof(int) * (size_t)n;
    return (b + 15) & ~(size_t)15;
}

// A team of TW warps per node.  TW = 1: every warp of the block is a team
// (the systems of up to ~50 unknowns); TW > 1: the block is one team, whose
// warps share the factorisation's pivot search, row operations and trailing
// updates, the FP64 residuals, the assembly and the packing (larger
// systems, whose one-warp solve is latency-bound at a few warps per SM).
// The triangular solves of the refinement run on the team's first warp.
// BATCH (TW = 1 only): the work items are (model, node) pairs of many models
// (SEBatch); each warp copies its current model's argument block into shared
// memory, and the dynamic shared memory per warp fits the largest model.
// Otherwise the nodes of the one model a0.
// MR: rows per lane of the triangular solves and the team factorisation
// (c_dim <= 32 MR).
template <int TW, bool BATCH, int MR>
__global__ void __launch_bounds__(TW == 1 ? 256 : 32 * TW, TW == 1 ? 3 : 24 / TW) k_solve_se(SEArgs a0, SEBatch bw) {
    static_assert(TW == 1 || !BATCH, "teams of several warps run the single-model kernel");
    constexpr int TS = 32 * TW;   // threads per team
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ SEArgs margs[BATCH ? 8 : 1];
    __shared__ double red_v[TW];  // cross-warp reductions of a team
    __shared__ int red_i[TW];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int tid = (TW == 1) ? lane : (int)threadIdx.x;    // thread within the team
    const int teams = (TW == 1) ? (int)(blockDim.x >> 5) : 1;
    const int team = (TW == 1) ? wib : 0;
    auto tsync = [&]() {
        if constexpr (TW == 1) __syncwarp();
        else __syncthreads();
    };
    auto team_max = [&](double v) {
        v = warp_max(v);
        if constexpr (TW > 1) {
            if (lane == 0) red_v[wib] = v;
            __syncthreads();
            v = red_v[0];
            for (int q = 1; q < TW; q++) v = fmax(v, red_v[q]);
            __syncthreads();
        }
        return v;
    };
    const long long n_items = BATCH ? bw.n_items : (long long)a0.bulk;
    const size_t wbytes = BATCH ? bw.warp_bytes : se_warp_bytes(a0.c_dim, a0.n_feat);
    unsigned char *base = smem + wbytes * team;
    double *const A64 = (BATCH ? bw.a64 : a0.a64) +
                        (size_t)((long long)blockIdx.x * teams + team) * (BATCH ? bw.a64_stride : a0.a64_stride);
    int cur_model = -1;

    for (long long item = (long long)blockIdx.x * teams + team; item < n_items; item += (long long)gridDim.x * teams) {
        int node;
        if (BATCH) {
            const int2 wi = bw.items[item];
            if (wi.x != cur_model) {
                tsync();
                const int *src = reinterpret_cast<const int *>(bw.models + wi.x);
                int *dst = reinterpret_cast<int *>(&margs[wib]);
                for (int k = tid; k < (int)(sizeof(SEArgs) / sizeof(int)); k += TS) dst[k] = src[k];
                tsync();
                cur_model = wi.x;
            }
            node = wi.y;
        } else {
            node = (int)item;
        }
        const SEArgs &a = BATCH ? margs[wib] : a0;
        const int n = a.c_dim;
        double *feat = (double *)base;
        double *x = feat + (size_t)a.n_feat;
        double *r = x + n;   // scratch (the rates)
        float *LU = (float *)(r + n);
        float *d32 = LU + (size_t)n * n;
        float *scl = d32 + n;
        int *piv = (int *)(scl + n);
        if (!(a.ab[node] > 0.0)) continue;  // main_para.f90:213 (pops stay 0)
        const double T = a.tkin[node], nH2 = a.h2[node];
        // ---- features (make_AC miscellaneous.f90:331-390) ----
        for (int t = tid; t < a.n_trans; t += TS) {
            const int rr = a.tr_rad[t], cc = a.tr_col[t];
            const double B21 = a.tr_B21[t];
            double j0 = 0.0, j2 = 0.0, je = 0.0, ls = 0.0, C21 = 0.0;
            if (rr >= 0) {
                j0 = a.J0[(size_t)node * a.L + rr];
                j2 = a.J2[(size_t)node * a.L + rr];
                je = a.JE ? a.JE[(size_t)node * a.L + rr] : j0;
                ls = a.LS ? a.LS[(size_t)node * a.L + rr] : 0.0;
            }
            if (cc >= 0) {
                // temperature interpolation (first bracket; below the table the
                // first bracket extrapolates, as the reference's loop does)
                const int nT = a.c_temp;
                double cr = 0.0;
                for (int p = 0; p < a.c_par; p++) {
                    const double *Ct = a.Cji + (size_t)nT * (cc + (size_t)a.c_num * p);
                    double v = (T <= a.col_temps[0]) ? Ct[0] : 0.0;
                    for (int i = 1; i < nT; i++)
                        if (a.col_temps[i] > T) {
                            const double ddT = (T - a.col_temps[i - 1]) / (a.col_temps[i] - a.col_temps[i - 1]);
                            v = Ct[i - 1] + ddT * (Ct[i] - Ct[i - 1]);
                            break;
                        }
                    cr += (a.c_par == 2 ? (p == 0 ? 0.25 : 0.75) : 1.0) * v;
                }
                C21 = cr * nH2 * 1e-6;
            }
            double *f = feat + NF * (size_t)t;
            f[0] = B21 * j0;
            f[1] = B21 * j2;
            f[2] = a.tr_A[t];
            f[3] = C21;
            f[4] = C21 * exp(-HK * a.tr_nu[t] / T);
            f[5] = B21 * je;
            f[6] = a.tr_A[t] * (1.0 - ls);
        }
        if (a.depol) {
            // make_depolarization_temp: every bracket with col_temps(i) > T
            // overwrites D0 (the loop has no exit), so the last bracket
            // decides below the table's top; at or above it the reference
            // leaves D0 unset (0 here)
            const int nT = a.c_temp;
            const double *ct = a.col_temps;
            for (int d = tid; d < a.n_dep; d += TS) {
                const double *tab = a.dep_tab + (size_t)nT * d;
                double v = 0.0;
                if (T <= ct[0]) v = tab[0];
                if (nT >= 2 && ct[nT - 1] > T) {
                    const double ddT = (T - ct[nT - 2]) / (ct[nT - 1] - ct[nT - 2]);
                    v = tab[nT - 2] + ddT * (tab[nT - 1] - tab[nT - 2]);
                }
                v = v * nH2 * 1e-6;
                feat[NF * (size_t)a.n_trans + d] = v;
                if (a.depol == 2) feat[NF * (size_t)a.n_trans + a.n_dep + d] = v;
            }
        }
        for (int i = tid; i < n * n; i += TS) A64[i] = 0.0;
        tsync();
        // ---- assembly (setup_stateq) ----
        // entries with terms, four records per thread in flight; each entry's
        // terms summed in program order
        for (int e0 = tid; e0 < a.n_asm; e0 += 4 * TS) {
            int4 rec[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int e = e0 + u * TS;
                rec[u] = (e < a.n_asm) ? a.asm_rec[e] : make_int4(-1, 0, 0, 0);
            }
#pragma unroll
            for (int u = 0; u < 4; u++) {
                if (rec[u].x < 0) continue;
                double v = 0.0;
                for (int q = rec[u].y; q < rec[u].z; q++) v = fma(a.term_c[q], feat[a.term_f[q]], v);
                A64[rec[u].x] = v;
            }
        }
        tsync();
        // ---- normalisation row (em_coefs.f90:158-164) ----
        for (int j = tid; j < n; j += TS) A64[(size_t)n * j] = 0.0;
        tsync();
        if (tid == 0)
            for (int i = 0; i < a.nlev; i++) A64[(size_t)n * a.norm_col[i]] = a.norm_val[i];
        tsync();
        // ---- FP32 LU of the row-scaled matrix (skipped in FP64 mode) ----
        int st = 0;
        bool ok = false, conv = false;
        if (!a.fp64_only) {
            for (int i = tid; i < n; i += TS) {
                double m = 0.0;
                for (int j = 0; j < n; j++) m = fmax(m, fabs(A64[i + (size_t)n * j]));
                const float sc = (m > 0.0) ? (float)(1.0 / m) : 1.f;
                scl[i] = sc;
                for (int j = 0; j < n; j++) LU[i + (size_t)n * j] = (float)(A64[i + (size_t)n * j] * (double)sc);
            }
            tsync();
            ok = team_lu<float, TW, MR>(n, LU, piv, tid, red_v, red_i);
        }
        if (ok) {
            for (int i = tid; i < n; i += TS) x[i] = 0.0;
            tsync();
            double xmax = 0.0, dprev = 1e300;
            for (int it = 0; it < 10; it++) {
                // r = e_1 - A x (FP64)
                for (int i = tid; i < n; i += TS) {
                    double s = (i == 0) ? 1.0 : 0.0;
                    for (int j = 0; j < n; j++) s -= A64[i + (size_t)n * j] * x[j];
                    d32[i] = (float)(s * (double)scl[i]);
                }
                tsync();
                if (TW == 1 || wib == 0) warp_lu_solve<float, float, MR>(n, LU, piv, d32, lane);
                tsync();
                double dm = 0.0;
                for (int i = tid; i < n; i += TS) {
                    x[i] += (double)d32[i];
                    dm = fmax(dm, fabs((double)d32[i]));
                }
                tsync();
                double xm = 0.0;
                for (int i = tid; i < n; i += TS) xm = fmax(xm, fabs(x[i]));
                dm = team_max(dm);
                xmax = team_max(xm);
                if (!(dm == dm) || !(xmax == xmax)) break;  // NaN
                // converged: the correction is at the level FP64 residuals can
                // resolve (~cond(SA) * eps), or it stopped shrinking there
                if (dm <= 2e-14 * xmax) { conv = true; break; }
                if (it >= 2 && dm <= 1e-12 * xmax && dm > 0.5 * dprev) { conv = true; break; }
                dprev = dm;
            }
        }
        if (!conv) {
            // FP64 LU on the device (reuses LU32 + d32 storage as FP64 space
            // is not available; re-assemble into A64 in place)
            double *M = A64;
            st |= ok ? PORTAL_NODE_REFINE : 0;
            bool ok64 = team_lu<double, TW, MR>(n, M, piv, tid, red_v, red_i);
            if (!ok64) {
                st |= PORTAL_NODE_SINGULAR;
            } else {
                for (int i = tid; i < n; i += TS) x[i] = (i == 0) ? 1.0 : 0.0;
                tsync();
                if (TW == 1 || wib == 0) warp_lu_solve<double, double, MR>(n, M, piv, x, lane);
                tsync();
                st |= PORTAL_NODE_REFINE;
            }
        }
        tsync();
        // ---- packing (main_sub.f90:112-137) ----
        for (int c2 = tid; c2 < 2 * a.nlev; c2 += TS) {
            const int p = a.pack[c2];
            double v = (p >= 0 && !(st & PORTAL_NODE_SINGULAR)) ? x[p] : 0.0;
            if (st & PORTAL_NODE_SINGULAR) v = 0.0;
            a.pops[(size_t)node + (size_t)a.N * c2] = v;
        }
        tsync();
        for (int l = tid; l < a.nlev; l += TS) {
            const double v0 = a.pops[(size_t)node + (size_t)a.N * (2 * l)];
            if (v0 != v0) {
                a.pops[(size_t)node + (size_t)a.N * (2 * l)] = 0.0;
                a.pops[(size_t)node + (size_t)a.N * (2 * l + 1)] = 0.0;
            }
        }
        if (a.rates) {
            // extra_info rates (em_coefs.f90:188-198): per component i and kind
            // k (spontaneous, radiative, collisional), sum_j |M_k(i,j)| rho_j,
            // M_k the part of setup_stateq's matrix from A, from B J, from C
            // (pop_eqs.f90:424-426, 510-512, 558-559, 599-645); the unsplit
            // field's values (f0, f2) stand for f5, f6.  Row by row in
            // ascending column order, as the reference sums.
            for (int k = 0; k < 3; k++) {
                for (int i = tid; i < n; i += TS) {
                    double acc = 0.0;
                    if (!(st & PORTAL_NODE_SINGULAR))
                        for (int q = a.row_off[i]; q < a.row_off[i + 1]; q++) {
                            const int e = a.row_ent[q];
                            double v = 0.0;
                            for (int t = a.ent_off[e]; t < a.ent_off[e + 1]; t++) {
                                const int tf = a.term_f[t];
                                if (tf >= NF * a.n_trans) {
                                    // depolarisation: C_mat where col_dep is assigned; the
                                    // carried copies (mode 2) are in Amat only
                                    if (k == 2 && tf < NF * a.n_trans + a.n_dep) v += a.term_c[t] * feat[tf];
                                    continue;
                                }
                                const int f = tf % NF, base = tf - f;
                                const int kind = (f == 2 || f == 6) ? 0 : (f == 3 || f == 4) ? 2 : 1;
                                if (kind != k) continue;
                                const int fu = (f == 5) ? 0 : (f == 6) ? 2 : f;
                                v += a.term_c[t] * feat[base + fu];
                            }
                            acc += fabs(v) * x[a.ent_pos[e] / n];
                        }
                    r[i] = acc;
                }
                tsync();
                // packing as the populations (main_sub.f90:116-135): K = 2
                // components of J = 0 levels are 0; a NaN population zeroes the
                // K = 2 rate entry (twice, as in the reference)
                for (int c2 = tid; c2 < 2 * a.nlev; c2 += TS) {
                    const int pidx = a.pack[c2];
                    double v = (pidx >= 0) ? r[pidx] : 0.0;
                    if (c2 & 1) {
                        const double p0 = x[a.pack[c2 - 1]];
                        if (p0 != p0) v = 0.0;
                    }
                    a.rates[(size_t)node + (size_t)a.N * (k + 3 * (size_t)c2)] = v;
                }
                tsync();
            }
        }
        if (a.jj20)
            for (int l = tid; l < a.L; l += TS)
                a.jj20[(size_t)node + (size_t)a.N * l] =
                    a.J2[(size_t)node * a.L + l] / a.J0[(size_t)node * a.L + l];
        if (tid == 0) {
            a.status[node] |= st;
            if (st & PORTAL_NODE_SINGULAR) atomicAdd(a.nfail, 1);
        }
        tsync();
    }
}

// ---- host: the program ---------------------------------------------------

struct Program {
    int c_dim = 0, n_trans = 0, n_dep = 0;
    std::vector<int> count_array, tr_lo, tr_up, tr_rad, tr_col;
    std::vector<double> tr_nu, tr_A, tr_B21;
    std::vector<int> ent_off, ent_pos, term_f, pack, row_off, row_ent;
    std::vector<double> term_c;
    std::vector<double> dep_tab;   // (c_temp, n_dep) depolarisation coefficients
};

// de_polarization depol.f90:242-317 (Morris 1985 Eq. B11, the D^(K) of
// L&L04 Eq. 7.102) for level i (J = i - 1, the reference's assumption) and
// rank K at collision temperature l:
//   (2J+1)^2 sum_{m=1..2J} (-1)^m (2m+1) (J J m; 0 0 0)^2
//            ({J J m; J J 0} - {J J m; J J K}) C_j0(l, m)
// with C_j0(:, m) the first partner's rate of the collisional transition
// from level 1 to level m, 0 for m = 1 (the reference never sets it) and
// for m beyond the levels (the reference reads past its array there).
double depol_coefficient(const portal_ctx *c, int i, int K, int l) {
    const int j = i - 1, nT = c->c_temp;
    const double lj2 = std::pow(2.0 * j + 1.0, 2.0);
    double s = 0.0;
    for (int m = 1; m <= 2 * j; m++) {
        double cj = 0.0;
        if (m <= c->nlev)
            for (int q = 0; q < c->c_num; q++)
                if (c->c_trans[2 * q] == 1 && c->c_trans[2 * q + 1] == m) cj = c->Cji[l + (size_t)nT * q];
        const double fac = std::pow(-1.0, m) * (2.0 * m + 1.0);
        const double w1 = wigner3j(2 * j, 2 * j, 2 * m, 0, 0, 0);
        const double w2 = wigner6j(2 * j, 2 * j, 2 * m, 2 * j, 2 * j, 0);
        const double w3 = wigner6j(2 * j, 2 * j, 2 * m, 2 * j, 2 * j, 2 * K);
        s = s + lj2 * fac * w1 * w1 * (w2 - w3) * cj;
    }
    return s;
}

void build_program(const portal_ctx *c, int kmax, Program &P) {
    const int nlev = c->nlev;
    const std::vector<int> &J = c->j_lev;
    // setup_count_array miscellaneous.f90:206-239
    P.count_array.assign(nlev, 0);
    int cnt = 0;
    for (int i = 0; i < nlev; i++) {
        P.count_array[i] = cnt;
        for (int k = 0; k <= std::min(2 * J[i], kmax); k += 2) cnt++;
    }
    P.c_dim = cnt;
    // all_transitions miscellaneous.f90:394-460
    std::vector<int> T(nlev * nlev, 0);
    auto mark = [&](int a, int b) {
        if (c->e_levs[b] > c->e_levs[a]) T[a * nlev + b] = 1;
        else T[b * nlev + a] = 1;
    };
    for (int i = 0; i < c->r_num; i++) mark(c->r_trans[2 * i] - 1, c->r_trans[2 * i + 1] - 1);
    for (int i = 0; i < c->c_num; i++) mark(c->c_trans[2 * i] - 1, c->c_trans[2 * i + 1] - 1);
    for (int i = 0; i < nlev; i++)
        for (int j = 0; j < nlev; j++)
            if (T[i * nlev + j]) { P.tr_lo.push_back(i); P.tr_up.push_back(j); }
    P.n_trans = (int)P.tr_lo.size();
    // make_AC's matching (first radiative / collisional entry with the same
    // (lower, upper) ordering)
    for (int t = 0; t < P.n_trans; t++) {
        int lo = P.tr_lo[t], up = P.tr_up[t], rr = -1, cc = -1;
        for (int j = 0; j < c->r_num; j++)
            if (c->r_trans[2 * j] - 1 == lo && c->r_trans[2 * j + 1] - 1 == up) { rr = j; break; }
        for (int j = 0; j < c->c_num; j++)
            if (c->c_trans[2 * j] - 1 == lo && c->c_trans[2 * j + 1] - 1 == up) { cc = j; break; }
        double nu = c->e_levs[up] - c->e_levs[lo];
        double A = rr >= 0 ? c->A[rr] : 0.0;
        P.tr_rad.push_back(rr);
        P.tr_col.push_back(cc);
        P.tr_nu.push_back(nu);
        P.tr_A.push_back(A);
        P.tr_B21.push_back(A_TO_B * A / std::pow(nu, 3.0));
    }
    // coupling-constant cache
    std::map<std::tuple<int, int, int, int, int>, std::pair<double, double>> cache;
    auto cc_get = [&](int which, int j, int k, int j2, int k2) {
        auto key = std::make_tuple(which, j, k, j2, k2);
        auto it = cache.find(key);
        if (it != cache.end()) return it->second;
        double a0, a2;
        coupling_constants(which, j, k, j2, k2, &a0, &a2);
        return cache[key] = std::make_pair(a0, a2);
    };
    const int n = P.c_dim;
    std::vector<int> k_of(n, 0);  // K of each component
    for (int i = 0; i < nlev; i++)
        for (int k = 0; k <= std::min(2 * J[i], kmax); k += 2) k_of[P.count_array[i] + k / 2] = k;
    std::map<int, std::vector<std::pair<int, double>>> ent;  // pos -> terms
    // depolarisation rates: one per (level, K = 2 .. min(2J, kmax))
    std::vector<int> dep_id(nlev, -1);
    P.n_dep = 0;
    if (c->depol) {
        for (int i = 0; i < nlev; i++) {
            dep_id[i] = P.n_dep;
            P.n_dep += std::min(2 * J[i], kmax) / 2;
        }
        P.dep_tab.assign((size_t)c->c_temp * P.n_dep, 0.0);
        for (int i = 0; i < nlev; i++)
            for (int K = 2; K <= std::min(2 * J[i], kmax); K += 2)
                for (int l = 0; l < c->c_temp; l++)
                    P.dep_tab[(size_t)l + (size_t)c->c_temp * (dep_id[i] + K / 2 - 1)] =
                        depol_coefficient(c, i + 1, K, l);
    }
    int cur_dep = -1;  // the (level, K) col_dep holds (the reference's loop order)
    auto add = [&](int c1, int c2, int t, int f, double coef) {
        auto &v = ent[c1 + n * c2];
        // couplings between K = 0 components take the split field (f5, f6)
        const bool k00 = (k_of[c1] == 0 && k_of[c2] == 0);
        const int ff = (k00 && f == 0) ? 5 : (k00 && f == 2) ? 6 : f;
        if (coef != 0.0) v.push_back({NF * t + ff, coef});
    };
    auto touch = [&](int c1, int c2) { ent[c1 + n * c2]; };
    for (int i1 = 0; i1 < nlev; i1++) {
        std::vector<int> up, dn;  // transition ids in the reference's order
        for (int i2 = 0; i2 < nlev; i2++)
            for (int q = 0; q < P.n_trans; q++) {
                if (P.tr_lo[q] == i1 && P.tr_up[q] == i2) up.push_back(q);
                if (P.tr_lo[q] == i2 && P.tr_up[q] == i1) dn.push_back(q);
            }
        const int j1 = J[i1];
        const double g1 = 2.0 * j1 + 1.0;
        const int k1m = std::min(2 * j1, kmax);
        for (int q : up) {  // pop_eqs.f90:467-515
            int i2 = P.tr_up[q], j2 = J[i2];
            double g2 = 2.0 * j2 + 1.0;
            int c1 = P.count_array[i1];
            for (int k1 = 0; k1 <= k1m; k1 += 2, c1++) {
                int c2 = P.count_array[i2];
                for (int k2 = 0; k2 <= std::min(2 * j2, kmax); k2 += 2, c2++) {
                    auto ts = cc_get(1, j1, k1, j2, k2);
                    auto te = cc_get(2, j1, k1, j2, k2);
                    touch(c1, c2);
                    add(c1, c2, q, 0, ts.first);
                    add(c1, c2, q, 1, ts.second);
                    add(c1, c2, q, 2, te.first);
                    if (k1 == k2 && k1 == 0) add(c1, c2, q, 3, std::sqrt(g2 / g1));
                }
            }
        }
        for (int q : dn) {  // pop_eqs.f90:518-562
            int i2 = P.tr_lo[q], j2 = J[i2];
            double g2 = 2.0 * j2 + 1.0;
            int c1 = P.count_array[i1];
            for (int k1 = 0; k1 <= k1m; k1 += 2, c1++) {
                int c2 = P.count_array[i2];
                for (int k2 = 0; k2 <= std::min(2 * j2, kmax); k2 += 2, c2++) {
                    auto ta = cc_get(0, j1, k1, j2, k2);
                    touch(c1, c2);
                    add(c1, c2, q, 0, (g1 / g2) * ta.first);
                    add(c1, c2, q, 1, (g1 / g2) * ta.second);
                    if (k1 == k2 && k1 == 0) add(c1, c2, q, 4, std::sqrt(g2 / g1) * (g1 / g2));
                }
            }
        }
        // diagonal block pop_eqs.f90:564-650
        int c1 = P.count_array[i1];
        for (int k1 = 0; k1 <= k1m; k1 += 2, c1++) {
            int c2 = P.count_array[i1];
            for (int k2 = 0; k2 <= k1m; k2 += 2, c2++) {
                touch(c1, c2);
                // col_dep (pop_eqs.f90:642-648), read after the rates below in
                // the reference; a term's position in the entry's sum does not
                // change the FP64 assembly beyond rounding
                if (c->depol) {
                    if (k1 == k2 && k1 >= 2) {
                        cur_dep = dep_id[i1] + k1 / 2 - 1;
                        ent[c1 + n * c2].push_back({NF * P.n_trans + cur_dep, -1.0});
                    } else if (c->depol == 2 && cur_dep >= 0) {
                        ent[c1 + n * c2].push_back({NF * P.n_trans + P.n_dep + cur_dep, -1.0});
                    }
                }
                for (int q : up) {
                    int j3 = J[P.tr_up[q]];
                    double g3 = 2.0 * j3 + 1.0;
                    auto ra = cc_get(3, j1, k1, j3, k2);
                    add(c1, c2, q, 0, -(g3 / g1) * ra.first);
                    add(c1, c2, q, 1, -(g3 / g1) * ra.second);
                    if (k1 == k2) add(c1, c2, q, 4, -(g3 / g1));
                }
                for (int q : dn) {
                    int j3 = J[P.tr_lo[q]];
                    auto rs = cc_get(4, j1, k1, j3, k2);
                    add(c1, c2, q, 0, -rs.first);
                    add(c1, c2, q, 1, -rs.second);
                    if (k1 == k2) {
                        add(c1, c2, q, 2, -1.0);
                        add(c1, c2, q, 3, -1.0);
                    }
                }
            }
        }
    }
    P.ent_off.assign(1, 0);
    P.ent_pos.clear(); P.term_f.clear(); P.term_c.clear();
    for (auto &kv : ent) {
        P.ent_pos.push_back(kv.first);
        for (auto &tc : kv.second) { P.term_f.push_back(tc.first); P.term_c.push_back(tc.second); }
        P.ent_off.push_back((int)P.term_f.size());
    }
    // the entries of each row in ascending column order (ent is keyed by
    // c1 + n c2: column-major)
    P.row_off.assign(n + 1, 0);
    for (int pos : P.ent_pos) P.row_off[pos % n + 1]++;
    for (int i = 0; i < n; i++) P.row_off[i + 1] += P.row_off[i];
    P.row_ent.assign(P.ent_pos.size(), 0);
    {
        std::vector<int> fill(P.row_off.begin(), P.row_off.end() - 1);
        for (int e = 0; e < (int)P.ent_pos.size(); e++) P.row_ent[fill[P.ent_pos[e] % n]++] = e;
    }
    // packing main_sub.f90:112-129: the alignment of a J != 0 level is the
    // component after its rho^0_0.  With kmax = 0 there is none, and the
    // reference then reads the next level's rho^0_0 (and, for the last
    // level, past the end of rhovec); the first is kept, the read past the
    // end gives 0 here.
    P.pack.assign(2 * nlev, -1);
    for (int i = 0; i < nlev; i++) {
        P.pack[2 * i] = P.count_array[i];
        if (J[i] != 0 && P.count_array[i] + 1 < P.c_dim) P.pack[2 * i + 1] = P.count_array[i] + 1;
    }
}

}  // namespace

namespace portal {

int prepare_se(portal_ctx *c, int kmax) {
    if (c->se_kmax == kmax) return PORTAL_OK;
    if (c->depol)
        for (int i = 0; i < c->nlev; i++)
            if (c->j_lev[i] != i)
                return set_err(c, PORTAL_ERR_ARG, "depolarising collisions need j_lev(i) = i - 1 "
                                                  "(de_polarization's assumption, depol.f90:283)");
    Program P;
    build_program(c, kmax, P);
    // pack ints: tr_rad | tr_col | ent_off | ent_pos | term_f | norm_col | pack | col? ;
    std::vector<int> I;
    std::vector<double> D;
    auto putI = [&](const std::vector<int> &v) { size_t o = I.size(); I.insert(I.end(), v.begin(), v.end()); return o; };
    auto putD = [&](const std::vector<double> &v) { size_t o = D.size(); D.insert(D.end(), v.begin(), v.end()); return o; };
    std::vector<double> norm_val(c->nlev);
    for (int i = 0; i < c->nlev; i++) norm_val[i] = std::sqrt(2.0 * c->j_lev[i] + 1.0);
    size_t o_rad = putI(P.tr_rad), o_col = putI(P.tr_col), o_eoff = putI(P.ent_off),
           o_epos = putI(P.ent_pos), o_tf = putI(P.term_f), o_nc = putI(P.count_array),
           o_pack = putI(P.pack), o_roff = putI(P.row_off), o_rent = putI(P.row_ent);
    // the assembly's records (pos, first term, end, 0) of the entries that have
    // terms, 16-byte aligned for one load each (the matrix is zeroed first)
    std::vector<int> asm_rec;
    for (size_t e = 0; e < P.ent_pos.size(); e++)
        if (P.ent_off[e + 1] > P.ent_off[e])
            asm_rec.insert(asm_rec.end(), {P.ent_pos[e], P.ent_off[e], P.ent_off[e + 1], 0});
    while (I.size() % 4) I.push_back(0);
    const size_t o_asm = putI(asm_rec);
    size_t o_nu = putD(P.tr_nu), o_A = putD(P.tr_A), o_B = putD(P.tr_B21), o_tc = putD(P.term_c),
           o_nv = putD(norm_val), o_ct = putD(c->col_temps), o_C = putD(c->Cji), o_dep = putD(P.dep_tab);
    if (c->se_ints.reserve(I.size()) || c->se_dbls.reserve(D.size()))
        return set_err(c, PORTAL_ERR_NOMEM, "SE program");
    PCHECK(c, cudaMemcpyAsync(c->se_ints.p, I.data(), I.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    PCHECK(c, cudaMemcpyAsync(c->se_dbls.p, D.data(), D.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    PCHECK(c, cudaStreamSynchronize(c->stream));
    c->se_kmax = kmax;
    c->c_dim = P.c_dim;
    c->n_trans = P.n_trans;
    c->count_array = P.count_array;
    // remember offsets in the context (packed into se_off)
    c->se_ni = (int)P.ent_pos.size();
    c->se_offs[0] = o_rad; c->se_offs[1] = o_col; c->se_offs[2] = o_eoff; c->se_offs[3] = o_epos;
    c->se_offs[4] = o_tf; c->se_offs[5] = o_nc; c->se_offs[6] = o_pack;
    c->se_offs[7] = o_nu; c->se_offs[8] = o_A; c->se_offs[9] = o_B; c->se_offs[10] = o_tc;
    c->se_offs[11] = o_nv; c->se_offs[12] = o_ct; c->se_offs[13] = o_C;
    c->se_offs[14] = o_roff; c->se_offs[15] = o_rent; c->se_offs[16] = o_dep; c->se_offs[17] = o_asm;
    c->se_nasm = (int)(asm_rec.size() / 4);
    c->n_dep = P.n_dep;
    c->n_feat = NF * P.n_trans + (c->depol == 2 ? 2 : 1) * P.n_dep;
    return PORTAL_OK;
}

// Validates kmax, builds the SE program of the molecule (once per kmax),
// sizes the outputs and fills the kernel's argument block.
int se_prepare(portal_ctx *c, int kmax, SEArgs *out, size_t *warp_bytes) {
    if (!c->have_cloud || !c->have_mol) return set_err(c, PORTAL_ERR_STATE, "no cloud or molecule");
    if (kmax < 2 || (kmax & 1))
        return set_err(c, PORTAL_ERR_ARG, "kmax must be even and >= 2 (trace_node packs rho^2_0)");
    int rc = prepare_se(c, kmax);
    if (rc) return rc;
    const int n = c->c_dim;
    const size_t wb = se_warp_bytes(n, c->n_feat);
    if (wb > 200 * 1024 || n > 32 * SE_MAX_ROWS)
        return set_err(c, PORTAL_ERR_ARG, "SE system too large for shared memory");
    if (c->pops.reserve((size_t)c->N * 2 * c->nlev) || c->jj20.reserve((size_t)c->N * c->r_num))
        return set_err(c, PORTAL_ERR_NOMEM, "SE outputs");
    SEArgs a;
    a.N = c->N; a.bulk = c->bulk; a.c_dim = n; a.n_trans = c->n_trans; a.nlev = c->nlev; a.L = c->r_num;
    a.c_temp = c->c_temp; a.c_num = c->c_num; a.c_par = c->c_par; a.nent = c->se_ni;
    a.n_feat = c->n_feat; a.n_dep = c->n_dep; a.depol = c->depol;
    a.J0 = c->J0.p; a.J2 = c->J2.p; a.h2 = c->h2.p; a.tkin = c->tkin.p; a.ab = c->active_ab();
    a.JE = c->ali_valid ? c->JE.p : nullptr;
    a.LS = c->ali_valid ? c->LS.p : nullptr;
    const int *I = c->se_ints.p;
    const double *D = c->se_dbls.p;
    a.tr_rad = I + c->se_offs[0]; a.tr_col = I + c->se_offs[1]; a.ent_off = I + c->se_offs[2];
    a.ent_pos = I + c->se_offs[3]; a.term_f = I + c->se_offs[4]; a.norm_col = I + c->se_offs[5];
    a.pack = I + c->se_offs[6];
    a.tr_nu = D + c->se_offs[7]; a.tr_A = D + c->se_offs[8]; a.tr_B21 = D + c->se_offs[9];
    a.term_c = D + c->se_offs[10]; a.norm_val = D + c->se_offs[11]; a.col_temps = D + c->se_offs[12];
    a.Cji = D + c->se_offs[13];
    a.row_off = I + c->se_offs[14]; a.row_ent = I + c->se_offs[15];
    a.asm_rec = reinterpret_cast<const int4 *>(I + c->se_offs[17]);
    a.n_asm = c->se_nasm;
    a.dep_tab = c->n_dep ? D + c->se_offs[16] : nullptr;
    a.pops = c->pops.p; a.jj20 = c->jj20.p; a.status = c->status.p;
    a.rates = nullptr;
    a.nfail = (int *)(c->counters.p + 2);
    // PORTAL_SE_FP64=1: every system factorised in FP64 (the refinement's
    // fallback path), flagged PORTAL_NODE_REFINE
    {
        const char *e = getenv("PORTAL_SE_FP64");
        a.fp64_only = (e && e[0] == '1') ? 1 : 0;
    }
    *out = a;
    if (warp_bytes) *warp_bytes = wb;
    return PORTAL_OK;
}

// The per-pass device work before the solve: zeroed outputs and failure
// count.  Stream-ordered only (capturable).
int se_pass(portal_ctx *c, cudaStream_t s) {
    PCHECK(c, cudaMemsetAsync(c->pops.p, 0, (size_t)c->N * 2 * c->nlev * sizeof(double), s));
    PCHECK(c, cudaMemsetAsync(c->jj20.p, 0, (size_t)c->N * c->r_num * sizeof(double), s));
    PCHECK(c, cudaMemsetAsync(c->counters.p + 2, 0, sizeof(unsigned long long), s));
    return PORTAL_OK;
}

size_t se_matrix_doubles(const portal_ctx *c) { return (size_t)c->c_dim * c->c_dim; }

// The batched kernel's instance for the batch's largest system (a64_stride =
// its c_dim^2): 3 rows per lane up to 96 unknowns, SE_MAX_ROWS above.
static const void *se_batch_kernel(size_t a64_stride) {
    return a64_stride <= 96 * 96 ? (const void *)k_solve_se<1, true, 3> : (const void *)k_solve_se<1, true, SE_MAX_ROWS>;
}

int se_batch_blocks_per_sm(int warps_per_block, size_t warp_bytes, size_t a64_stride, int *blocks) {
    const size_t smem = warp_bytes * warps_per_block;
    const void *k = se_batch_kernel(a64_stride);
    *blocks = 0;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return PORTAL_ERR_CUDA;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k, 32 * warps_per_block, smem) == cudaSuccess
               ? PORTAL_OK
               : PORTAL_ERR_CUDA;
}

// (the kernel's dynamic shared memory limit must have been raised by
// se_batch_blocks_per_sm for at least this many warps)
int se_batch_launch(cudaStream_t s, int grid, int warps_per_block, const SEBatch &bw) {
    const size_t smem = bw.warp_bytes * warps_per_block;
    SEArgs a0{};
    SEBatch b = bw;
    void *args[] = {&a0, &b};
    if (cudaLaunchKernel(se_batch_kernel(bw.a64_stride), dim3(grid), dim3(32 * warps_per_block), args, smem, s) !=
        cudaSuccess)
        return PORTAL_ERR_CUDA;
    return cudaGetLastError() == cudaSuccess ? PORTAL_OK : PORTAL_ERR_CUDA;
}

// Warps per node: one up to SE_TEAM_MIN_N unknowns, a team of four above
// (PORTAL_SE_TEAM=1|4 overrides).  Teams of two measured slower than either
// on 34 x 34 and 74 x 74 systems.
constexpr int SE_TEAM_MIN_N = 48;
inline int se_team_warps(int n) {
    const char *e = getenv("PORTAL_SE_TEAM");
    if (e) {
        const int v = atoi(e);
        if (v == 1 || v == 4) return v;
    }
    return n >= SE_TEAM_MIN_N ? 4 : 1;
}

// TW = 1: blocks of up to 8 independent warps; TW > 1: one team per block.
// One FP64 matrix slot per team of the grid.
template <int TW, int MR>
int launch_se(portal_ctx *c, SEArgs &a, size_t wb) {
    auto kern = k_solve_se<TW, false, MR>;
    const int teams = (TW == 1) ? (int)std::min<size_t>(8, (200 * 1024) / wb) : 1;
    const size_t smem = wb * teams;
    PCHECK(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int nb = 0;
    PCHECK(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, 32 * TW * teams, smem));
    const int grid = c->sm_count * std::max(1, nb);
    if (c->se_a64.reserve((size_t)grid * teams * a.a64_stride))
        return set_err(c, PORTAL_ERR_NOMEM, "SE matrix scratch");
    a.a64 = c->se_a64.p;
    timer_start(c, T_SE);
    kern<<<grid, 32 * TW * teams, smem, c->stream>>>(a, SEBatch{});
    timer_stop(c, T_SE);
    PCHECK(c, cudaGetLastError());
    return PORTAL_OK;
}

int run_solve_se(portal_ctx *c, int kmax, int *n_singular, bool rates) {
    SEArgs a;
    size_t wb = 0;
    int rc = se_prepare(c, kmax, &a, &wb);
    if (rc) return rc;
    if (rates) {
        const size_t nr = (size_t)c->N * 3 * 2 * c->nlev;
        if (c->rates.reserve(nr)) return set_err(c, PORTAL_ERR_NOMEM, "rates output");
        PCHECK(c, cudaMemsetAsync(c->rates.p, 0, nr * sizeof(double), c->stream));
        a.rates = c->rates.p;
    }
    if ((rc = se_pass(c, c->stream))) return rc;
    a.a64_stride = (size_t)c->c_dim * c->c_dim;
    const bool few_rows = c->c_dim <= 96;
    if (se_team_warps(c->c_dim) == 4)
        rc = few_rows ? launch_se<4, 3>(c, a, wb) : launch_se<4, SE_MAX_ROWS>(c, a, wb);
    else
        rc = few_rows ? launch_se<1, 3>(c, a, wb) : launch_se<1, SE_MAX_ROWS>(c, a, wb);
    if (rc) return rc;
    int nf = 0;
    PCHECK(c, cudaMemcpyAsync(&nf, c->counters.p + 2, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    PCHECK(c, cudaStreamSynchronize(c->stream));
    timer_collect(c, T_SE);
    if (n_singular) *n_singular = nf;
    return PORTAL_OK;
}

}  // namespace portal

extern "C" int portal_solve_se(portal_ctx *c, int kmax, const double *J0, const double *J2,
                               double *pol_pops, double *rates, double *JJ_20, int *status) {
    if (!c) return PORTAL_ERR_ARG;
    if (!c->have_cloud || !c->have_mol) return set_err(c, PORTAL_ERR_STATE, "no cloud or molecule");
    cudaSetDevice(c->device);
    const size_t LN = (size_t)c->r_num * c->N;
    if ((J0 == nullptr) != (J2 == nullptr))
        return set_err(c, PORTAL_ERR_ARG, "portal_solve_se: pass both J0 and J2 or neither");
    if (J0) {
        if (c->J0.reserve(LN) || c->J2.reserve(LN)) return set_err(c, PORTAL_ERR_NOMEM, "J buffers");
        PCHECK(c, cudaMemcpyAsync(c->J0.p, J0, LN * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        PCHECK(c, cudaMemcpyAsync(c->J2.p, J2, LN * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        PCHECK(c, cudaMemsetAsync(c->status.p, 0, (size_t)c->N * sizeof(int), c->stream));
        c->j_valid = true;
        c->ali_valid = false;  // a field from the host carries no split
    } else if (!c->j_valid) {
        return set_err(c, PORTAL_ERR_STATE, "portal_solve_se: no device-resident radiation field");
    }
    timers_reset(c);
    int nsing = 0;
    int rc = portal::run_solve_se(c, kmax, &nsing, rates != nullptr);
    if (rc) return rc;
    if (pol_pops)
        PCHECK(c, cudaMemcpyAsync(pol_pops, c->pops.p, (size_t)c->N * 2 * c->nlev * sizeof(double),
                                  cudaMemcpyDeviceToHost, c->stream));
    if (JJ_20)
        PCHECK(c, cudaMemcpyAsync(JJ_20, c->jj20.p, LN * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if (status)
        PCHECK(c, cudaMemcpyAsync(status, c->status.p, (size_t)c->N * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    if (rates)
        PCHECK(c, cudaMemcpyAsync(rates, c->rates.p, (size_t)c->N * 3 * 2 * c->nlev * sizeof(double),
                                  cudaMemcpyDeviceToHost, c->stream));
    PCHECK(c, cudaStreamSynchronize(c->stream));
    if (nsing) return set_err(c, PORTAL_ERR_SINGULAR, std::to_string(nsing) + " singular SE systems");
    return PORTAL_OK;
}

extern "C" int portal_set_depolarization(portal_ctx *c, int mode) {
    if (!c) return PORTAL_ERR_ARG;
    if (mode < 0 || mode > 2) return set_err(c, PORTAL_ERR_ARG, "portal_set_depolarization: mode 0, 1 or 2");
    if (mode != c->depol) {
        c->depol = mode;
        c->se_kmax = -1;  // rebuild the SE program
    }
    return PORTAL_OK;
}
