// Plain Lambda iteration of the node loop.
//
// PORTAL itself makes one pass (main_para.f90:210-257): the radiation field of
// LIME's populations, then one SE solve per node.  Iterating that pass is the
// natural extension: iteration k takes level populations n^k, computes
// J(n^k) (inverse_rt), solves the SE (get_rhovec) and sets
//     n_J^{k+1} = n_mol sqrt(2J+1) rho^0_0(J)
// (N_J ~ sqrt(2J+1) rho^0_0, em_coefs.f90:91-94, with sum_J sqrt(2J+1)
// rho^0_0 = 1 from the normalisation row em_coefs.f90:158-164, so the total
// n_mol is kept).  Iteration 1 from the cloud's populations is exactly the
// reference's single pass.  The residual is the largest relative change of
// rho^0_0 over nodes and levels (levels below 1e-12 of the node's largest
// population are ignored); the loop stops when it falls below tol.
//
// Optional Ng acceleration (ng_period > 0): after every ng_period plain
// passes the state jumps to the order-2 Ng extrapolation of the last four
// iterates (Ng 1974, J. Chem. Phys. 61, 2680; the form of Olson, Auer &
// Buchler 1986, JQSRT 35, 431).  Convergence is still decided by the plain
// pass alone (the change one radiation field + SE pass makes), so the state
// it stops at is a fixed point of the plain iteration to tol.
//
// Optional local operator (local_operator != 0): the passes solve the
// preconditioned SE (the split J0 = J_eff + L* S of the radiation-field
// kernel; Rybicki & Hummer 1991), the accelerated Lambda iteration with the
// diagonal of the Lambda operator.  Its fixed point is the plain one; when
// an accelerated pass changes the populations by less than tol, a plain pass
// follows and decides: below tol it ends the iteration, otherwise the
// accelerated passes resume.
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace portal {
int run_radiation_field(portal_ctx *c, int nth, int nph, int nvel, const double *gvec, double dx,
                        int n_depth, long long *n_segments, int *n_failed, bool split);
int run_solve_se(portal_ctx *c, int kmax, int *n_singular, bool rates);
}  // namespace portal
using namespace portal;

namespace {

// rho^0_0 of the current populations, n_J / (n_mol sqrt(2J+1))
__global__ void k_pops_to_rho(int N, int nlev, const double *__restrict__ levp,
                              const double *__restrict__ nmol, const int *__restrict__ jl,
                              double *__restrict__ rho) {
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    const double m = nmol[n];
    for (int l = 0; l < nlev; l++)
        rho[(size_t)nlev * n + l] = (m > 0.0) ? levp[(size_t)nlev * n + l] / (m * sqrt(2.0 * jl[l] + 1.0)) : 0.0;
}

// warm start given as pol_pops (N, 2 nlev): populations from its rho^0_0
__global__ void k_rho_to_pops(int N, int bulk, int nlev, const double *__restrict__ pp,
                              const double *__restrict__ nmol, const double *__restrict__ ab,
                              const int *__restrict__ jl, double *__restrict__ levp) {
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= bulk || !(ab[n] > 0.0)) return;
    for (int l = 0; l < nlev; l++)
        levp[(size_t)nlev * n + l] = nmol[n] * sqrt(2.0 * jl[l] + 1.0) * pp[(size_t)n + (size_t)N * (2 * l)];
}

// populations from the SE solution, and the residual (max relative change)
__global__ void k_update(int N, int bulk, int nlev, const double *__restrict__ pops,
                         const double *__restrict__ nmol, const double *__restrict__ ab,
                         const int *__restrict__ jl, double *__restrict__ levp,
                         double *__restrict__ rho_prev, unsigned long long *__restrict__ resid) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    double r = 0.0;
    if (n < bulk && ab[n] > 0.0) {
        double big = 0.0;
        for (int l = 0; l < nlev; l++) big = fmax(big, fabs(pops[(size_t)n + (size_t)N * (2 * l)]));
        const double floor_ = 1e-12 * big;
        for (int l = 0; l < nlev; l++) {
            const double rho = pops[(size_t)n + (size_t)N * (2 * l)];
            const double old = rho_prev[(size_t)nlev * n + l];
            const double d = fabs(rho - old) / fmax(fabs(rho), floor_ > 0.0 ? floor_ : 1e-300);
            if (fabs(rho) >= floor_) r = fmax(r, d);
            rho_prev[(size_t)nlev * n + l] = rho;
            levp[(size_t)nlev * n + l] = nmol[n] * sqrt(2.0 * jl[l] + 1.0) * rho;
        }
        if (!(r == r)) r = 1e300;  // NaN populations never count as converged
    }
    for (int o = 16; o >= 1; o >>= 1) r = fmax(r, __shfl_xor_sync(0xffffffffu, r, o));
    if ((threadIdx.x & 31) == 0 && r > 0.0) atomicMax(resid, (unsigned long long)__double_as_longlong(r));
}

// Ng (1974) extrapolation of order 2 over the last four iterates x3 (newest),
// x2, x1, x0 of rho^0_0: with d0 = x3-x2, d1 = x2-x1, d2 = x1-x0 and weights
// 1/x3^2, the normal equations of min |d0 - a (d0-d1) - b (d0-d2)|^2.
// Partial sums per block (deterministic), combined by k_ng_final.
__global__ void k_ng_sums(int N, int bulk, int nlev, const double *__restrict__ ab,
                          const double *__restrict__ x0, const double *__restrict__ x1,
                          const double *__restrict__ x2, const double *__restrict__ x3,
                          double *__restrict__ part) {
    __shared__ double red[5][256];
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    double s[5] = {0, 0, 0, 0, 0};
    if (n < bulk && ab[n] > 0.0) {
        double big = 0.0;
        for (int l = 0; l < nlev; l++) big = fmax(big, fabs(x3[(size_t)nlev * n + l]));
        for (int l = 0; l < nlev; l++) {
            const size_t i = (size_t)nlev * n + l;
            const double v3 = x3[i];
            if (!(fabs(v3) >= 1e-12 * big) || v3 == 0.0) continue;
            const double w = 1.0 / (v3 * v3);
            const double d0 = v3 - x2[i], d1 = x2[i] - x1[i], d2 = x1[i] - x0[i];
            const double p = d0 - d1, q = d0 - d2;
            s[0] += w * p * p;
            s[1] += w * p * q;
            s[2] += w * q * q;
            s[3] += w * d0 * p;
            s[4] += w * d0 * q;
        }
    }
    for (int k = 0; k < 5; k++) red[k][threadIdx.x] = s[k];
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h)
            for (int k = 0; k < 5; k++) red[k][threadIdx.x] += red[k][threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < 5; k++) part[5 * (size_t)blockIdx.x + k] = red[k][0];
}

__global__ void k_ng_final(int nblocks, const double *__restrict__ part, double *__restrict__ out) {
    if (threadIdx.x >= 5) return;
    double s = 0.0;
    for (int b = 0; b < nblocks; b++) s += part[5 * (size_t)b + threadIdx.x];
    out[threadIdx.x] = s;
}

// x = (1-a-b) x3 + a x2 + b x1 per bulk node; entries that would turn
// non-positive keep x3's value, then the node is renormalised
// (sum_J sqrt(2J+1) rho^0_0 = 1) and its populations set from it
__global__ void k_ng_apply(int N, int bulk, int nlev, double a, double b, const double *__restrict__ ab,
                           const double *__restrict__ nmol, const int *__restrict__ jl,
                           const double *__restrict__ x1, const double *__restrict__ x2,
                           const double *__restrict__ x3, double *__restrict__ rho, double *__restrict__ levp) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= bulk || !(ab[n] > 0.0)) return;
    double norm = 0.0;
    for (int l = 0; l < nlev; l++) {
        const size_t i = (size_t)nlev * n + l;
        double v = (1.0 - a - b) * x3[i] + a * x2[i] + b * x1[i];
        if (!(v > 0.0)) v = x3[i];
        rho[i] = v;
        norm += sqrt(2.0 * jl[l] + 1.0) * v;
    }
    const double sc = (norm > 0.0) ? 1.0 / norm : 1.0;
    for (int l = 0; l < nlev; l++) {
        const size_t i = (size_t)nlev * n + l;
        rho[i] *= sc;
        levp[i] = nmol[n] * sqrt(2.0 * jl[l] + 1.0) * rho[i];
    }
}

}  // namespace

extern "C" int portal_lambda_iterate(portal_ctx *c, int nth, int nph, int nvel, const double *gvec,
                                     double dx, int n_depth, int kmax, double tol, int max_iter,
                                     int ng_period, int local_operator, const double *start_pops, double *pol_pops, double *lev_p_out,
                                     int *iterations, double *residuals, long long *n_segments) {
    if (!c) return PORTAL_ERR_ARG;
    if (!c->have_cloud || !c->have_mol) return set_err(c, PORTAL_ERR_STATE, "no cloud or molecule");
    if (max_iter < 1 || !(tol > 0.0) || ng_period < 0 || (ng_period > 0 && ng_period < 3))
        return set_err(c, PORTAL_ERR_ARG, "portal_lambda_iterate: max_iter >= 1, tol > 0, ng_period 0 or >= 3");
    cudaSetDevice(c->device);
    timers_reset(c);
    const int N = c->N, nlev = c->nlev;
    DevBuf<int> jl;
    DevBuf<double> rho_prev;
    if (jl.reserve(nlev) || rho_prev.reserve((size_t)nlev * N) || c->pops.reserve((size_t)N * 2 * nlev))
        return set_err(c, PORTAL_ERR_NOMEM, "lambda buffers");
    PCHECK(c, cudaMemcpyAsync(jl.p, c->j_lev.data(), nlev * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    const int tb = 256, nb = (N + tb - 1) / tb;
    if (start_pops) {
        DevBuf<double> sp;
        if (sp.reserve((size_t)N * 2 * nlev)) return set_err(c, PORTAL_ERR_NOMEM, "start pops");
        PCHECK(c, cudaMemcpyAsync(sp.p, start_pops, (size_t)N * 2 * nlev * sizeof(double),
                                  cudaMemcpyHostToDevice, c->stream));
        k_rho_to_pops<<<nb, tb, 0, c->stream>>>(N, c->bulk, nlev, sp.p, c->nmol.p, c->active_ab(), jl.p, c->levp.p);
        PCHECK(c, cudaGetLastError());
        PCHECK(c, cudaStreamSynchronize(c->stream));
    }
    k_pops_to_rho<<<nb, tb, 0, c->stream>>>(N, nlev, c->levp.p, c->nmol.p, jl.p, rho_prev.p);
    PCHECK(c, cudaGetLastError());
    // Ng acceleration: the last four iterates (ring), block partial sums
    DevBuf<double> ring, part;
    const size_t nv = (size_t)nlev * N;
    if (ng_period > 0 && (ring.reserve(4 * nv) || part.reserve(5 * (size_t)nb + 5)))
        return set_err(c, PORTAL_ERR_NOMEM, "Ng buffers");
    int n_hist = 0, since_ng = 0;
    auto push_hist = [&]() -> int {
        PCHECK(c, cudaMemcpyAsync(ring.p + (size_t)(n_hist % 4) * nv, rho_prev.p, nv * sizeof(double),
                                  cudaMemcpyDeviceToDevice, c->stream));
        n_hist++;
        return PORTAL_OK;
    };
    if (ng_period > 0 && push_hist()) return PORTAL_ERR_CUDA;
    long long nseg_tot = 0;
    int it = 0, rc = PORTAL_OK;
    double r = 1e300;
    bool verify = false;  // this pass is the plain pass that decides convergence
    while (it < max_iter) {
        long long nseg = 0;
        int nfail = 0;
        const bool split = local_operator && !verify;
        if ((rc = run_radiation_field(c, nth, nph, nvel, gvec, dx, n_depth, &nseg, &nfail, split))) return rc;
        nseg_tot += nseg;
        int nsing = 0;
        if ((rc = run_solve_se(c, kmax, &nsing, false))) return rc;
        if (nsing) return set_err(c, PORTAL_ERR_SINGULAR, std::to_string(nsing) + " singular SE systems");
        PCHECK(c, cudaMemsetAsync(c->counters.p + 3, 0, sizeof(unsigned long long), c->stream));
        k_update<<<nb, tb, 0, c->stream>>>(N, c->bulk, nlev, c->pops.p, c->nmol.p, c->active_ab(), jl.p, c->levp.p,
                                           rho_prev.p, c->counters.p + 3);
        PCHECK(c, cudaGetLastError());
        unsigned long long rb = 0;
        PCHECK(c, cudaMemcpyAsync(&rb, c->counters.p + 3, sizeof rb, cudaMemcpyDeviceToHost, c->stream));
        PCHECK(c, cudaStreamSynchronize(c->stream));
        double rv;
        memcpy(&rv, &rb, sizeof rv);
        r = rv;
        if (residuals) residuals[it] = r;
        it++;
        if (r < tol) {
            if (!local_operator || verify) break;
            verify = true;  // an accelerated pass converged: a plain pass decides
            continue;
        }
        if (verify) {
            // the plain pass did not confirm: resume the accelerated passes
            // from its result, with a fresh Ng history (a different map)
            verify = false;
            if (ng_period > 0) {
                n_hist = 0;
                since_ng = 0;
                if (push_hist()) return PORTAL_ERR_CUDA;
            }
            continue;
        }
        if (ng_period > 0) {
            if (push_hist()) return PORTAL_ERR_CUDA;
            since_ng++;
            if (since_ng >= ng_period && n_hist >= 4) {
                const double *x3 = ring.p + (size_t)((n_hist - 1) % 4) * nv;
                const double *x2 = ring.p + (size_t)((n_hist - 2) % 4) * nv;
                const double *x1 = ring.p + (size_t)((n_hist - 3) % 4) * nv;
                const double *x0 = ring.p + (size_t)((n_hist - 4) % 4) * nv;
                k_ng_sums<<<nb, tb, 0, c->stream>>>(N, c->bulk, nlev, c->active_ab(), x0, x1, x2, x3, part.p);
                k_ng_final<<<1, 32, 0, c->stream>>>(nb, part.p, part.p + 5 * (size_t)nb);
                PCHECK(c, cudaGetLastError());
                double S[5];
                PCHECK(c, cudaMemcpyAsync(S, part.p + 5 * (size_t)nb, sizeof S, cudaMemcpyDeviceToHost, c->stream));
                PCHECK(c, cudaStreamSynchronize(c->stream));
                const double det = S[0] * S[2] - S[1] * S[1];
                if (det > 1e-14 * S[0] * S[2] && S[0] > 0.0 && S[2] > 0.0) {
                    const double a = (S[3] * S[2] - S[1] * S[4]) / det;
                    const double b = (S[0] * S[4] - S[1] * S[3]) / det;
                    if (std::isfinite(a) && std::isfinite(b)) {
                        k_ng_apply<<<nb, tb, 0, c->stream>>>(N, c->bulk, nlev, a, b, c->active_ab(), c->nmol.p, jl.p, x1,
                                                            x2, x3, rho_prev.p, c->levp.p);
                        PCHECK(c, cudaGetLastError());
                        // the extrapolated state starts a new plain sequence
                        n_hist = 0;
                        if (push_hist()) return PORTAL_ERR_CUDA;
                    }
                }
                since_ng = 0;
            }
        }
    }
    if (iterations) *iterations = it;
    if (n_segments) *n_segments = nseg_tot;
    if (pol_pops)
        PCHECK(c, cudaMemcpyAsync(pol_pops, c->pops.p, (size_t)N * 2 * nlev * sizeof(double),
                                  cudaMemcpyDeviceToHost, c->stream));
    if (lev_p_out)
        PCHECK(c, cudaMemcpyAsync(lev_p_out, c->levp.p, (size_t)N * nlev * sizeof(double),
                                  cudaMemcpyDeviceToHost, c->stream));
    PCHECK(c, cudaStreamSynchronize(c->stream));
    c->j_valid = false;
    c->ali_valid = false;
    return PORTAL_OK;
}
