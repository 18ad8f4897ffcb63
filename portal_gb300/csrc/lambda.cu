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
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace portal {
int run_radiation_field(portal_ctx *c, int nth, int nph, int nvel, const double *gvec, double dx,
                        int n_depth, long long *n_segments, int *n_failed);
int run_solve_se(portal_ctx *c, int kmax, int *n_singular);
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

}  // namespace

extern "C" int portal_lambda_iterate(portal_ctx *c, int nth, int nph, int nvel, const double *gvec,
                                     double dx, int n_depth, int kmax, double tol, int max_iter,
                                     const double *start_pops, double *pol_pops, double *lev_p_out,
                                     int *iterations, double *residuals, long long *n_segments) {
    if (!c) return PORTAL_ERR_ARG;
    if (!c->have_cloud || !c->have_mol) return set_err(c, PORTAL_ERR_STATE, "no cloud or molecule");
    if (max_iter < 1 || !(tol > 0.0)) return set_err(c, PORTAL_ERR_ARG, "portal_lambda_iterate: max_iter >= 1, tol > 0");
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
        k_rho_to_pops<<<nb, tb, 0, c->stream>>>(N, c->bulk, nlev, sp.p, c->nmol.p, c->ab.p, jl.p, c->levp.p);
        PCHECK(c, cudaGetLastError());
        PCHECK(c, cudaStreamSynchronize(c->stream));
    }
    k_pops_to_rho<<<nb, tb, 0, c->stream>>>(N, nlev, c->levp.p, c->nmol.p, jl.p, rho_prev.p);
    PCHECK(c, cudaGetLastError());
    long long nseg_tot = 0;
    int it = 0, rc = PORTAL_OK;
    double r = 1e300;
    while (it < max_iter) {
        long long nseg = 0;
        if ((rc = run_radiation_field(c, nth, nph, nvel, gvec, dx, n_depth, &nseg, nullptr))) return rc;
        nseg_tot += nseg;
        int nsing = 0;
        if ((rc = run_solve_se(c, kmax, &nsing))) return rc;
        if (nsing) return set_err(c, PORTAL_ERR_SINGULAR, std::to_string(nsing) + " singular SE systems");
        PCHECK(c, cudaMemsetAsync(c->counters.p + 3, 0, sizeof(unsigned long long), c->stream));
        k_update<<<nb, tb, 0, c->stream>>>(N, c->bulk, nlev, c->pops.p, c->nmol.p, c->ab.p, jl.p, c->levp.p,
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
        if (r < tol) break;
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
    return PORTAL_OK;
}
