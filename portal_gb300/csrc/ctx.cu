// Context lifetime, molecule / cloud ingestion into the device layout.
//
// Device layout of a cloud (N nodes, nnz directed Delaunay edges):
//   pos64  (3,N) FP64   node positions (normalised by r_max), for per-ray
//                       FP64 set-up (direction, sphere exit)
//   cellv  (N) float4   (v_x, v_y, v_z, b) -- what the ray integration
//                       gathers per crossed cell
//   nb_off (N+1), nb_idx (nnz)  neighbour CSR, ascending ids per node as
//                       SortUnique leaves them (unique.f90:43-59)
//   edge   (nnz) float4 (e, |e|^2/2) with e = X_n - X_c evaluated in FP64:
//                       the Voronoi face between c and n is
//                       { P : e.(P - X_c) = |e|^2/2 }, so a walk that keeps
//                       its photon position relative to the current node
//                       finds every face crossing in FP32 without absolute
//                       coordinates
//   levp   (nlev,N) FP64 level populations, plus the per-node scalars
//                       (b, T_kin, T_dust, dust, n_H2, abundance) in FP64.
#include <cmath>
#include <cstring>

#include "common.cuh"

using namespace portal;

extern "C" const char *portal_strerror(int code) {
    switch (code) {
    case PORTAL_OK: return "ok";
    case PORTAL_ERR_CUDA: return "CUDA error";
    case PORTAL_ERR_ARG: return "invalid argument";
    case PORTAL_ERR_STATE: return "missing cloud, molecule or preceding result";
    case PORTAL_ERR_DEPTH: return "a ray walk needed more cells than n_depth (adjust n_depth parameter! Make it bigger.)";
    case PORTAL_ERR_SINGULAR: return "Density-matrix calculation: failed (singular SE matrix)";
    case PORTAL_ERR_NOMEM: return "device memory allocation failed";
    case PORTAL_ERR_NODEVICE: return "no usable CUDA device for this sm_103a build";
    default: return "unknown error";
    }
}

static std::string g_create_err;

extern "C" const char *portal_last_error(const portal_ctx *ctx) {
    return ctx ? ctx->err.c_str() : g_create_err.c_str();
}

extern "C" int portal_create(portal_ctx **out, int device) {
    if (!out) return PORTAL_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev <= device || device < 0) {
        g_create_err = std::string("no CUDA device ") + std::to_string(device) + ": " +
                       (e == cudaSuccess ? "not present" : cudaGetErrorString(e));
        return PORTAL_ERR_NODEVICE;
    }
    e = cudaSetDevice(device);
    if (e != cudaSuccess) { g_create_err = cudaGetErrorString(e); return PORTAL_ERR_CUDA; }
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, device);
    if (prop.major != 10 || prop.minor != 3) {
        g_create_err = std::string("device ") + prop.name + " is sm_" + std::to_string(prop.major) +
                       std::to_string(prop.minor) + "; this library is built for sm_103a only";
        return PORTAL_ERR_NODEVICE;
    }
    portal_ctx *c = new portal_ctx();
    c->device = device;
    c->sm_count = prop.multiProcessorCount;
    e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { g_create_err = cudaGetErrorString(e); delete c; return PORTAL_ERR_CUDA; }
    c->stream = c->own_stream;
    for (int i = 0; i < 2 * T_NSLOT; i++) cudaEventCreate(&c->ev[i]);
    c->ev_ready = true;
    if (c->counters.reserve(8) != cudaSuccess) { delete c; return PORTAL_ERR_NOMEM; }
    *out = c;
    return PORTAL_OK;
}

extern "C" int portal_destroy(portal_ctx *c) {
    if (!c) return PORTAL_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->ev_ready)
        for (int i = 0; i < 2 * T_NSLOT; i++) cudaEventDestroy(c->ev[i]);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    delete c;  // DevBuf destructors free device memory
    return PORTAL_OK;
}

extern "C" int portal_set_molecule(portal_ctx *c, int nlev, const int *j_lev, const double *e_levs,
                                   int r_num, const int *r_trans, const double *t_Aji,
                                   const double *nu, const double *t_Bij, const double *kd_v,
                                   int c_num, const int *c_trans, int c_temp, int c_par,
                                   const double *col_temps, const double *t_Cji) {
    if (!c) return PORTAL_ERR_ARG;
    if (nlev < 1 || r_num < 1 || c_num < 0 || c_temp < 1 || c_par < 1 || c_par > 2 || !j_lev ||
        !e_levs || !r_trans || !t_Aji || !nu || !t_Bij || !kd_v || !col_temps ||
        (c_num > 0 && (!c_trans || !t_Cji)))
        return set_err(c, PORTAL_ERR_ARG, "portal_set_molecule: bad sizes or NULL array");
    for (int i = 0; i < 2 * r_num; i++)
        if (r_trans[i] < 1 || r_trans[i] > nlev)
            return set_err(c, PORTAL_ERR_ARG, "portal_set_molecule: r_trans level out of range");
    for (int i = 0; i < 2 * c_num; i++)
        if (c_trans[i] < 1 || c_trans[i] > nlev)
            return set_err(c, PORTAL_ERR_ARG, "portal_set_molecule: c_trans level out of range");
    for (int i = 0; i < nlev; i++)
        if (j_lev[i] < 0 || j_lev[i] > 60)
            return set_err(c, PORTAL_ERR_ARG, "portal_set_molecule: J out of range 0..60");
    c->nlev = nlev; c->r_num = r_num; c->c_num = c_num; c->c_temp = c_temp; c->c_par = c_par;
    c->j_lev.assign(j_lev, j_lev + nlev);
    c->e_levs.assign(e_levs, e_levs + nlev);
    c->r_trans.assign(r_trans, r_trans + 2 * r_num);
    c->A.assign(t_Aji, t_Aji + r_num);
    c->nu.assign(nu, nu + r_num);
    c->Bij.assign(t_Bij, t_Bij + r_num);
    c->kd_v.assign(kd_v, kd_v + r_num);
    c->c_trans.assign(c_trans, c_trans + 2 * c_num);
    c->col_temps.assign(col_temps, col_temps + c_temp);
    c->Cji.assign(t_Cji, t_Cji + (size_t)c_temp * c_num * c_par);
    c->have_mol = true;
    c->se_kmax = -1;  // SE program must be rebuilt
    c->j_valid = false;
    c->ali_valid = false;
    return PORTAL_OK;
}

// Edge geometry from the FP64 positions; one thread per (node, slot).
__global__ void k_build_edges(int N, int maxne, const int *__restrict__ del_ne,
                              const int *__restrict__ off, const double *__restrict__ pos,
                              int *__restrict__ nb_idx, float4 *__restrict__ edge) {
    long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long tot = (long long)N * maxne;
    if (tid >= tot) return;
    int s = (int)(tid / N);
    int i = (int)(tid - (long long)s * N);
    int o = off[i], deg = off[i + 1] - o;
    if (s >= deg) return;
    int nb = del_ne[(size_t)i + (size_t)N * s] - 1;
    double ex = pos[3 * (size_t)nb] - pos[3 * (size_t)i];
    double ey = pos[3 * (size_t)nb + 1] - pos[3 * (size_t)i + 1];
    double ez = pos[3 * (size_t)nb + 2] - pos[3 * (size_t)i + 2];
    double h = 0.5 * (ex * ex + ey * ey + ez * ez);
    nb_idx[o + s] = nb;
    edge[o + s] = make_float4((float)ex, (float)ey, (float)ez, (float)h);
}

__global__ void k_cellv(int N, const double *__restrict__ vel, const double *__restrict__ b,
                        float4 *__restrict__ cellv) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    cellv[i] = make_float4((float)vel[3 * (size_t)i], (float)vel[3 * (size_t)i + 1],
                           (float)vel[3 * (size_t)i + 2], (float)b[i]);
}

static int upload(portal_ctx *c, double *dst, const double *src, size_t n) {
    PCHECK(c, cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    return PORTAL_OK;
}

static int star_refresh(portal_ctx *c);

extern "C" int portal_set_cloud(portal_ctx *c, int N, int bulk, int nlev, const double *xyz,
                                const double *vel_all, const double *b_all, const double *temp_all,
                                const double *dust_p, const double *h2_dens, const double *ab_all,
                                const double *lev_p, const double *bvec_all, int maxne,
                                const int *del_ne, const int *del_num_ne, double tx) {
    if (!c) return PORTAL_ERR_ARG;
    if (N < 1 || bulk < 0 || bulk > N || nlev < 1 || maxne < 1 || !xyz || !vel_all || !b_all ||
        !temp_all || !dust_p || !h2_dens || !ab_all || !lev_p || !bvec_all || !del_ne ||
        !del_num_ne || !(tx > 0.0))
        return set_err(c, PORTAL_ERR_ARG, "portal_set_cloud: bad sizes or NULL array");
    if (c->have_mol && nlev != c->nlev)
        return set_err(c, PORTAL_ERR_ARG, "portal_set_cloud: nlev differs from the molecule's");
    cudaSetDevice(c->device);
    // CSR offsets + validation on the host (cheap, and fails loudly before
    // any kernel can read out of bounds)
    std::vector<int> off(N + 1);
    off[0] = 0;
    int maxdeg = 0;
    for (int i = 0; i < N; i++) {
        int d = del_num_ne[i];
        if (d < 0 || d > maxne)
            return set_err(c, PORTAL_ERR_ARG, "portal_set_cloud: del_num_ne outside 0..maxne");
        if ((long long)off[i] + d > 2000000000LL)
            return set_err(c, PORTAL_ERR_ARG, "portal_set_cloud: more than 2e9 neighbour entries");
        off[i + 1] = off[i] + d;
        if (d > maxdeg) maxdeg = d;
        for (int s = 0; s < d; s++) {
            int nb = del_ne[(size_t)i + (size_t)N * s];
            if (nb < 1 || nb > N || nb == i + 1)
                return set_err(c, PORTAL_ERR_ARG, "portal_set_cloud: neighbour id out of range");
        }
    }
    int nnz = off[N];
    c->have_cloud = false;
    c->j_valid = false;
    c->ali_valid = false;
    if (c->pos64.reserve(3 * (size_t)N) || c->bvec64.reserve(3 * (size_t)N) ||
        c->cellv.reserve(N) || c->nb_off.reserve(N + 1) || c->nb_idx.reserve(nnz) ||
        c->edge.reserve(nnz) || c->levp.reserve((size_t)nlev * N) || c->b64.reserve(N) ||
        c->tkin.reserve(N) || c->tdust.reserve(N) || c->dustp.reserve(N) || c->h2.reserve(N) ||
        c->ab.reserve(N) || c->status.reserve(N) || c->nmol.reserve(N))
        return set_err(c, PORTAL_ERR_NOMEM, "portal_set_cloud: device allocation failed");
    std::vector<double> tk(N), td(N), nm(N);
    bool dust = false;
    for (int i = 0; i < N; i++) {
        tk[i] = temp_all[2 * (size_t)i];
        td[i] = temp_all[2 * (size_t)i + 1];
        double s = 0.0;
        for (int l = 0; l < nlev; l++) s += lev_p[(size_t)nlev * i + l];
        nm[i] = s;
        if (dust_p[i] != 0.0) dust = true;
    }
    int rc;
    if ((rc = upload(c, c->pos64.p, xyz, 3 * (size_t)N))) return rc;
    if ((rc = upload(c, c->bvec64.p, bvec_all, 3 * (size_t)N))) return rc;
    if ((rc = upload(c, c->levp.p, lev_p, (size_t)nlev * N))) return rc;
    if ((rc = upload(c, c->b64.p, b_all, N))) return rc;
    if ((rc = upload(c, c->tkin.p, tk.data(), N))) return rc;
    if ((rc = upload(c, c->tdust.p, td.data(), N))) return rc;
    if ((rc = upload(c, c->dustp.p, dust_p, N))) return rc;
    if ((rc = upload(c, c->h2.p, h2_dens, N))) return rc;
    if ((rc = upload(c, c->ab.p, ab_all, N))) return rc;
    if ((rc = upload(c, c->nmol.p, nm.data(), N))) return rc;
    PCHECK(c, cudaMemcpyAsync(c->nb_off.p, off.data(), (N + 1) * sizeof(int),
                              cudaMemcpyHostToDevice, c->stream));
    DevBuf<int> dne;
    if (dne.reserve((size_t)N * maxne) || c->vel64.reserve(3 * (size_t)N))
        return set_err(c, PORTAL_ERR_NOMEM, "portal_set_cloud: staging allocation failed");
    PCHECK(c, cudaMemcpyAsync(dne.p, del_ne, (size_t)N * maxne * sizeof(int),
                              cudaMemcpyHostToDevice, c->stream));
    PCHECK(c, cudaMemcpyAsync(c->vel64.p, vel_all, 3 * (size_t)N * sizeof(double),
                              cudaMemcpyHostToDevice, c->stream));
    long long tot = (long long)N * maxne;
    k_build_edges<<<(unsigned)((tot + 255) / 256), 256, 0, c->stream>>>(N, maxne, dne.p, c->nb_off.p,
                                                                      c->pos64.p, c->nb_idx.p,
                                                                      c->edge.p);
    PCHECK(c, cudaGetLastError());
    k_cellv<<<(N + 255) / 256, 256, 0, c->stream>>>(N, c->vel64.p, c->b64.p, c->cellv.p);
    PCHECK(c, cudaGetLastError());
    PCHECK(c, cudaStreamSynchronize(c->stream));  // staging buffers die at scope end
    c->N = N; c->bulk = bulk; c->nnz = nnz; c->maxdeg = maxdeg; c->tx = tx;
    c->has_dust = dust;
    if (!c->have_mol) c->nlev = nlev;
    c->have_cloud = true;
    return star_refresh(c);
}

namespace {
// star mode: the node loop skips nodes with |X| <= R_star (main_para.f90:232,
// which compares |X| with R_star, the star taken as centred)
__global__ void k_star_mask(int N, double R, const double *__restrict__ pos, const double *__restrict__ ab,
                            double *__restrict__ out) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    const double x = pos[3 * (size_t)n], y = pos[3 * (size_t)n + 1], z = pos[3 * (size_t)n + 2];
    out[n] = (__dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z))) > R) ? ab[n]
                                                                                                      : 0.0;
}
}  // namespace

// The abundances with the star's interior masked out (star mode, with a cloud).
static int star_refresh(portal_ctx *c) {
    if (!c->star_mode || !c->have_cloud) return PORTAL_OK;
    if (c->ab_star.reserve(c->N)) return set_err(c, PORTAL_ERR_NOMEM, "star mask");
    k_star_mask<<<(c->N + 255) / 256, 256, 0, c->stream>>>(c->N, c->R_star(), c->pos64.p, c->ab.p, c->ab_star.p);
    PCHECK(c, cudaGetLastError());
    PCHECK(c, cudaStreamSynchronize(c->stream));
    return PORTAL_OK;
}

extern "C" int portal_set_star(portal_ctx *c, int star_mod, double T_star, double R_star,
                               const double *X_star) {
    if (!c) return PORTAL_ERR_ARG;
    if (star_mod != 0 && star_mod != 1) return set_err(c, PORTAL_ERR_ARG, "portal_set_star: star_mod 0 or 1");
    if (star_mod == 1 && (!X_star || !(R_star > 0.0) || !(T_star >= 0.0)))
        return set_err(c, PORTAL_ERR_ARG, "portal_set_star: R_star > 0, T_star >= 0 and X_star(3) needed");
    cudaSetDevice(c->device);
    c->star_mode = star_mod;
    c->T_star = star_mod ? T_star : 0.0;
    c->R_star_m = star_mod ? R_star : 0.0;
    for (int k = 0; k < 3; k++) c->X_star[k] = star_mod ? X_star[k] : 0.0;
    c->j_valid = false;
    c->ali_valid = false;
    return star_refresh(c);
}

extern "C" int portal_set_populations(portal_ctx *c, const double *lev_p) {
    if (!c || !lev_p) return PORTAL_ERR_ARG;
    if (!c->have_cloud) return set_err(c, PORTAL_ERR_STATE, "portal_set_populations: no cloud");
    cudaSetDevice(c->device);
    PCHECK(c, cudaMemcpyAsync(c->levp.p, lev_p, (size_t)c->nlev * c->N * sizeof(double),
                              cudaMemcpyHostToDevice, c->stream));
    PCHECK(c, cudaStreamSynchronize(c->stream));
    c->j_valid = false;
    c->ali_valid = false;
    return PORTAL_OK;
}

extern "C" int portal_set_stream(portal_ctx *c, void *stream) {
    if (!c) return PORTAL_ERR_ARG;
    cudaSetDevice(c->device);
    PCHECK(c, cudaStreamSynchronize(c->stream));
    c->stream = stream ? (cudaStream_t)stream : c->own_stream;
    return PORTAL_OK;
}

extern "C" int portal_get_results(portal_ctx *c, double *J0, double *J2, double *pol_pops, int *status) {
    if (!c) return PORTAL_ERR_ARG;
    if (!c->j_valid) return set_err(c, PORTAL_ERR_STATE, "no device-resident results");
    cudaSetDevice(c->device);
    const size_t LN = (size_t)c->r_num * c->N;
    if (J0) PCHECK(c, cudaMemcpyAsync(J0, c->J0.p, LN * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if (J2) PCHECK(c, cudaMemcpyAsync(J2, c->J2.p, LN * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if (pol_pops) {
        if (!c->pops.p || c->se_kmax < 0) return set_err(c, PORTAL_ERR_STATE, "no device-resident populations");
        PCHECK(c, cudaMemcpyAsync(pol_pops, c->pops.p, (size_t)c->N * 2 * c->nlev * sizeof(double),
                                  cudaMemcpyDeviceToHost, c->stream));
    }
    if (status)
        PCHECK(c, cudaMemcpyAsync(status, c->status.p, (size_t)c->N * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    PCHECK(c, cudaStreamSynchronize(c->stream));
    return PORTAL_OK;
}

extern "C" int portal_last_kernel_times(const portal_ctx *c, double *times_ms, int *launches, int n) {
    if (!c) return PORTAL_ERR_ARG;
    for (int i = 0; i < n && i < T_NSLOT; i++) {
        if (times_ms) times_ms[i] = c->t_ms[i];
        if (launches) launches[i] = c->t_launch[i];
    }
    return PORTAL_OK;
}

namespace portal {

void gauss_legendre(int n, double *x, double *w) {
    const long double pi = 3.141592653589793238462643383279502884L;
    for (int i = 0; i < n; i++) {
        long double z = cosl(pi * (i + 0.75L) / (n + 0.5L)), pp = 1.0L;
        for (int it = 0; it < 100; it++) {
            long double p0 = 1.0L, p1 = z;
            for (int k = 2; k <= n; k++) {
                long double p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            if (n == 1) { p1 = z; p0 = 1.0L; }
            pp = n * (z * p1 - p0) / (z * z - 1.0L);
            long double dz = p1 / pp;
            z -= dz;
            if (fabsl(dz) < 1e-19L) break;
        }
        long double p0 = 1.0L, p1 = z;
        for (int k = 2; k <= n; k++) {
            long double p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
            p0 = p1;
            p1 = p2;
        }
        pp = n * (z * p1 - p0) / (z * z - 1.0L);
        x[n - 1 - i] = (double)z;
        w[n - 1 - i] = (double)(2.0L / ((1.0L - z * z) * pp * pp));
    }
}

int legendre_all(int nth, int nph, std::vector<double> &xth) {
    const double pi = std::acos(-1.0);
    std::vector<double> x(nth), w(nth);
    gauss_legendre(nth, x.data(), w.data());
    xth.clear();
    int n = 0;
    for (int i = 0; i < nth; i++) {
        int np = (int)std::ceil(nph * std::sin(std::acos(x[i])));
        double w_ph = 2.0 * pi / np;
        double ww = w_ph * w[i];
        for (int j = 1; j <= np; j++) {
            xth.push_back(x[i]);
            xth.push_back((j - 1) * w_ph);
            xth.push_back(ww / (4.0 * pi));
            n++;
        }
    }
    return n;
}

}  // namespace portal
