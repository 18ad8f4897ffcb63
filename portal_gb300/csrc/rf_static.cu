// Radiation field without any device allocation.
//
// Some callers cannot call cudaMalloc: code running inside a host that owns
// all device memory through its own pool (a Fortran program built with CUDA
// Fortran device arrays, a solver framework that hands out pre-sized
// buffers), or code that must not allocate between two steps of a
// simulation.  For them this file provides portal_radiation_field_static: the
// same computation as portal_radiation_field (inverse_rt of every bulk node),
// reading the reference-layout arrays the caller already keeps on the
// device, writing J^0_0 / J^2_0 into the caller's device buffers, and using
// as scratch only the fixed array `g_rf_scratch` below, which is part of the
// library image: every GPU that loads the library holds its 64 MiB until the
// process exits.
//
// The kernel is a variant of k_radiation_field (rf.cu): the same
// thread-per-ray Voronoi walk and lanes-over-channels integration, but the
// face geometry, cell velocities and line opacities are formed on the fly
// from the reference-layout arrays instead of the context's precomputed
// tables, and the grid is fixed so that the walk lists fit the static array.
#include <cmath>
#include <cstdlib>
#include <mutex>
#include <vector>

#include "common.cuh"

using namespace portal;

namespace {

// ---- the static scratch ---------------------------------------------------
constexpr size_t RS_BYTES = 64ull << 20;          // 64 MiB
constexpr int RS_BLOCKS = 152, RS_WARPS = 2;       // fixed grid: 304 warps
constexpr int RS_MAX_DIRS = 8192;                  // direction table capacity
constexpr int RS_MAX_CH = 288;                     // velocity channels
constexpr int RS_MAX_LINES = 64;
// layout: [0, 256) counters | [256, +48*RS_MAX_DIRS) directions (6 doubles)
//         | channel tables (2 * RS_MAX_CH floats) | walk lists (int2)
constexpr size_t RS_OFF_DIRS = 256;
constexpr size_t RS_OFF_CH = RS_OFF_DIRS + 48ull * RS_MAX_DIRS;
constexpr size_t RS_OFF_WALK = (RS_OFF_CH + 8ull * RS_MAX_CH + 255) & ~255ull;
constexpr size_t RS_WALK_ENTRIES = (RS_BYTES - RS_OFF_WALK) / sizeof(int2);
// longest walk (cells per ray) the array can hold: 32 rays per warp
constexpr int RS_MAX_DEPTH = (int)(RS_WALK_ENTRIES / ((size_t)RS_BLOCKS * RS_WARPS * 32));

static __device__ __align__(256) unsigned char g_rf_scratch[RS_BYTES];

struct RsLine {
    double nu, A, B, kd, glo, gup, bb_cmb;
    int lo, up;
};
__constant__ RsLine c_rs_lines[RS_MAX_LINES];

struct RsArgs {
    int N, bulk, nlev, L, nvel, nch, ndir, n_depth, maxne;
    float dx32;
    double tdx;  // tx * dx
    double gx, gy, gz;
    const double *xyz, *vel, *b_all, *temp_all, *dust_p, *ab, *lev_p, *bvec;
    const int *del_ne, *del_num_ne;
    double *J0, *J2;
    int *status;
    unsigned char *scratch;
};

__device__ __forceinline__ float rs_ex2(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// ray_in's opacity factors of one (cell, line) (inverse_rt.f90:263-301), the
// same FP64 expressions the context path tabulates
__device__ float4 rs_line_coef(const RsArgs &a, int n, int l) {
    const RsLine lc = c_rs_lines[l];
    const double p1 = a.lev_p[(size_t)a.nlev * n + lc.lo];
    const double p2 = a.lev_p[(size_t)a.nlev * n + lc.up];
    const double c1 = 2.2102191e-42 * lc.nu, c2 = 5.272859e-35 * lc.nu;
    const double cnu = 299792458.0 / lc.nu;
    const double kv = c1 * lc.B * (p1 - lc.glo * p2 / lc.gup);
    const double ev = c2 * lc.A * p2;
    const double phif = cnu / (1.7724538509055160273 * a.b_all[n]) * a.tdx;
    const double Ad = lc.kd * a.dust_p[n] * a.tdx;
    const double Td = a.temp_all[2 * (size_t)n + 1];
    double Ibb = 0.0;
    if (Td != 0.0) Ibb = 1.4744995e-50 * lc.nu * lc.nu * lc.nu / (exp(4.79924e-11 / Td * lc.nu) - 1.0);
    // the line's source function as the FP64 ratio (full FP32 precision for
    // weak lines whose kv, ev alone would be FP32 denormals)
    return make_float4((float)(kv * phif), (float)(kv != 0.0 ? ev / kv : 0.0), (float)Ad, (float)(Ad * Ibb));
}

constexpr int RS_NLG = 5;
constexpr float RS_LOG2E = 1.4426950408889634f;
constexpr float RS_FACE_EPS = 2e-8f;

template <int NS>
__global__ void __launch_bounds__(64, 1) k_rf_static(RsArgs a) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const long long gw = (long long)blockIdx.x * RS_WARPS + wib;
    unsigned long long *counter = (unsigned long long *)a.scratch;
    const double *dirs = (const double *)(a.scratch + RS_OFF_DIRS);
    const float *chq = (const float *)(a.scratch + RS_OFF_CH);
    const float *chw = chq + RS_MAX_CH;
    int2 *const wbase = (int2 *)(a.scratch + RS_OFF_WALK) + (size_t)gw * 32 * a.n_depth;
    __shared__ float s_q0[RS_WARPS][32], s_dq[RS_WARPS][32];
    __shared__ float4 s_c[RS_WARPS][32][RS_NLG];
    __shared__ float4 s_dir[RS_WARPS][32];
    __shared__ int s_K[RS_WARPS][32];
    for (;;) {
        int node = 0;
        if (lane == 0) node = (int)atomicAdd(counter, 1ULL);
        node = __shfl_sync(FULL, node, 0);
        if (node >= a.bulk) break;
        double acc0a = 0.0, acc0b = 0.0, acc2a = 0.0, acc2b = 0.0;
        int st = 0;
        if (a.ab[node] > 0.0) {
            const double bx = a.bvec[3 * (size_t)node], by = a.bvec[3 * (size_t)node + 1],
                         bz = a.bvec[3 * (size_t)node + 2];
            double xx = by * a.gz - bz * a.gy, xy = bz * a.gx - bx * a.gz, xz = bx * a.gy - by * a.gx;
            const double xn = sqrt(xx * xx + xy * xy + xz * xz);
            xx /= xn; xy /= xn; xz /= xn;
            const double wx = xy * bz - xz * by, wy = xz * bx - xx * bz, wz = xx * by - xy * bx;
            const double px = a.xyz[3 * (size_t)node], py = a.xyz[3 * (size_t)node + 1],
                         pz = a.xyz[3 * (size_t)node + 2];
            const float vnx = (float)a.vel[3 * (size_t)node], vny = (float)a.vel[3 * (size_t)node + 1],
                        vnz = (float)a.vel[3 * (size_t)node + 2];
            const float bnode = (float)a.b_all[node];
            const float dqfac = 2.f * bnode / (float)a.nvel;
            for (int k0 = 0; k0 < a.ndir && st == 0; k0 += 32) {
                const int nr = min(32, a.ndir - k0);
                int K = 0;
                bool over = false;
                if (lane < nr) {
                    const double *dr = dirs + 6 * (size_t)(k0 + lane);
                    const double dx = dr[0] * bx + dr[1] * (dr[2] * wx + dr[3] * xx);
                    const double dy = dr[0] * by + dr[1] * (dr[2] * wy + dr[3] * xy);
                    const double dz = dr[0] * bz + dr[1] * (dr[2] * wz + dr[3] * xz);
                    const double sexit = sphere_exit(px, py, pz, dx, dy, dz);
                    const float fdx = (float)dx, fdy = (float)dy, fdz = (float)dz;
                    s_dir[wib][lane] = make_float4(fdx, fdy, fdz, vnx * fdx + vny * fdy + vnz * fdz);
                    int2 *wl = wbase + (size_t)lane * a.n_depth;
                    double s = 0.0;
                    float rx = 0.f, ry = 0.f, rz = 0.f;
                    int c = node;
                    for (;;) {
                        const float tsph = (float)(sexit - s);
                        const int deg = a.del_num_ne[c];
                        const double cx = a.xyz[3 * (size_t)c], cy = a.xyz[3 * (size_t)c + 1],
                                     cz = a.xyz[3 * (size_t)c + 2];
                        float bnum = tsph, bden = 1.f, bex = 0.f, bey = 0.f, bez = 0.f;
                        int bnb = -1;
                        for (int j = 0; j < deg; j++) {
                            const int nb = a.del_ne[(size_t)c + (size_t)a.N * j] - 1;
                            const double ex = a.xyz[3 * (size_t)nb] - cx, ey = a.xyz[3 * (size_t)nb + 1] - cy,
                                         ez = a.xyz[3 * (size_t)nb + 2] - cz;
                            const float fex = (float)ex, fey = (float)ey, fez = (float)ez;
                            const float h = (float)(0.5 * (ex * ex + ey * ey + ez * ez));
                            const float den = fex * fdx + fey * fdy + fez * fdz;
                            const float num = h - (fex * rx + fey * ry + fez * rz);
                            if (den > 0.f && num > RS_FACE_EPS * den && num * bden <= bnum * den) {
                                bnum = num; bden = den; bnb = nb;
                                bex = fex; bey = fey; bez = fez;
                            }
                        }
                        const float delta = (bnb < 0) ? tsph : bnum / bden;
                        if (K >= a.n_depth) { over = true; break; }
                        wl[K] = make_int2(c, (int)roundf(delta / a.dx32));
                        K++;
                        if (bnb < 0) break;
                        s += (double)delta;
                        rx = fmaf(delta, fdx, rx) - bex;
                        ry = fmaf(delta, fdy, ry) - bey;
                        rz = fmaf(delta, fdz, rz) - bez;
                        c = bnb;
                    }
                }
                s_K[wib][lane] = over ? -1 : K;
                if (__any_sync(FULL, over)) { st |= PORTAL_NODE_DEPTH; break; }
                __syncwarp();
                for (int rr = 0; rr < nr; rr++) {
                    const int Kr = s_K[wib][rr];
                    const int2 *wl = wbase + (size_t)rr * a.n_depth;
                    const float4 d4 = s_dir[wib][rr];
                    const double *dr = dirs + 6 * (size_t)(k0 + rr);
                    const int steps0 = wl[0].y;
                    for (int l0 = 0; l0 < a.L; l0 += RS_NLG) {
                        float I[NS][RS_NLG];
#pragma unroll
                        for (int l = 0; l < RS_NLG; l++) {
                            const float bb = (l0 + l < a.L) ? (float)c_rs_lines[l0 + l].bb_cmb : 0.f;
#pragma unroll
                            for (int s2 = 0; s2 < NS; s2++) I[s2][l] = bb;
                        }
                        for (int hi = Kr - 1; hi >= 1; hi -= 32) {
                            const int nc = min(32, hi);
                            __syncwarp();
                            if (lane < nc) {
                                const int2 wc = wl[hi - lane];
                                const float vp = (float)a.vel[3 * (size_t)wc.x] * d4.x +
                                                 (float)a.vel[3 * (size_t)wc.x + 1] * d4.y +
                                                 (float)a.vel[3 * (size_t)wc.x + 2] * d4.z;
                                const float ib = 1.f / (float)a.b_all[wc.x];
                                s_q0[wib][lane] = (d4.w - vp) * ib;
                                s_dq[wib][lane] = dqfac * ib;
                                const float fst = (float)wc.y;
#pragma unroll
                                for (int l = 0; l < RS_NLG; l++)
                                    if (l0 + l < a.L) {
                                        const float4 v = rs_line_coef(a, wc.x, l0 + l);
                                        const float tc = v.x * fst;  // line-centre optical depth
                                        s_c[wib][lane][l] = make_float4(tc, v.y * tc, v.z * fst, v.w * fst);
                                    }
                            }
                            __syncwarp();
                            for (int u = 0; u < nc; u++) {
                                const float q0 = s_q0[wib][u], dq = s_dq[wib][u];
                                float g[NS];
#pragma unroll
                                for (int s2 = 0; s2 < NS; s2++) {
                                    const float q = fmaf(dq, (float)(lane + 32 * s2 - a.nvel), q0);
                                    g[s2] = rs_ex2(-q * q * RS_LOG2E);
                                }
#pragma unroll
                                for (int l = 0; l < RS_NLG; l++) {
                                    if (l0 + l < a.L) {
                                        const float4 cf = s_c[wib][u][l];
#pragma unroll
                                        for (int s2 = 0; s2 < NS; s2++) {
                                            // tau = (kv phi + alpha) dx n, S = (ev phi + j)/(kv phi + alpha)
                                            const float tau = fmaf(cf.x, g[s2], cf.z);
                                            const float Sv = fmaf(cf.y, g[s2], cf.w) / tau;
                                            const float x = tau * RS_LOG2E;
                                            const float om = one_minus_exp(x, rs_ex2(-x));
                                            const float In = fmaf(om, Sv - I[s2][l], I[s2][l]);
                                            I[s2][l] = (tau > 1e-30f) ? In : I[s2][l];
                                        }
                                    }
                                }
                            }
                        }
                        // central cell and the weighted channel sum (inverse_rt.f90:320-339)
                        float part[RS_NLG];
#pragma unroll
                        for (int l = 0; l < RS_NLG; l++) {
                            part[l] = 0.f;
                            if (l0 + l < a.L) {
                                const float4 v = rs_line_coef(a, node, l0 + l);
#pragma unroll
                                for (int s2 = 0; s2 < NS; s2++) {
                                    const int ch = lane + 32 * s2;
                                    if (ch < a.nch) {
                                        const float g0 = rs_ex2(-chq[ch] * chq[ch] * RS_LOG2E);
                                        const float kap = fmaf(v.x, g0, v.z);
                                        const float tau = kap * (float)steps0;
                                        const float Sv = fmaf(v.y * v.x, g0, v.w) / kap;
                                        const float x = tau * RS_LOG2E;
                                        const float om = one_minus_exp(x, rs_ex2(-x));
                                        part[l] = fmaf(chw[ch], fmaf(om, Sv - I[s2][l], I[s2][l]), part[l]);
                                    }
                                }
                            }
                        }
#pragma unroll
                        for (int l = 0; l < RS_NLG; l++) {
                            float v = part[l];
#pragma unroll
                            for (int o2 = 16; o2 >= 1; o2 >>= 1) v += __shfl_xor_sync(FULL, v, o2);
                            const int line = l0 + l;
                            if (line < a.L && (line & 31) == lane) {
                                if (line < 32) { acc0a += dr[4] * (double)v; acc2a += dr[5] * (double)v; }
                                else { acc0b += dr[4] * (double)v; acc2b += dr[5] * (double)v; }
                            }
                        }
                    }
                }
                __syncwarp();
            }
        }
        if (lane < a.L) {
            a.J0[(size_t)node * a.L + lane] = st ? 0.0 : acc0a;
            a.J2[(size_t)node * a.L + lane] = st ? 0.0 : acc2a;
        }
        if (lane + 32 < a.L) {
            a.J0[(size_t)node * a.L + lane + 32] = st ? 0.0 : acc0b;
            a.J2[(size_t)node * a.L + lane + 32] = st ? 0.0 : acc2b;
        }
        if (lane == 0 && a.status) a.status[node] = st;
        __syncwarp();
    }
}

// The host side of each call's line constants, direction and channel
// tables.  Kept in static storage (not on the call's stack) so that the
// memory a copy reads from stays valid after the call returns; filled and
// copied under g_rs_tables_mutex.
std::mutex g_rs_tables_mutex;
RsLine g_rs_hlines[RS_MAX_LINES];
double g_rs_hdirs[6 * RS_MAX_DIRS];
float g_rs_hch[2 * RS_MAX_CH];

}  // namespace

extern "C" int portal_radiation_field_static(
    void *cuda_stream, int node_num, int bulk_node_num, int nlev, const double *xyz,
    const double *vel_all, const double *b_all, const double *temp_all, const double *dust_p,
    const double *ab_all, const double *lev_p, const double *bvec_all, int maxne, const int *del_ne,
    const int *del_num_ne, double tx, const int *j_lev, int r_num, const int *r_trans,
    const double *t_Aji, const double *nu, const double *t_Bij, const double *kd_v, int nth, int nph,
    int nvel, const double *gvec, double dx, int n_depth, double *J0, double *J2, int *status) {
    if (node_num < 1 || bulk_node_num < 0 || bulk_node_num > node_num || nlev < 1 || maxne < 1 ||
        !xyz || !vel_all || !b_all || !temp_all || !dust_p || !ab_all || !lev_p || !bvec_all ||
        !del_ne || !del_num_ne || !(tx > 0.0) || !j_lev || r_num < 1 || !r_trans || !t_Aji || !nu ||
        !t_Bij || !kd_v || nth < 1 || nph < 1 || nvel < 1 || !gvec || !(dx > 0.0) || n_depth < 1 ||
        !J0 || !J2)
        return PORTAL_ERR_ARG;
    if (r_num > RS_MAX_LINES || 2 * nvel + 1 > RS_MAX_CH || nth * nph > RS_MAX_DIRS ||
        n_depth > RS_MAX_DEPTH)
        return PORTAL_ERR_ARG;  // beyond the static scratch (see portal_radiation_field_static_limits)
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return PORTAL_ERR_NODEVICE;
    // the current device's address of g_rf_scratch, looked up on every call
    // (a cached address would go stale when the module is reloaded)
    unsigned char *scratch = nullptr;
    {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_rf_scratch) != cudaSuccess || !p) return PORTAL_ERR_CUDA;
        scratch = (unsigned char *)p;
    }
    cudaStream_t st = (cudaStream_t)cuda_stream;
    for (int k = 0; k < r_num; k++) {
        const int lo = r_trans[2 * k] - 1, up = r_trans[2 * k + 1] - 1;
        if (lo < 0 || lo >= nlev || up < 0 || up >= nlev) return PORTAL_ERR_ARG;
    }
    std::vector<double> xth;
    const int ndir = legendre_all(nth, nph, xth);
    if (ndir > RS_MAX_DIRS) return PORTAL_ERR_ARG;
    const int nch = 2 * nvel + 1;
    {
        std::lock_guard<std::mutex> lk(g_rs_tables_mutex);
        // line constants
        RsLine *h = g_rs_hlines;
        for (int k = 0; k < r_num; k++) {
            const int lo = r_trans[2 * k] - 1, up = r_trans[2 * k + 1] - 1;
            h[k].nu = nu[k]; h[k].A = t_Aji[k]; h[k].B = t_Bij[k]; h[k].kd = kd_v[k];
            h[k].glo = 2.0 * j_lev[lo] + 1.0; h[k].gup = 2.0 * j_lev[up] + 1.0;
            h[k].bb_cmb = 1.4744995e-50 * std::pow(nu[k], 3.0) * std::pow(std::exp(4.79924e-11 / 2.73 * nu[k]) - 1.0, -1.0);
            h[k].lo = lo; h[k].up = up;
        }
        // direction and channel tables, copied into the static device array
        double *dt = g_rs_hdirs;
        for (int k = 0; k < ndir; k++) {
            const double mu = xth[3 * k], ph = xth[3 * k + 1], w = xth[3 * k + 2];
            const double th = std::acos(mu);
            dt[6 * k] = std::cos(th); dt[6 * k + 1] = std::sin(th);
            dt[6 * k + 2] = std::cos(ph); dt[6 * k + 3] = std::sin(ph);
            dt[6 * k + 4] = w; dt[6 * k + 5] = w * (3.0 * mu * mu - 1.0) / 2.0 / std::sqrt(2.0);
        }
        float *ct = g_rs_hch;
        for (int i = 0; i < 2 * RS_MAX_CH; i++) ct[i] = 0.f;
        const double spi = std::sqrt(std::acos(-1.0));
        for (int i = 0; i < nch; i++) {
            const double q0 = 2.0 * (i - nvel) / nvel;
            ct[i] = (float)q0;
            ct[RS_MAX_CH + i] = (float)(std::exp(-q0 * q0) * 2.0 / (spi * nvel));
        }
        if (cudaMemcpyToSymbolAsync(c_rs_lines, h, sizeof(RsLine) * r_num, 0, cudaMemcpyHostToDevice, st) !=
                cudaSuccess ||
            cudaMemcpyAsync(scratch + RS_OFF_DIRS, dt, 6 * sizeof(double) * (size_t)ndir, cudaMemcpyHostToDevice,
                            st) != cudaSuccess ||
            cudaMemcpyAsync(scratch + RS_OFF_CH, ct, 2 * RS_MAX_CH * sizeof(float), cudaMemcpyHostToDevice, st) !=
                cudaSuccess)
            return PORTAL_ERR_CUDA;
    }
    if (cudaMemsetAsync(scratch, 0, 256, st) != cudaSuccess)   // the node counter starts at zero
        return PORTAL_ERR_CUDA;
    // the rows of the non-bulk nodes, which the kernel does not visit, are
    // zero as in portal_radiation_field
    if (bulk_node_num < node_num) {
        const size_t rest = (size_t)(node_num - bulk_node_num);
        if (cudaMemsetAsync(J0 + (size_t)r_num * bulk_node_num, 0, rest * r_num * sizeof(double), st) !=
                cudaSuccess ||
            cudaMemsetAsync(J2 + (size_t)r_num * bulk_node_num, 0, rest * r_num * sizeof(double), st) !=
                cudaSuccess ||
            (status && cudaMemsetAsync(status + bulk_node_num, 0, rest * sizeof(int), st) != cudaSuccess))
            return PORTAL_ERR_CUDA;
    }
    RsArgs a;
    a.N = node_num; a.bulk = bulk_node_num; a.nlev = nlev; a.L = r_num; a.nvel = nvel; a.nch = nch;
    a.ndir = ndir; a.n_depth = n_depth; a.maxne = maxne; a.dx32 = (float)dx; a.tdx = tx * dx;
    a.gx = gvec[0]; a.gy = gvec[1]; a.gz = gvec[2];
    a.xyz = xyz; a.vel = vel_all; a.b_all = b_all; a.temp_all = temp_all; a.dust_p = dust_p; a.ab = ab_all;
    a.lev_p = lev_p; a.bvec = bvec_all; a.del_ne = del_ne; a.del_num_ne = del_num_ne;
    a.J0 = J0; a.J2 = J2; a.status = status; a.scratch = scratch;
    const dim3 grid(RS_BLOCKS), block(32 * RS_WARPS);
    if (nch <= 32) k_rf_static<1><<<grid, block, 0, st>>>(a);
    else if (nch <= 64) k_rf_static<2><<<grid, block, 0, st>>>(a);
    else if (nch <= 96) k_rf_static<3><<<grid, block, 0, st>>>(a);
    else if (nch <= 160) k_rf_static<5><<<grid, block, 0, st>>>(a);
    else k_rf_static<9><<<grid, block, 0, st>>>(a);
    if (cudaGetLastError() != cudaSuccess) return PORTAL_ERR_CUDA;
    return PORTAL_OK;
}

extern "C" void portal_radiation_field_static_limits(int *max_n_depth, int *max_lines, int *max_channels,
                                                     int *max_directions, long long *scratch_bytes) {
    if (max_n_depth) *max_n_depth = RS_MAX_DEPTH;
    if (max_lines) *max_lines = RS_MAX_LINES;
    if (max_channels) *max_channels = RS_MAX_CH;
    if (max_directions) *max_directions = RS_MAX_DIRS;
    if (scratch_bytes) *scratch_bytes = (long long)RS_BYTES;
}
