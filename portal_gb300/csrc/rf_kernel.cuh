// The radiation-field kernel (the template shared by the single-model calls
// in rf.cu and the batched launch in rf_batch.cu) and the line-table kernel.
// See rf.cu for the algorithm.
#pragma once

#include <type_traits>

#include <cmath>

#include "internal.cuh"

using namespace portal;

namespace {

constexpr float LOG2E_F = 1.4426950408889634f;
// sqrt(log2 e): a profile argument q scaled by it gives exp(-q^2) = 2^(-q'^2),
// one ex2 of q'^2 with the sign folded into the instruction
constexpr float SQL2E_F = 1.2011224087864498f;
// line-centre optical depth (log2 units) below which every channel of a cell
// takes the Taylor form: x = A g <= A with the profile g = ex2(-q'^2) <= 1
// (ex2 of a non-positive argument does not exceed 1: checked over every float
// of [-1/16, 0]), below the switch OM_TAYLOR_X of one_minus_exp with 0.5 % to
// spare
constexpr float OM_THIN_A = 0.0625f;
// Face crossings closer than this (in units of r_max) are not taken.  The
// reference uses 1e-10 (miscellaneous.f90:1048) against FP64 noise ~1e-16;
// the FP32 walk's noise in t is ~1e-9, and a crossing shorter than 2e-8 is
// 0.02 trace steps, i.e. it contributes nint(...) = 0 steps either way.
constexpr float FACE_EPS = 2e-8f;

struct LineConst {
    double nu, A, B, kd, glo, gup, bb_cmb;
    int lo, up;
};
constexpr int MAX_LINES = 64;

// Compensated (Kahan) FP32 sum: J of one node is a sum of a few hundred ray
// contributions; the compensation keeps it to ~1e-7 of the sum of magnitudes
// without the FP64 pipe.  The terms are passed as explicitly rounded products
// (__fmul_rn at the call sites) and summed with explicit roundings: a
// multiply the compiler fuses into the first subtraction in one kernel
// variant and not in another would make the result depend on the line
// grouping of the variant.
struct KahanF {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float y = __fsub_rn(x, c);
        const float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

// Row stride (float2 per cell) of the remainder channel's (cell, line)
// table: odd, so the staging lanes' 64-bit row stores of a half-warp fall in
// distinct banks.
__host__ __device__ __forceinline__ int rem_row_stride(int lines) { return lines | 1; }

// Line groups up to these widths run the cell loop two cells per iteration,
// and instantiate it for every count of Taylor-only lines; wider groups one
// cell per iteration, all or none of the lines Taylor-only (the larger
// bodies cost more in instruction fetch than they gain).
constexpr int UNROLL_MAX_NLG = 4;
constexpr int SUFFIX_MAX_NLG = 3;

// f(std::integral_constant<int, k>) for the run-time count k in [0, NLG] of
// Taylor-only lines: every k for groups up to SUFFIX_MAX_NLG lines, 0 or NLG
// for wider ones, 0 alone with dust
template <int NLG, bool DUST, int K = 0, typename F>
__device__ __forceinline__ void with_thin_lines(int k, F &f) {
    if constexpr (DUST) {
        f(std::integral_constant<int, 0>{});
    } else if constexpr (NLG > SUFFIX_MAX_NLG) {
        if (k == NLG) f(std::integral_constant<int, NLG>{});
        else f(std::integral_constant<int, 0>{});
    } else if constexpr (K < NLG) {
        if (k == K) f(std::integral_constant<int, K>{});
        else with_thin_lines<NLG, DUST, K + 1>(k, f);
    } else {
        f(std::integral_constant<int, NLG>{});
    }
}

__device__ __forceinline__ float ex2(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Line table: one thread per (node, line).
__global__ void k_line_table(int N, int L, double dxp, const LineConst *__restrict__ lines,
                             const double *__restrict__ levp, int nlev, const double *__restrict__ b,
                             const double *__restrict__ dustp, const double *__restrict__ tdust,
                             float4 *__restrict__ ltab) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)N * L) return;
    int n = (int)(t / L), l = (int)(t - (long long)n * L);
    const LineConst lc = lines[l];
    double p1 = levp[(size_t)nlev * n + lc.lo];
    double p2 = levp[(size_t)nlev * n + lc.up];
    // ray_in inverse_rt.f90:263-266, 293-294, 298-301
    double c1 = 2.2102191e-42 * lc.nu;
    double c2 = 5.272859e-35 * lc.nu;
    double cnu = 299792458.0 / lc.nu;
    double kv = c1 * lc.B * (p1 - lc.glo * p2 / lc.gup);
    double ev = c2 * lc.A * p2;
    double phif = cnu / (1.7724538509055160273 * b[n]) * dxp;
    double Ad = lc.kd * dustp[n] * dxp;
    double Td = tdust[n];
    double Ibb = 0.0;
    if (Td != 0.0) {  // black_body miscellaneous.f90:263-285
        double c2b = 4.79924e-11 / Td;
        Ibb = 1.4744995e-50 * lc.nu * lc.nu * lc.nu / (exp(c2b * lc.nu) - 1.0);
    }
    // (optical depth per trace step at unit profile, line source function
    // ev/kv, dust optical depth per step, dust emissivity per step): the
    // source function is stored as the FP64 ratio, not the emissivity, so a
    // weak line's S keeps full FP32 precision where kv and ev alone would be
    // FP32 denormals
    ltab[t] = make_float4((float)(kv * phif), (float)(kv != 0.0 ? ev / kv : 0.0), (float)Ad, (float)(Ad * Ibb));
}

template <int NLG, bool DUST>
struct CellRec {
    float2 qd[32];       // profile argument at channel 0 and its step per channel, times sqrt(log2 e)
    float2 AS[32][NLG];  // (A * steps, S) without dust, (A * steps, E * steps) with dust
    float Ad[32][DUST ? NLG : 1];   // dust tau per cell (dust only)
    float Jd[32][DUST ? NLG : 1];   // dust emissivity * steps (dust only)
};

// Per-warp shared state of the node being processed and its current batch of
// (up to) 32 rays (RayBatch; RayBatchStar in the batched kernel).
struct RayBatch {
    double frame[13];    // b(3), x(3), w(3), node position(3), |p|^2
    float4 dir[32];      // (d_x, d_y, d_z, v_node . d) per ray
    int K[32];           // segments per ray (-1: n_depth overflow)
    float km[6];         // the node's second moment of line 1 (lane 0 accumulates)
};
// The batched kernel's: also the per-node ray sets of star mode.
struct RayBatchStar {
    double frame[13];
    double sk[7];        // star direction k(3), th_star, dth_star, dth_rest, th_i
    int sn[2];           // star rays, all rays of the node (-1: more than nth nph)
    unsigned smask;      // star rays of the batch
    float4 dir[32];
    float2 wts[32];      // (w, w c_in / sqrt 2) per ray
    int K[32];
    float km[6];
};

constexpr double PI_D = 3.141592653589793;  // acos(-1.d0)

// star_all (miscellaneous.f90:1139-1226, circle_points :1228-1265) for ray
// i of a node outside the star: (cos th, ph) of the ray in the field frame
// and its quadrature weight.  sk as in RayBatchStar; f the node frame b (0-2),
// x = b x g / |b x g| (3-5), x x b (6-8).  The first n_star rays cover the
// star's cone (one ray: the reference's x(1:2) = cos(1), i.e. 1 rad off the
// star direction; fewer than ten: a circle at th_star / 2; more: Vogel's
// spiral), the others nth bands of ceiling(nph sin th) rays from th_star to
// pi about the star direction.  Each direction, built about the star
// direction with find_dir (gauge g), is re-expressed by find_angles in the
// field frame (miscellaneous.f90:86-134).
// Returns the direction's (cos th, sin th, cos ph, sin ph) in the field
// frame as inverse_rt rebuilds it (find_dir of acos(mu), ph) and stores the
// weights (w, w c_in / sqrt 2) in *wts.  Out of line: the default path
// keeps the kernel's own code.
// a ray direction in the field frame: (cos th, sin th, cos ph, sin ph)
struct RayDir {
    double ct, st, cp, sp;
};
__device__ __noinline__ RayDir star_ray(const double *sk, int n_star, int i, int nth, int nph, double gx,
                                         double gy, double gz, const double *f, float2 *wts) {
    double x1 = 1.0, x2 = 0.0, w = 0.0;
    if (i < n_star) {
        const double ths = sk[3], dth = sk[4];
        if (n_star == 1) {
            x1 = cos(1.0);
            x2 = cos(1.0);
            w = 2.0 * PI_D * dth;
        } else if (n_star < 10) {
            const double wph = 2.0 * PI_D / n_star;
            x1 = cos(ths / 2.0);
            x2 = i * wph;
            w = wph * dth;
        } else {
            x1 = cos(ths * sqrt(1.0 * (i + 1) / n_star));
            x2 = (i + 1) * (PI_D * (3.0 - sqrt(5.0)));
            w = dth * 2.0 * PI_D / n_star;
        }
        w = w / (4.0 * PI_D);
    } else {
        const double dr = sk[5], thi = sk[6];
        int j = i - n_star, b = 1, np = 1;
        double th = thi;
        for (; b <= nth; b++) {
            th = (b - 1) * dr + thi;
            np = (int)ceil(nph * sin(th));
            if (j < np) break;
            j -= np;
        }
        if (b <= nth) {
            double wth;
            if (b == 1) wth = cos(sk[3]) - cos((b - 0.5) * dr + thi);
            else if (b == nth) wth = cos((b - 1.5) * dr + thi) + 1.0;
            else wth = cos((b - 1.5) * dr + thi) - cos((b - 0.5) * dr + thi);
            const double wph = 2.0 * PI_D / np;
            x1 = cos(th);
            x2 = j * wph;
            w = wth * wph / (4.0 * PI_D);
        }
    }
    // find_dir about k: x_k = k x g / |k x g|, d = cos t k + sin t (cos x2 (x_k x k) + sin x2 x_k)
    const double kx = sk[0], ky = sk[1], kz = sk[2];
    double ux = ky * gz - kz * gy, uy = kz * gx - kx * gz, uz = kx * gy - ky * gx;
    const double un = sqrt(ux * ux + uy * uy + uz * uz);
    ux /= un; uy /= un; uz /= un;
    const double vx = uy * kz - uz * ky, vy = uz * kx - ux * kz, vz = ux * ky - uy * kx;
    const double t = acos(x1), ct = cos(t), st = sin(t), cp = cos(x2), sp = sin(x2);
    const double dx = ct * kx + st * (cp * vx + sp * ux);
    const double dy = ct * ky + st * (cp * vy + sp * uy);
    const double dz = ct * kz + st * (cp * vz + sp * uz);
    // find_angles in the field frame
    const double bd = f[0] * dx + f[1] * dy + f[2] * dz;
    const double thb = (bd > 1.0) ? 0.0 : (bd < -1.0) ? PI_D : acos(bd);
    const double cx = f[1] * dz - f[2] * dy, cy = f[2] * dx - f[0] * dz, cz = f[0] * dy - f[1] * dx;
    const double mub = cos(thb);
    const double phb = atan2(f[3] * dx + f[4] * dy + f[5] * dz, f[3] * cx + f[4] * cy + f[5] * cz);
    *wts = make_float2((float)w, (float)(w * ((3.0 * mub * mub - 1.0) / 2.0) / sqrt(2.0)));
    const double th = acos(mub);
    return RayDir{cos(th), sin(th), cos(phb), sin(phb)};
}

// trace_node's star geometry (main_sub.f90:56-66) and star_all's ray counts
// for the node at p: fills sk and sn of the warp's RayBatchStar.
__device__ __noinline__ void star_node(double *sk, int *sn, double xs, double ys, double zs, double Rs, int nth,
                                       int nph, double px, double py, double pz) {
    const double kx = xs - px, ky = ys - py, kz = zs - pz;
    const double d = sqrt(kx * kx + ky * ky + kz * kz);
    const double q = Rs / d;
    const double dOm = PI_D * (q * q);
    sk[0] = kx / d; sk[1] = ky / d; sk[2] = kz / d;
    const double dth = dOm / (2.0 * PI_D);
    const double ths = acos(1 - dth);
    const double dOm_max = 4.0 * PI_D / (nth * nph);
    const int ns = (int)ceil(dOm / dOm_max);
    const double dr = (PI_D - ths) / nth, thi = ths + dr / 2.0;
    sk[3] = ths; sk[4] = dth; sk[5] = dr; sk[6] = thi;
    int nv = ns;
    for (int b = 1; b <= nth; b++) nv += (int)ceil(nph * sin((b - 1) * dr + thi));
    sn[0] = ns;
    // the reference stops when the rays exceed nth nph (miscellaneous.f90:1203-1206)
    sn[1] = (ns > nth * nph || nv > nth * nph) ? -1 : nv;
}

// check_neigh_fast's star test (miscellaneous.f90:1056-1069) from the node
// at p along d: the star's surface, when the ray meets it first, ends it.
__device__ __noinline__ double star_exit(double sexit, double px, double py, double pz, double dx, double dy,
                                         double dz, double xs, double ys, double zs, double Rs) {
    const double ex = px - xs, ey = py - ys, ez = pz - zs;
    const double qa = dx * dx + dy * dy + dz * dz;
    const double qb = 2.0 * (ex * dx + ey * dy + ez * dz);
    const double qc = (ex * ex + ey * ey + ez * ez) - Rs * Rs;
    const double dis = qb * qb - 4.0 * qa * qc;
    if (dis > 0.0) {
        double r1 = (-qb + sqrt(dis)) / (2.0 * qa);
        const double r2 = (-qb - sqrt(dis)) / (2.0 * qa);
        if (r2 > 0.0) r1 = r2;
        if (r1 > 0.0 && r1 < sexit) return r1;
    }
    return sexit;
}

// NS channel slots per lane, NLG lines per register group.
// RT = 0: nch <= 32 NS, every channel in a slot.  RT = 1: nch = 32 NS + 1
// (the reference's 2 nvel + 1 channels with nvel a multiple of 16): the
// last channel (nv = +nvel) is integrated lanes-over-lines (lane = line,
// L <= 32) in the first line-group pass instead of costing a whole slot of
// 32 lanes for one channel.  Its transfer weights (1 - e^-tau, S) per (cell,
// line) are formed by the staging lanes (lane = cell) into a per-warp table
// of dynamic shared memory, rem_row_stride(L) float2 per cell; the
// lanes-over-lines pass then only runs the recurrence.
// BATCH: the work items are (model, node) pairs of many models (RFBatch);
// each warp copies the argument block of its current model into shared
// memory.  Otherwise the nodes of the one model a0.
template <int NS, int NLG, bool DUST, bool BATCH, int RT>
__global__ void __launch_bounds__(256, (NLG <= 5 && NS <= 5) ? 2 : 1) k_radiation_field(RFArgs a0, RFBatch bw) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const long long gw = (long long)blockIdx.x * (blockDim.x >> 5) + wib;
    const int n_depth = BATCH ? bw.n_depth : a0.n_depth;
    int2 *const wbase = (BATCH ? bw.walk : a0.walk) + (size_t)gw * 32 * (size_t)n_depth;
    __shared__ CellRec<NLG, DUST> recs[8];
    using RB = typename std::conditional<BATCH, RayBatchStar, RayBatch>::type;
    __shared__ RB rbs[8];
    __shared__ RFArgs margs[BATCH ? 8 : 1];
    extern __shared__ float2 rem_dyn[];
    CellRec<NLG, DUST> &R = recs[wib];
    RB &B = rbs[wib];
    const int rem_ld = rem_row_stride(BATCH ? bw.rem_lines : a0.L);
    float2 *const remS = rem_dyn + (size_t)wib * 32 * rem_ld;   // RT: this warp's (cell, line) table

    unsigned long long nseg = 0;
    int cur_model = -1;
    for (;;) {
        int node = 0;
        if (BATCH) {
            long long item = 0;
            if (lane == 0) item = (long long)atomicAdd(&bw.queue[0], 1ULL);
            item = __shfl_sync(FULL, item, 0);
            if (item >= bw.n_items) break;
            const int2 wi = bw.items[item];
            if (wi.x != cur_model) {
                __syncwarp();
                const int *src = reinterpret_cast<const int *>(bw.models + wi.x);
                int *dst = reinterpret_cast<int *>(&margs[wib]);
                for (int k = lane; k < (int)(sizeof(RFArgs) / sizeof(int)); k += 32) dst[k] = src[k];
                __syncwarp();
                cur_model = wi.x;
            }
            node = wi.y;
        } else {
            if (lane == 0) node = (int)atomicAdd(&a0.counters[0], 1ULL);
            node = __shfl_sync(FULL, node, 0);
            if (node >= a0.bulk) break;
        }
        const RFArgs &a = BATCH ? margs[wib] : a0;
        KahanF acc0a, acc0b, acc2a, acc2b;  // lines lane and lane+32, compensated FP32
        KahanF accEa, accEb, accLa, accLb;  // J_eff and L* of the same lines (split field only)
        const bool split = (a.JE != nullptr);
        int st = 0;
        int node_seg = 0;   // the node's ray segments (sum of node_count over its rays)
        if (a.ab[node] > 0.0) {
            if (lane == 0) {
                // node frame (find_dir miscellaneous.f90:48-82): x = b x g / |b x g|,
                // dir = R(b,ph) R(x,th) b = cos th b + sin th (cos ph (x x b) + sin ph x)
                const double bx = a.bvec[3 * (size_t)node], by = a.bvec[3 * (size_t)node + 1],
                             bz = a.bvec[3 * (size_t)node + 2];
                double xx = by * a.gz - bz * a.gy, xy = bz * a.gx - bx * a.gz, xz = bx * a.gy - by * a.gx;
                const double xn = sqrt(xx * xx + xy * xy + xz * xz);
                xx /= xn; xy /= xn; xz /= xn;
                const double px = a.pos[3 * (size_t)node], py = a.pos[3 * (size_t)node + 1],
                             pz = a.pos[3 * (size_t)node + 2];
                double *f = B.frame;
                f[0] = bx; f[1] = by; f[2] = bz; f[3] = xx; f[4] = xy; f[5] = xz;
                f[6] = xy * bz - xz * by; f[7] = xz * bx - xx * bz; f[8] = xx * by - xy * bx;
                f[9] = px; f[10] = py; f[11] = pz; f[12] = px * px + py * py + pz * pz;
                for (int k = 0; k < 6; k++) B.km[k] = 0.f;
                if constexpr (BATCH) {
                    if (a.star) {
                        star_node(B.sk, B.sn, a.xs, a.ys, a.zs, a.Rs, a.nth, a.nph, px, py, pz);
                    } else {
                        B.sn[0] = 0;
                        B.sn[1] = a.ndir;
                    }
                }
            }
            __syncwarp();
            // star mode runs in the batched kernel only: its node's ray count lives in
            // shared memory (read where used, holding no register through the
            // integration); the single-model kernel uses the common direction table
            const volatile int *vsn = nullptr;
            if constexpr (BATCH) {
                vsn = B.sn;
                if (vsn[1] < 0) st |= PORTAL_NODE_STAR;
            }
            auto n_rays = [&]() -> int {
                if constexpr (BATCH) return vsn[1];
                else return a.ndir;
            };
            const float4 cvn = a.cellv[node];
            const float dqfac = 2.f * cvn.w / (float)a.nvel;

            for (int k0 = 0; st == 0 && k0 < n_rays(); k0 += 32) {
                const int nr = min(32, n_rays() - k0);
                // ---- (1)+(2) set-up and walk, one lane per ray ----
                int K = 0;
                bool over = false;
                bool sray = false;
                unsigned smask = 0u;
                if constexpr (BATCH) {
                    sray = a.star && lane < nr && k0 + lane < vsn[0];
                    smask = __ballot_sync(FULL, sray);
                }
                if (lane < nr) {
                    const double *f = B.frame;
                    double mu, sth, cph, sph;
                    bool tab = true;
                    if constexpr (BATCH) {
                        if (a.star) {
                            const RayDir r = star_ray(B.sk, vsn[0], k0 + lane, a.nth, a.nph, a.gx, a.gy, a.gz, f,
                                                      &B.wts[lane]);
                            mu = r.ct; sth = r.st; cph = r.cp; sph = r.sp;
                            tab = false;
                        }
                    }
                    if (tab) {
                        const double *dr = a.dirs + 6 * (size_t)(k0 + lane);
                        mu = dr[0]; sth = dr[1]; cph = dr[2]; sph = dr[3];
                        if constexpr (BATCH) B.wts[lane] = make_float2((float)dr[4], (float)dr[5]);
                    }
                    const double dx = mu * f[0] + sth * (cph * f[6] + sph * f[3]);
                    const double dy = mu * f[1] + sth * (cph * f[7] + sph * f[4]);
                    const double dz = mu * f[2] + sth * (cph * f[8] + sph * f[5]);
                    double sexit = sphere_exit(f[9], f[10], f[11], dx, dy, dz);
                    if constexpr (BATCH) {
                        if (sray) sexit = star_exit(sexit, f[9], f[10], f[11], dx, dy, dz, a.xs, a.ys, a.zs, a.Rs);
                    }
                    const float fdx = (float)dx, fdy = (float)dy, fdz = (float)dz;
                    B.dir[lane] = make_float4(fdx, fdy, fdz, cvn.x * fdx + cvn.y * fdy + cvn.z * fdz);
                    int2 *wl = wbase + (size_t)lane * n_depth;
                    // distance left to the sphere exit as an unevaluated float pair
                    // (rh + rl), decremented exactly by each step
                    float rh = (float)sexit, rl = (float)(sexit - (double)rh);
                    float rx = 0.f, ry = 0.f, rz = 0.f;
                    int c = node;
                    for (;;) {
                        const float tsph = rh + rl;
                        const int o = a.off[c], deg = a.off[c + 1] - o;
                        // check_neigh_fast's scan: best starts at the sphere exit, a
                        // neighbour replaces it when FACE_EPS < t <= best (so among equal
                        // t the later neighbour wins).  t = num/den compared by cross
                        // multiplication (den > 0).
                        float bnum = tsph, bden = 1.f;
                        int bj = -1;
                        for (int j = 0; j < deg; j++) {
                            const float4 e = a.edge[o + j];
                            const float den = e.x * fdx + e.y * fdy + e.z * fdz;
                            const float num = e.w - (e.x * rx + e.y * ry + e.z * rz);
                            if (den > 0.f && num > FACE_EPS * den && num * bden <= bnum * den) {
                                bnum = num;
                                bden = den;
                                bj = j;
                            }
                        }
                        const float delta = (bj < 0) ? tsph : bnum / bden;
                        if (K >= n_depth) { over = true; break; }
                        wl[K] = make_int2(c, (int)roundf(delta / a.dx32));  // nint(delta_x/dx)
                        K++;
                        if (bj < 0) break;
                        const float4 e = a.edge[o + bj];
                        {   // (rh, rl) -= delta: two-sum, then renormalise
                            const float t = rh - delta;
                            const float bv = t - rh;
                            const float err = (rh - (t - bv)) - (delta + bv);
                            const float lo = rl + err;
                            rh = t + lo;
                            rl = lo - (rh - t);
                        }
                        rx = fmaf(delta, fdx, rx) - e.x;
                        ry = fmaf(delta, fdy, ry) - e.y;
                        rz = fmaf(delta, fdz, rz) - e.z;
                        c = a.idx[o + bj];
                    }
                }
                B.K[lane] = over ? -1 : K;
                if constexpr (BATCH) {
                    if (lane == 0) B.smask = smask;
                }
                if (__any_sync(FULL, over)) { st |= PORTAL_NODE_DEPTH; break; }
                __syncwarp();

                // ---- (3)+(4) channel integration of each ray of the batch ----
                for (int rr = 0; rr < nr; rr++) {
                    const int Kr = B.K[rr];
                    const int2 *wl = wbase + (size_t)rr * n_depth;
                    const float4 d4 = B.dir[rr];
                    float wgt, wgt2;
                    if constexpr (BATCH) {
                        const float2 wt = B.wts[rr];
                        wgt = wt.x;
                        wgt2 = wt.y;
                    } else {
                        const double *dr = a.dirs + 6 * (size_t)(k0 + rr);
                        wgt = (float)dr[4];
                        wgt2 = (float)dr[5];
                    }
                    // the incoming intensity: B(T_star) for a star ray (inverse_rt.f90:113-118),
                    // the ray's flag read from shared memory where it is used
                    auto bb_in = [&](int l) -> float {
                        if constexpr (BATCH) {
                            const volatile unsigned *vsm = &B.smask;
                            return ((*vsm >> rr) & 1u) ? a.bbs[l] : a.bb[l];
                        } else {
                            return a.bb[l];
                        }
                    };
                    node_seg += Kr;
                    const int2 w0 = wl[0];
                    // the remainder channel of this lane's line (RT): intensity, and
                    // its central-cell contributions to J0 (and J_eff, L*)
                    float Irem = 0.f, remJ = 0.f, remE = 0.f, remL = 0.f;
                    if (RT && lane < a.L) Irem = bb_in(lane);
                    for (int l0 = 0; l0 < a.L; l0 += NLG) {
                        // intensities of the lane's channels: slot pairs (s, s+1) in one
                        // float2 (packed FP32x2 arithmetic), an odd last slot in .x
                        float2 I2[(NS + 1) / 2][NLG];
#define IV(s, l) (((s) & 1) ? I2[(s) >> 1][l].y : I2[(s) >> 1][l].x)
#pragma unroll
                        for (int l = 0; l < NLG; l++) {
                            const float bb = (l0 + l < a.L) ? bb_in(l0 + l) : 0.f;
#pragma unroll
                            for (int s2 = 0; s2 < NS; s2++) IV(s2, l) = bb;
                        }
                        // walk records of the chunk (lane = cell), the next chunk's
                        // loaded while this one is integrated
                        int2 wcp = make_int2(0, 0);
                        if (lane < min(32, Kr - 1)) wcp = wl[Kr - 1 - lane];
                        for (int hi = Kr - 1; hi >= 1; hi -= 32) {
                            const int nc = min(32, hi);
                            const int2 wc = wcp;
                            if (lane < min(32, hi - 32)) wcp = wl[hi - 32 - lane];
                            __syncwarp();
                            unsigned thin_m = (1u << NLG) - 1u;   // the group's lines thin in this cell
                            if (lane < nc) {
                                const float4 cv = a.cellv[wc.x];
                                const float vp = fmaf(cv.z, d4.z, fmaf(cv.y, d4.y, __fmul_rn(cv.x, d4.x)));
                                const float ib = SQL2E_F * (1.f / cv.w);
                                const float2 qdl = make_float2((d4.w - vp) * ib, dqfac * ib);
                                R.qd[lane] = qdl;
                                const float fst = (float)wc.y;
                                if (RT && l0 == 0) {
                                    // the remainder channel's transfer weight and source
                                    // function of this cell for every line
                                    const float q = fmaf(qdl.y, (float)(32 * NS - a.nvel), qdl.x);
                                    const float gr = ex2(-(q * q));
                                    const float2 *lr = reinterpret_cast<const float2 *>(a.ltab + (size_t)wc.x * a.L);
                                    float2 *dst = remS + lane * rem_ld;
#pragma unroll 4
                                    for (int l = 0; l < a.L; l++) {
                                        const float2 v = lr[2 * l];
                                        const float As = (v.x > 0.f) ? v.x * fst * LOG2E_F : 0.f;
                                        const float Ss = (v.x > 0.f) ? v.y : 0.f;
                                        const float x = As * gr;
                                        dst[l] = make_float2(one_minus_exp(x, ex2(-x)), Ss);
                                    }
                                }
                                const float4 *lt = a.ltab + (size_t)wc.x * a.L + l0;
#pragma unroll
                                for (int l = 0; l < NLG; l++) {
                                    if (DUST) {
                                        if (l0 + l < a.L) {
                                            const float4 v = lt[l];
                                            R.AS[lane][l] = make_float2(v.x * fst, v.y * v.x * fst);   // emissivity x steps
                                            R.Ad[lane][DUST ? l : 0] = v.z * fst;
                                            R.Jd[lane][DUST ? l : 0] = v.w * fst;
                                        }
                                    } else {
                                        // optical depth at unit profile in log2 units (ex2
                                        // takes it as is) and the source function.  A cell
                                        // line with kv <= 0 fails ray_in's gate tau > 1e-30
                                        // in every channel (inverse_rt.f90:308), and so does
                                        // a padding line of the last group: both get A = S
                                        // = 0, which leaves I unchanged exactly.
                                        float As = 0.f, Ss = 0.f;
                                        if (l0 + l < a.L) {
                                            const float4 v = lt[l];
                                            if (v.x > 0.f) {
                                                As = v.x * fst * LOG2E_F;
                                                Ss = v.y;
                                            }
                                        }
                                        R.AS[lane][l] = make_float2(As, Ss);
                                        if (!(As < OM_THIN_A)) thin_m &= ~(1u << l);
                                    }
                                }
                            }
                            // A line whose line-centre optical depth is below OM_THIN_A
                            // in every cell of the chunk takes the Taylor form of
                            // 1 - e^-tau in every channel: the branch-free update would
                            // select exactly that value, so it skips the ex2 and the
                            // select.  Decided per chunk of 32 cells, uniform over the
                            // warp, for the group's last tk lines (a rotor's higher lines
                            // are the thinner ones); the cell loop is instantiated per tk
                            // (groups of at most 5 lines; wider groups: none or all).
                            int tk = 0;
                            if (!DUST) {
                                const unsigned tm = __reduce_and_sync(FULL, thin_m);
                                tk = __clz(~(tm << (32 - NLG)));   // trailing run of thin lines
                                if (NLG > SUFFIX_MAX_NLG && tk != NLG) tk = 0;
                            }
                            __syncwarp();
                            if (RT && l0 == 0 && lane < a.L) {
                                // the remainder channel, lane = line, the same cells inward
                                for (int u = 0; u < nc; u++) {
                                    const float2 r = remS[u * rem_ld + lane];
                                    Irem = fmaf(r.x, r.y - Irem, Irem);
                                }
                            }
                            // one cell's update of the group's lines in every channel slot
                            auto cell_step = [&](auto tk_tag, int u) {
                                constexpr int TK = decltype(tk_tag)::value;   // the last TK lines: Taylor only
                                const float2 qd = R.qd[u];
                                const float q0 = qd.x, dq = qd.y;
                                // Gaussian profile of the cell at the lane's channels,
                                // exp(-q^2) = 2^(-q'^2) with q' = q sqrt(log2 e) (staged
                                // scaled); slot pairs on the packed pipe (the same
                                // roundings per slot as the odd slot's scalar form)
                                float g[NS];
#pragma unroll
                                for (int s2 = 0; s2 + 1 < NS; s2 += 2) {
                                    const float2 ch2 = make_float2((float)(lane + 32 * s2 - a.nvel),
                                                                   (float)(lane + 32 * (s2 + 1) - a.nvel));
                                    const float2 q = __ffma2_rn(make_float2(dq, dq), ch2, make_float2(q0, q0));
                                    const float2 t = __fmul2_rn(q, q);
                                    g[s2] = ex2(-t.x);
                                    g[s2 + 1] = ex2(-t.y);
                                }
                                if (NS & 1) {
                                    const float q = fmaf(dq, (float)(lane + 32 * (NS - 1) - a.nvel), q0);
                                    g[NS - 1] = ex2(-(q * q));
                                }
#pragma unroll
                                for (int l = 0; l < NLG; l++) {
                                    const float2 ASu = R.AS[u][l];
                                    const float Au = ASu.x;
                                    const float Su = ASu.y;
                                    if (DUST) {
                                        if (l0 + l < a.L) {
                                            const float Adu = R.Ad[u][DUST ? l : 0], Jdu = R.Jd[u][DUST ? l : 0];
#pragma unroll
                                            for (int s2 = 0; s2 < NS; s2++) {
                                                // tau = (kv phi + alpha) dx n, S = (ev phi + j)/(kv phi + alpha)
                                                const float tau = fmaf(Au, g[s2], Adu);
                                                const float Sv = fmaf(Su, g[s2], Jdu) / tau;
                                                const float x = tau * LOG2E_F;
                                                const float om = one_minus_exp(x, ex2(-x));
                                                const float In = fmaf(om, Sv - IV(s2, l), IV(s2, l));
                                                IV(s2, l) = (tau > 1e-30f) ? In : IV(s2, l);
                                            }
                                        }
                                    } else {
                                        // I' = I + (1 - e^-tau)(S - I) with 1 - e^-tau accurate
                                        // down to tau = 0 and rounded as the reference's FP64
                                        // (one_minus_exp).  ray_in's gate tau > 1e-30
                                        // (inverse_rt.f90:308) needs no test: lines with kv <= 0
                                        // carry A = S = 0 and leave I unchanged exactly, and
                                        // 0 < tau < 2^-54 rounds to a zero weight as in FP64.
                                        // Branch-free inside a cell, so the NS x NLG update
                                        // chains interleave: a warp-uniform branch per cell to
                                        // a Taylor-only path measured 24 % slower in spite of
                                        // skipping the ex2 (1.45e9 against 1.90e9 segments/s);
                                        // decided once per chunk of 32 cells (TK) it gains
                                        // (1.96e9 -> 2.03e9).  Channel-slot pairs go through
                                        // the packed FP32x2 pipe (one issue slot for two
                                        // updates).
                                        const float2 A2 = make_float2(Au, Au), S2 = make_float2(Su, Su);
#pragma unroll
                                        for (int s2 = 0; s2 + 1 < NS; s2 += 2) {
                                            const float2 x = __fmul2_rn(A2, make_float2(g[s2], g[s2 + 1]));
                                            const float2 om = (l >= NLG - TK) ? om_taylor2(x)
                                                                              : one_minus_exp2(x, ex2(-x.x), ex2(-x.y));
                                            float2 &Ip = I2[s2 >> 1][l];
                                            Ip = __ffma2_rn(om, __ffma2_rn(Ip, make_float2(-1.f, -1.f), S2), Ip);
                                        }
                                        if (NS & 1) {
                                            const float x = Au * g[NS - 1];
                                            const float om = (l >= NLG - TK) ? om_taylor(x) : one_minus_exp(x, ex2(-x));
                                            float &Is = I2[NS >> 1][l].x;
                                            Is = fmaf(om, Su - Is, Is);
                                        }
                                    }
                                }
                            };
                            // two cells per iteration: the second cell's profile and
                            // transfer weights do not depend on the first's update and
                            // fill its dependency stalls (2.10e9 -> 2.22e9 segments/s on
                            // the benchmark sphere with the walk-record prefetch above;
                            // 4 cells per iteration: 2.21e9)
                            auto run = [&](auto tk_tag) {
                                if constexpr (NLG <= UNROLL_MAX_NLG) {
#pragma unroll 2
                                    for (int u = 0; u < nc; u++) cell_step(tk_tag, u);
                                } else {
#pragma unroll 1
                                    for (int u = 0; u < nc; u++) cell_step(tk_tag, u);
                                }
                            };
                            with_thin_lines<NLG, DUST>(tk, run);
                        }
                        // central cell (inverse_rt.f90:320-339): no gate, profile at
                        // the node's own b, then the weighted channel sum
                        const float fst0 = (float)w0.y;
                        if (RT && l0 == 0 && lane < a.L) {
                            const int ch = 32 * NS;
                            const float4 v = a.ltab[(size_t)node * a.L + lane];
                            const float q0c = a.chq[ch];
                            const float g0 = ex2(-q0c * q0c * LOG2E_F);
                            const float x = v.x * g0 * fst0 * LOG2E_F;
                            const float om = one_minus_exp(x, ex2(-x));
                            remJ = __fmul_rn(a.chw[ch], fmaf(om, v.y - Irem, Irem));
                            if (split) {
                                remE = __fmul_rn(a.chw[ch], fmaf(om, -Irem, Irem));
                                remL = __fmul_rn(a.chw[ch], om);
                            }
                        }
                        float part[NLG], pe[NLG], pl[NLG];
#pragma unroll
                        for (int l = 0; l < NLG; l++) {
                            part[l] = 0.f;
                            pe[l] = 0.f;
                            pl[l] = 0.f;
                            if (l0 + l < a.L) {
                                const float4 v = a.ltab[(size_t)node * a.L + l0 + l];
#pragma unroll
                                for (int s2 = 0; s2 < NS; s2++) {
                                    const int ch = lane + 32 * s2;
                                    if (ch < a.nch) {
                                        const float q0c = a.chq[ch];
                                        const float g0 = ex2(-q0c * q0c * LOG2E_F);
                                        float tau, Sv, lf = 1.f, Sd = 0.f;
                                        if (DUST) {
                                            const float kap = fmaf(v.x, g0, v.z);
                                            tau = kap * fst0;
                                            Sv = fmaf(v.y * v.x, g0, v.w) / kap;
                                            lf = v.x * g0 / kap;   // line share of the opacity
                                            Sd = v.w / kap;        // dust emission share of S
                                        } else {
                                            tau = v.x * g0 * fst0;
                                            Sv = v.y;
                                        }
                                        const float x = tau * LOG2E_F;
                                        const float e = ex2(-x);
                                        const float om = one_minus_exp(x, e);
                                        const float Io = fmaf(om, Sv - IV(s2, l), IV(s2, l));
                                        part[l] = fmaf(a.chw[ch], Io, part[l]);
                                        if (split) {
                                            pe[l] = fmaf(a.chw[ch], fmaf(om, Sd - IV(s2, l), IV(s2, l)), pe[l]);
                                            pl[l] = fmaf(a.chw[ch], lf * om, pl[l]);
                                        }
                                    }
                                }
                            }
                        }
#pragma unroll
                        for (int l = 0; l < NLG; l++) {
                            float v = part[l];
#pragma unroll
                            for (int o2 = 16; o2 >= 1; o2 >>= 1) v += __shfl_xor_sync(FULL, v, o2);
                            const int line = l0 + l;
                            if (line < a.L && (line & 31) == lane) {
                                if (line < 32) {
                                    if (RT) v = __fadd_rn(v, remJ);   // this lane's line: its remainder channel
                                    acc0a.add(__fmul_rn(wgt, v));
                                    acc2a.add(__fmul_rn(wgt2, v));
                                    if (line == 0) {
                                        // the full second moment of line 1's field, sum w I n n,
                                        // whose traceless part is J^2_Q in any frame
                                        const float wv = __fmul_rn(wgt, v);
                                        B.km[0] = fmaf(wv * d4.x, d4.x, B.km[0]);
                                        B.km[1] = fmaf(wv * d4.y, d4.y, B.km[1]);
                                        B.km[2] = fmaf(wv * d4.z, d4.z, B.km[2]);
                                        B.km[3] = fmaf(wv * d4.x, d4.y, B.km[3]);
                                        B.km[4] = fmaf(wv * d4.x, d4.z, B.km[4]);
                                        B.km[5] = fmaf(wv * d4.y, d4.z, B.km[5]);
                                    }
                                } else {
                                    acc0b.add(__fmul_rn(wgt, v));
                                    acc2b.add(__fmul_rn(wgt2, v));
                                }
                            }
                        }
                        if (split) {
#pragma unroll
                            for (int l = 0; l < NLG; l++) {
                                float ve = pe[l], vl = pl[l];
#pragma unroll
                                for (int o2 = 16; o2 >= 1; o2 >>= 1) {
                                    ve += __shfl_xor_sync(FULL, ve, o2);
                                    vl += __shfl_xor_sync(FULL, vl, o2);
                                }
                                const int line = l0 + l;
                                if (line < a.L && (line & 31) == lane) {
                                    if (line < 32) {
                                        if (RT) {
                                            ve = __fadd_rn(ve, remE);
                                            vl = __fadd_rn(vl, remL);
                                        }
                                        accEa.add(__fmul_rn(wgt, ve));
                                        accLa.add(__fmul_rn(wgt, vl));
                                    } else {
                                        accEb.add(__fmul_rn(wgt, ve));
                                        accLb.add(__fmul_rn(wgt, vl));
                                    }
                                }
                            }
                        }
                    }
                }
                __syncwarp();
            }
        }
#undef IV
        if (lane < a.L) {
            a.J0[(size_t)node * a.L + lane] = (st == 0) ? acc0a.value() : 0.0;
            a.J2[(size_t)node * a.L + lane] = (st == 0) ? acc2a.value() : 0.0;
        }
        if (lane + 32 < a.L) {
            a.J0[(size_t)node * a.L + lane + 32] = (st == 0) ? acc0b.value() : 0.0;
            a.J2[(size_t)node * a.L + lane + 32] = (st == 0) ? acc2b.value() : 0.0;
        }
        if (split) {
            if (lane < a.L) {
                a.JE[(size_t)node * a.L + lane] = (st == 0) ? accEa.value() : 0.0;
                a.LS[(size_t)node * a.L + lane] = (st == 0) ? accLa.value() : 0.0;
            }
            if (lane + 32 < a.L) {
                a.JE[(size_t)node * a.L + lane + 32] = (st == 0) ? accEb.value() : 0.0;
                a.LS[(size_t)node * a.L + lane + 32] = (st == 0) ? accLb.value() : 0.0;
            }
        }
        if (lane == 0) {
            a.status[node] = st;
            if (a.segs) a.segs[node] = node_seg;
            if (a.kmom)
                for (int k = 0; k < 6; k++)
                    a.kmom[(size_t)k * a.N + node] = (st == 0 && a.ab[node] > 0.0) ? B.km[k] : 0.f;
        }
        nseg += (unsigned long long)node_seg;
        __syncwarp();
    }
    // segment count (every lane holds the same count)
    if (lane == 0) atomicAdd(BATCH ? &bw.queue[1] : &a0.counters[1], nseg);
}

}  // namespace

namespace {

// Channel layout: (slots per lane, remainder channel).  2 nvel + 1 channels
// with nvel a multiple of 16 take 2 nvel / 32 full slots plus the
// lanes-over-lines remainder channel (no dust, at most 32 lines); any other
// count is padded to whole slots.
struct ChanLayout {
    int ns, rt;
};
inline ChanLayout chan_layout(int nch, bool dust, int max_lines) {
    if (!dust && max_lines <= 32 && nch > 32 && nch % 32 == 1) {
        const int k = nch / 32;
        if (k == 1 || k == 2 || k == 4 || k == 8) return {k, 1};
    }
    if (nch <= 32) return {1, 0};
    if (nch <= 64) return {2, 0};
    if (nch <= 96) return {3, 0};
    if (nch <= 160) return {5, 0};
    return {9, 0};
}

}  // namespace
