// Stokes image of one inclination: the pixel mode of finish_portal.x.
//
// Reference: para_finish.f90:170-185 (line data), :222-240 (population
// read-back), :354-448 (pixel grid and the three OpenMP loops);
// rotate_all_save miscellaneous.f90:844-907; comp_emcoefs em_coefs.f90:1-113;
// trace_out_raytrace raytrace.f90:58-177 with check_neigh
// miscellaneous.f90:1-46; ray_in_raytrace raytrace.f90:179-323 with
// polarize_prop :1-56 and rot_stokes / rot_stokes_back
// miscellaneous.f90:463-551.
//
// Kernels:
//   k_im_nodes   per node: the inclination rotation (FP64) and the
//                population read-back, then per (node, line) the emission /
//                absorption coefficients, stored as per-trace-step factors at
//                the profile peak (float4), plus per-node Stokes-rotation
//                constants.
//   k_image      one warp per 32 pixels (persistent):
//                 (1) one lane per pixel: the start node (argmin of the FP64
//                     distance, lowest index on ties) and the fixed-step
//                     march along +z.  The step at which a neighbour becomes
//                     nearer is predicted from the bisector-plane crossing,
//                     the photon's z is advanced by the reference's own
//                     sequence of FP64 additions (computed in exact jumps,
//                     add_steps), and check_neigh is replayed exactly (FP64,
//                     strict <, list order) around each predicted change and
//                     at the exit -- over the neighbours that can come within
//                     1e-12 of the current node's squared distance before the
//                     next predicted change, the others being unable to win
//                     -- so the recorded (node, step) list is the reference's;
//                 (2) per pixel, lanes over velocity channels, lines looped:
//                     the polarized propagation in the numerically stable
//                     form o11 = (phi(p)+phi(m))/2, o12 = -(phi(p)-phi(m))/2,
//                     e ch = (E_p+E_m)/2, e sh = (E_p-E_m)/2 with p, m =
//                     tau_I -/+ tau_Q, E = exp(-.), phi(x) = (1-e^-x)/x,
//                     algebraically identical to raytrace.f90:41-53; the
//                     optical depth summed with compensation; the
//                     channel-independent dust terms once per pixel.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"

namespace portal {
double wigner6j(int tj1, int tj2, int tj3, int tj4, int tj5, int tj6);
}
using namespace portal;

namespace {

struct ImLine {
    double nu0, A, kd, w1, w2, fas, bb_cmb, bb_star;
    int lo, up, j1, j2;  // 0-based levels
};
constexpr int IM_MAX_LINES = 16;
__constant__ ImLine c_im[IM_MAX_LINES];

struct ImNodeArgs {
    int N, bulk, nlev, nlines;
    double R[9];              // R_tot column-major
    double tdx;               // tx * dx
    const double *xyz, *vel, *bvec, *b, *tdust, *levp, *pops_in;
    const int *j_lev;
    double *xyz_r;            // (3,N) rotated positions
    double *nrm2;             // (N) |X|^2 of the rotated positions (the march's predictions)
    float4 *cellv;            // (vz, 1/b, cos 2alpha, sin 2alpha)
    float4 *cellb;            // (mu2, cos 2phi, sin 2phi, dust rho)
    float4 *coef;             // (nlines, N): eta_I, eta_Q, eps_I, eps_Q per step / (b sqrt(pi)) / peak
};

__global__ void k_im_nodes(ImNodeArgs a) {
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= a.N) return;
    // rotate_all_save: x' = R_tot x for positions, velocities, field
    double x[3], v[3], bb[3];
    for (int j = 0; j < 3; j++) {
        double sx = 0.0, sv = 0.0, sb = 0.0;
        for (int k = 0; k < 3; k++) {
            // uncontracted, as the reference's sums (the per-node mode starts
            // its rays at these positions)
            sv = __dadd_rn(sv, __dmul_rn(a.R[j + 3 * k], a.vel[3 * (size_t)n + k]));
            sb = __dadd_rn(sb, __dmul_rn(a.R[j + 3 * k], a.bvec[3 * (size_t)n + k]));
            sx = __dadd_rn(sx, __dmul_rn(a.R[j + 3 * k], a.xyz[3 * (size_t)n + k]));
        }
        x[j] = sx; v[j] = sv; bb[j] = sb;
    }
    for (int j = 0; j < 3; j++) a.xyz_r[3 * (size_t)n + j] = x[j];
    a.nrm2[n] = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
    // rot_stokes: alpha = acos(chi_y), negative when chi_x > 0
    const double cn = sqrt(bb[0] * bb[0] + bb[1] * bb[1]);
    const double chx = bb[0] / cn, chy = bb[1] / cn;
    double al = acos(chy);
    if (chx > 0.0) al = -al;
    // dust angle raytrace.f90:281-285: phi = acos(b_y/|b_xy|), negative when b_x < 0
    double ph = acos(bb[1] / sqrt(bb[0] * bb[0] + bb[1] * bb[1]));
    if (bb[0] < 0.0) ph = -ph;
    a.cellv[n] = make_float4((float)v[2], (float)(1.0 / a.b[n]), (float)cos(2.0 * al), (float)sin(2.0 * al));
    a.cellb[n] = make_float4((float)(1.0 - bb[2] * bb[2]), (float)cos(2.0 * ph), (float)sin(2.0 * ph), 0.f);
    // population read-back para_finish.f90:226-239 and comp_emcoefs for the
    // bulk nodes with a non-zero first population (:418)
    const int N = a.N, nlev = a.nlev;
    auto lp = [&](int l) { return a.levp[(size_t)nlev * n + l]; };
    auto sg = [&](int l) { return sqrt(2.0 * a.j_lev[l] + 1.0); };
    auto pp0 = [&](int l) {  // rho^0_0 of level l after read-back
        return lp(l) / sg(l);
    };
    auto pp2 = [&](int l) {  // rho^2_0 after read-back
        const double r0 = a.pops_in[(size_t)n + (size_t)N * (2 * l)];
        const double r2 = a.pops_in[(size_t)n + (size_t)N * (2 * l + 1)];
        if (l == 0) return r2;  // level 1's alignment keeps the value read
        return (r2 / r0) * lp(l) / sg(l);
    };
    const double th = acos(bb[2]);
    const double ct = cos(th), st = sin(th);
    const double tki = (3.0 * ct * ct - 1.0) / (2.0 * sqrt(2.0));
    const double tkq = -3.0 * st * st / (2.0 * sqrt(2.0));
    const double spi_b = 1.7724538509055160273 * a.b[n];
    for (int j = 0; j < a.nlines; j++) {
        float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
        if (n < a.bulk && pp0(0) != 0.0) {
            const ImLine L = c_im[j];
            const double r1_0 = pp0(L.lo), r2_0 = pp0(L.up);
            const double r1_2 = pp2(L.lo), r2_2 = pp2(L.up);
            const double g1 = 2.0 * L.j1 + 1.0, g2 = 2.0 * L.j2 + 1.0;
            const double wjj2_1 = L.fas * sqrt(3.0 * g1) * L.w1;
            const double wjj2_2 = L.fas * sqrt(3.0 * g2) * L.w2;
            const double na_I = 1.0 + wjj2_1 * (r1_2 / r1_0) * tki;
            const double na_Q = wjj2_1 * (r1_2 / r1_0) * tkq;
            const double ns_I = 1.0 + wjj2_2 * (r2_2 / r2_0) * tki;
            const double ns_Q = wjj2_2 * (r2_2 / r2_0) * tkq;
            const double b_to_a = L.nu0 * L.nu0 * L.nu0 / 6.781962e49;
            const double Bji = L.A / b_to_a;
            const double hv = 5.273e-35 * L.nu0;
            const double eI = hv * L.A * ns_I * sqrt(g2) * r2_0;
            const double eQ = hv * L.A * ns_Q * sqrt(g2) * r2_0;
            const double nI = hv * (g2 / g1) * Bji * (sqrt(g1) * r1_0 * na_I - sqrt(g2) * r2_0 * ns_I * g1 / g2);
            const double nQ = hv * (g2 / g1) * Bji * (sqrt(g1) * r1_0 * na_Q - sqrt(g2) * r2_0 * ns_Q * g1 / g2);
            // eta = cnu * v_corr * pol, v_corr = exp(-(dv/b)^2)/(b sqrt(pi)); per
            // trace step: * tx dx (raytrace.f90:221, 239, 250-258)
            const double cnu = (double)2.99792e8f / L.nu0;
            const double f = cnu / spi_b * a.tdx;
            // eta_Q exactly 0 (no alignment, sin(theta) = 0, or a line whose
            // w^(2) vanish) makes polarize_prop's eta_I/eta_Q * sinh(0) a NaN
            // (raytrace.f90:41-53): carried as a NaN coefficient, so I, Q, U
            // turn NaN wherever the reference's do, tau stays finite
            o = make_float4((float)(nI * f), nQ == 0.0 ? __int_as_float(0x7fc00000) : (float)(nQ * f),
                            (float)(eI * f), (float)(eQ * f));
        }
        a.coef[(size_t)j * N + n] = o;
    }
}

struct ImArgs {
    int N, npx, im_pix, nlines, nvel, nch, n_depth;
    int mode, nrays;         // 0: pixel grid, nrays = npx^2; 1: one ray per bulk node
    int star;                // star mode: rays starting on the star's disc start at its front
    double Rs, sx, sy, sz;   // R_star / tx and the rotated star position
    double im_size, dx, tdx, alpha, dvel, v0;
    const double *xyz;       // rotated (3,N)
    const double *nrm2;      // |X|^2 per node
    const int *off, *idx;    // neighbour CSR
    const float4 *cellv, *cellb, *coef;
    const double *dust_p, *tdust;
    int2 *walk;              // per warp: 32 pixels x n_depth
    unsigned long long *counters;
    int *status;
    float *out[8];           // (npx, npx, nch, nlines) or (nrays, nch, nlines) each, or null
};

__device__ __forceinline__ float phi1(float x) {  // (1 - e^-x)/x, stable near 0
    if (fabsf(x) < 0.1f)
        return 1.f + x * (-0.5f + x * (1.f / 6.f + x * (-1.f / 24.f + x * (1.f / 120.f + x * (-1.f / 720.f)))));
    return (1.f - expf(-x)) / x;
}

// Exponent of the lowest set bit of a double (v = m 2^e with m odd); a large
// value for 0, which constrains nothing.
__device__ __forceinline__ int lsb_exp(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffULL;
    if (b == 0ULL) return 1 << 20;
    int ex = (int)(b >> 52);
    unsigned long long m = b & 0xfffffffffffffULL;
    if (ex) {
        m |= 1ULL << 52;
        ex -= 1075;
    } else {
        ex = -1074;
    }
    return ex + __ffsll((long long)m) - 1;
}

// n successive FP64 additions z = z + dx, bit for bit, in O(binades) steps.
// While every partial sum z + j dx is representable -- all of them are
// multiples of g = min(lsb(z), lsb(dx)), so each is exact as long as its
// magnitude stays below L = g 2^53 -- the additions are exact and their
// result is the single correctly rounded fma(m, dx, z) (m dx itself is exact:
// dx is the REAL*4 step, a 24-bit mantissa, and m < 2^29).  Only a sum that
// enters a binade whose spacing exceeds g can round; that one addition is
// made as the reference makes it, after which z lies on the coarser grid.
__device__ double add_steps(double z, long long n, double dx, int e_dx) {
    while (n > 0) {
        const int eg = min(lsb_exp(z), e_dx);
        const double L = ldexp(1.0, eg + 53);
        long long m = (long long)floor(__ddiv_rn(__dsub_rn(L, z), dx)) - 2;  // z + m dx < L, with margin
        if (m > n) m = n;
        if (m > 0) {
            z = __fma_rn((double)m, dx, z);
            n -= m;
        }
        if (n > 0) {
            z = __dadd_rn(z, dx);
            n--;
        }
    }
    return z;
}

__device__ double black_body(double T, double nu) {
    if (T == 0.0) return 0.0;
    return 1.4744995e-50 * nu * nu * nu / (exp(4.79924e-11 / T * nu) - 1.0);
}

template <int NS>
__global__ void __launch_bounds__(128, 1) k_image(ImArgs a) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const long long gw = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    int2 *const wbase = a.walk + (size_t)gw * 32 * (size_t)a.n_depth;
    const int npix = a.nrays;
    const int e_dx = lsb_exp(a.dx);
    for (;;) {
        int p0 = 0;
        if (lane == 0) p0 = (int)atomicAdd(&a.counters[0], 32ULL);
        p0 = __shfl_sync(FULL, p0, 0);
        if (p0 >= npix) break;
        // ---- (1) march, one lane per pixel ----
        // Work index w -> the reference's pixel p = a npx + b (para_finish.f90:
        // 369-376) with a = w mod npx: consecutive work items step along the
        // cube's first (fastest) index, so the batch's stores of a channel fill
        // whole sectors instead of one float every npx^2 (mode 1: w is the node)
        const int w = p0 + lane;
        const int p = (a.mode == 1 || w >= npix) ? w : (w % a.npx) * a.npx + w / a.npx;
        int nc = 0, st = 0, fs = 0;  // fs: the ray starts on the star
        if (p < npix) {
            double x, y;
            if (a.mode == 1) {  // the node's rotated sky position (para_finish.f90:296)
                x = a.xyz[3 * (size_t)p];
                y = a.xyz[3 * (size_t)p + 1];
            } else {
                const int ia = p / a.npx - a.im_pix, ib = p % a.npx - a.im_pix;
                x = ia * a.im_size / a.im_pix;
                y = ib * a.im_size / a.im_pix;
            }
            // the oracle's FP64 arithmetic, without FMA contraction, throughout the march
            const double zs0 = -1.0 * __dsqrt_rn(__dsub_rn(__dsub_rn(1.0, __dmul_rn(x, x)), __dmul_rn(y, y)));
            double z0 = zs0;
            if (a.star) {  // raytrace.f90:103-115: on the star's disc, start at its front
                const double xc = __dsub_rn(x, a.sx), yc = __dsub_rn(y, a.sy);
                if (__dsqrt_rn(__dadd_rn(__dmul_rn(xc, xc), __dmul_rn(yc, yc))) < a.Rs) {
                    z0 = __dadd_rn(a.sz, a.Rs);
                    fs = 1;
                }
            }
            int2 *dl = wbase + (size_t)lane * a.n_depth;
            // nearest node to the start point (raytrace.f90:126-134 scans all
            // nodes; strict <, so the lowest index wins).  The same argmin by
            // greedy descent on the Delaunay graph: a node that is not the
            // nearest has a neighbour at most as far (the segment to the point
            // leaves its Voronoi cell through a face shared with that
            // neighbour), so descending in (distance, index) order from node 0
            // ends at the nearest node with the lowest index; distances are
            // computed exactly as the reference's norm2.
            auto dist = [&](int i) {
                return __dsqrt_rn(dsum3sq(x - a.xyz[3 * (size_t)i], y - a.xyz[3 * (size_t)i + 1],
                                          z0 - a.xyz[3 * (size_t)i + 2]));
            };
            int c = 0;
            double best = dist(0);
            for (int hop = 0; hop < a.N; hop++) {
                int nbest = c;
                double dbest = best;
                for (int q = a.off[c]; q < a.off[c + 1]; q++) {
                    const int nb = a.idx[q];
                    const double d = dist(nb);
                    if (d < dbest || (d == dbest && nb < nbest)) { dbest = d; nbest = nb; }
                }
                if (nbest == c) break;
                c = nbest;
                best = dbest;
            }
            if (!(best < 10.0)) { c = -1; st = 3; }  // start point outside the unit sphere (NaN; rsave = 10)
            double z = z0;
            int k = 0;
            const double zexit = -zs0;
            while (st == 0) {
                // predicted first step at which a neighbour is nearer than c
                const double cx = a.xyz[3 * (size_t)c], cy = a.xyz[3 * (size_t)c + 1],
                             cz = a.xyz[3 * (size_t)c + 2];
                const double cc = a.nrm2[c];
                const int o = a.off[c], deg = a.off[c + 1] - o;
                // Candidates of the replay below: the neighbours (of the first 64)
                // that come within 1e-12 of c's squared distance somewhere up to
                // z_lim.  Every other neighbour stays farther than c by more than
                // the FP64 rounding of both squared distances (~1e-15), so it
                // cannot win check_neigh's strict comparison and skipping it leaves
                // the scan's outcome unchanged.
                const double WIN = 6.0 * a.dx;
                unsigned long long cand = 0ULL;
                // the predicted crossing zt = tn / td, the minimum of A / (2 dzn) kept
                // as a fraction (compared by cross-multiplication, one division at the end)
                double tn = zexit, td = 1.0;
                for (int j = 0; j < deg; j++) {
                    const int nb = a.idx[o + j];
                    const double nx = a.xyz[3 * (size_t)nb], ny = a.xyz[3 * (size_t)nb + 1],
                                 nz = a.xyz[3 * (size_t)nb + 2];
                    // |P-X_n|^2 - |P-X_c|^2 = A - 2 z dzn along the ray
                    const double dzn = nz - cz;
                    const double A = a.nrm2[nb] - cc - 2.0 * x * (nx - cx) - 2.0 * y * (ny - cy);
                    if (A - 2.0 * z * dzn < 1e-12) {   // already (nearly) nearer: replay now
                        tn = z;
                        td = 1.0;
                        if (j < 64) cand |= 1ULL << j;
                    } else if (dzn > 0.0) {
                        const double d2 = 2.0 * dzn;
                        if (A * td < tn * d2) {
                            tn = A;
                            td = d2;
                        }
                        // A - 2 z' dzn <= 1e-12 for some z' <= zt + WIN (zt only falls
                        // further in this loop, so the set is a superset)
                        if (j < 64 && (A - 1e-12) * td <= d2 * (tn + WIN * td)) cand |= 1ULL << j;
                    }
                }
                const double zt = tn / td;
                const double z_lim = zt + WIN;
                long long kt = (long long)floor((zt - z0) / a.dx) - 3;
                if ((long long)k < kt) {  // the reference's own additions, in jumps
                    z = add_steps(z, kt - k, a.dx, e_dx);
                    k = (int)kt;
                }
                // exact replay of trace_out_raytrace's loop until c changes or the ray exits
                bool done = false, changed = false;
                while (!done && !changed) {
                    z = z + a.dx;
                    k++;
                    const bool exited = __dsqrt_rn(dsum3sq(x, y, z)) > 1.0;  // norm2(X_phot) > 1
                    if (exited) {
                        if (nc >= a.n_depth) { st = 1; break; }
                        dl[nc++] = make_int2(c, k);
                        done = true;
                    }
                    // check_neigh miscellaneous.f90:1-46, in list order: the candidates
                    // while z <= z_lim (and every neighbour past the 64th), else all
                    double d0 = dsum3sq(x - cx, y - cy, z - cz);
                    int nn = c;
                    auto probe = [&](int j) {
                        const int nb = a.idx[o + j];
                        const double ex = x - a.xyz[3 * (size_t)nb], ey = y - a.xyz[3 * (size_t)nb + 1],
                                     ez = z - a.xyz[3 * (size_t)nb + 2];
                        const double dd = dsum3sq(ex, ey, ez);
                        if (dd < d0) { d0 = dd; nn = nb; }
                    };
                    if (z <= z_lim) {
                        for (unsigned long long m = cand; m; m &= m - 1ULL) probe(__ffsll((long long)m) - 1);
                        for (int j = 64; j < deg; j++) probe(j);
                    } else {
                        for (int j = 0; j < deg; j++) probe(j);
                    }
                    if (nn != c) {
                        if (nc >= a.n_depth) { st = 1; break; }
                        dl[nc++] = make_int2(nn, k);
                        c = nn;
                        changed = true;
                    }
                }
                if (done || st) break;
            }
        }
        if (p < npix && a.status) a.status[p] = st;
        __syncwarp();
        // ---- (2) integration of each pixel of the batch, lanes over channels ----
        const int npx_b = min(32, npix - p0);
        for (int rr = 0; rr < npx_b; rr++) {
            const int ncr = __shfl_sync(FULL, nc, rr);
            const int str = __shfl_sync(FULL, st, rr);
            const int fsr = __shfl_sync(FULL, fs, rr);
            const int wr = p0 + rr;
            const int pix = (a.mode == 1) ? wr : (wr % a.npx) * a.npx + wr / a.npx;
            const int2 *dl = wbase + (size_t)rr * a.n_depth;
            for (int j = 0; j < a.nlines; j++) {
                const ImLine L = c_im[j];
                float I[NS], Q[NS], U[NS], tau[NS], tauc[NS];
                const double Iin_d = fsr ? L.bb_star : L.bb_cmb;  // I_in (raytrace.f90:97-115)
                const float Iin = (float)Iin_d;
#pragma unroll
                for (int s = 0; s < NS; s++) { I[s] = Iin; Q[s] = 0.f; U[s] = 0.f; tau[s] = 0.f; tauc[s] = 0.f; }
                // dust terms: channel independent, FP64, every lane alike
                double Id = Iin_d, sig0 = 0.0, sig2 = 0.0, Qd = 0.0, Ud = 0.0, taud = 0.0;
                for (int i = 0; i + 1 < ncr && str == 0; i++) {
                    const int2 e0 = dl[i], e1 = dl[i + 1];
                    const int cell = e0.x;
                    const int dk = e1.y - e0.y;
                    const float4 cv = a.cellv[cell];
                    const float4 cf = a.coef[(size_t)j * a.N + cell];
                    const float fdk = (float)dk;
#pragma unroll
                    for (int s = 0; s < NS; s++) {
                        const int ch = lane + 32 * s;
                        if (ch < a.nch) {
                            const float vobs = (float)((ch - a.nvel) * a.dvel + a.v0);
                            const float q = (vobs - cv.x) * cv.y;
                            const float vc = expf(-q * q) * fdk;
                            const float ta = cf.x * vc, tq = cf.y * vc, ei = cf.z * vc, eq = cf.w * vc;
                            if (ta > 1e-30f) {  // raytrace.f90:260
                                // rot_stokes into the node frame
                                const float Qn = Q[s] * cv.z + U[s] * cv.w;
                                const float Un = U[s] * cv.z - Q[s] * cv.w;
                                const float pm = ta - tq, pp = ta + tq;
                                const float Ep = expf(-pm), Em = expf(-pp);
                                const float fp = phi1(pm), fm = phi1(pp);
                                const float o11 = 0.5f * (fp + fm), o12 = -0.5f * (fp - fm);
                                const float ech = 0.5f * (Ep + Em), esh = 0.5f * (Ep - Em);
                                const float In = o11 * ei + o12 * eq + (ech * I[s] - esh * Qn);
                                const float Qo = o12 * ei + o11 * eq + (-esh * I[s] + ech * Qn);
                                const float Uo = Un * expf(-ta);
                                I[s] = In;
                                // rot_stokes_back
                                Q[s] = Qo * cv.z - Uo * cv.w;
                                U[s] = Uo * cv.z + Qo * cv.w;
                                // compensated tau sum
                                const float yk = ta - tauc[s];
                                const float tk = tau[s] + yk;
                                tauc[s] = (tk - tau[s]) - yk;
                                tau[s] = tk;
                            } else if (cv.z != cv.z) {
                                // the reference rotates Q, U into the node frame and back at
                                // every cell; a field along the line of sight has no frame
                                // (NaN angle), which makes them NaN there too
                                Q[s] = cv.z;
                                U[s] = cv.z;
                            }
                        }
                    }
                    // dust (raytrace.f90:268-290)
                    const double tau_d = L.kd * a.dust_p[cell] * (a.tdx * (double)dk);
                    if (tau_d > 1e-30) {
                        const float4 cb = a.cellb[cell];
                        const double Ibb = black_body(a.tdust[cell], L.nu0);
                        const double ed = exp(-tau_d);
                        const double mu2 = cb.x;
                        const double sI = 0.5 * a.alpha * (mu2 - 2.0 / 3.0), sQ = a.alpha * mu2;
                        Id = Id * ed + Ibb * (1 - ed);
                        sig0 = sig0 * ed + Ibb * (1 - ed);
                        sig2 = sig2 * ed + sI * Ibb * (1 - ed);
                        Qd = Qd * ed + sQ * Ibb * (1 - ed) * cb.y;
                        Ud = Ud * ed + sQ * Ibb * (1 - ed) * cb.z;
                        taud = taud + tau_d;
                    }
                }
                // finish (raytrace.f90:301-317)
                const double Ic = L.bb_cmb;
                double Idf = Id - Ic, Qdf = 0.0, Udf = 0.0, tdf = 0.0;
                if (Idf != 0.0) {
                    Qdf = Idf * Qd / (sig0 - sig2);
                    Udf = Idf * Ud / (sig0 - sig2);
                    tdf = taud;
                }
#pragma unroll
                for (int s = 0; s < NS; s++) {
                    const int ch = lane + 32 * s;
                    if (ch < a.nch) {
                        size_t o;
                        if (a.mode == 1) {
                            o = (size_t)pix + (size_t)a.nrays * ((size_t)ch + (size_t)a.nch * j);
                        } else {
                            const int ia = pix / a.npx, ib = pix % a.npx;
                            o = (size_t)ia + (size_t)a.npx * ((size_t)ib + (size_t)a.npx *
                                                              ((size_t)ch + (size_t)a.nch * j));
                        }
                        const bool bad = (str != 0);
                        const float vals[8] = {bad ? NAN : (float)((double)I[s] - Ic), bad ? NAN : Q[s],
                                               bad ? NAN : U[s], bad ? NAN : tau[s],
                                               bad ? NAN : (float)Idf, bad ? NAN : (float)Qdf,
                                               bad ? NAN : (float)Udf, bad ? NAN : (float)tdf};
#pragma unroll
                        for (int q2 = 0; q2 < 8; q2++)
                            if (a.out[q2]) a.out[q2][o] = vals[q2];
                    }
                }
            }
        }
        __syncwarp();
    }
}

}  // namespace

// mode 0: the pixel grid (2 im_pix + 1)^2; mode 1: one ray per bulk node
static int image_call(portal_ctx *c, const double *pol_pops, int nlines, const int *l1, const int *l2,
                      double th_inc, double ph_az, int nvel, double dvel, double v0, int mode, int im_pix,
                      double im_size, double alpha, double dx, int n_depth_rt, double *xy, float *const *dout,
                      int *status) {
    const char *fn = mode ? "portal_image_nodes" : "portal_image";
    if (!c->have_cloud || !c->have_mol) return set_err(c, PORTAL_ERR_STATE, "no cloud or molecule");
    if (nlines < 1 || nlines > IM_MAX_LINES || !l1 || !l2 || nvel < 0 || 2 * nvel + 1 > 288 ||
        im_pix < 1 || !(im_size > 0.0) || !(dx > 0.0) || n_depth_rt < 1)
        return set_err(c, PORTAL_ERR_ARG, std::string(fn) + ": bad arguments");
    if (mode == 0 && im_size * im_size * 2.0 >= 1.0)
        return set_err(c, PORTAL_ERR_ARG, "portal_image: im_size must keep the image corners inside "
                                          "the unit sphere (im_size < 1/sqrt(2))");
    if (!pol_pops && !c->pops.p)
        return set_err(c, PORTAL_ERR_STATE, std::string(fn) + ": no pol_pops (pass them or run portal_solve_se)");
    cudaSetDevice(c->device);
    timers_reset(c);
    const int N = c->N, nlev = c->nlev, nch = 2 * nvel + 1, npx = 2 * im_pix + 1;
    const int nrays = mode ? c->bulk : npx * npx;
    // line data (para_finish.f90:173-185): every line takes the frequency of the
    // last (l1, l2) pair, as the whole-array assignment there does
    ImLine h[IM_MAX_LINES];
    for (int i = 0; i < nlines; i++) {
        if (l1[i] < 1 || l1[i] > nlev || l2[i] < 1 || l2[i] > nlev)
            return set_err(c, PORTAL_ERR_ARG, std::string(fn) + ": line level out of range");
        if (mode && l1[i] > c->r_num)
            return set_err(c, PORTAL_ERR_ARG, "portal_image_nodes: t_Aji(l1) needs l1 <= the number of "
                                              "radiative transitions");
    }
    const double nu_last = c->e_levs[l2[nlines - 1] - 1] - c->e_levs[l1[nlines - 1] - 1];
    for (int i = 0; i < nlines; i++) {
        ImLine &L = h[i];
        L.nu0 = nu_last;
        L.A = 0.0; L.kd = 0.0;
        for (int r = 0; r < c->r_num; r++)
            if (l2[i] == c->r_trans[2 * r + 1] && l1[i] == c->r_trans[2 * r]) {
                L.A = c->A[r]; L.kd = c->kd_v[r];
                break;
            }
        if (mode) L.A = c->A[l1[i] - 1];  // para_finish.f90:303 passes t_Aji(l1(j))
        L.lo = l1[i] - 1; L.up = l2[i] - 1;
        L.j1 = c->j_lev[L.lo]; L.j2 = c->j_lev[L.up];
        L.w1 = wigner6j(2, 2, 4, 2 * L.j1, 2 * L.j1, 2 * L.j2);
        L.w2 = wigner6j(2, 2, 4, 2 * L.j2, 2 * L.j2, 2 * L.j1);
        L.fas = ((1 + L.j1 + L.j2) % 2 == 0) ? 1.0 : -1.0;
        L.bb_cmb = 1.4744995e-50 * std::pow(nu_last, 3.0) *
                   std::pow(std::exp(4.79924e-11 / 2.73 * nu_last) - 1.0, -1.0);
        L.bb_star = (c->star_mode && c->T_star > 0.0)
                        ? 1.4744995e-50 * std::pow(nu_last, 3.0) *
                              std::pow(std::exp(4.79924e-11 / c->T_star * nu_last) - 1.0, -1.0)
                        : 0.0;
    }
    PCHECK(c, cudaMemcpyToSymbolAsync(c_im, h, sizeof(ImLine) * nlines, 0, cudaMemcpyHostToDevice, c->stream));
    // rotation R_tot = R_z(ph_az) R_x(th_inc) (rotmat miscellaneous.f90:146-181)
    auto rotmat = [](const double *nv, double th, double *R) {
        double ct = std::cos(th), oc = 1.0 - ct, s = std::sin(th);
        for (int i = 0; i < 3; i++) R[i + 3 * i] = ct + oc * nv[i] * nv[i];
        R[0 + 3 * 1] = nv[0] * nv[1] * oc - nv[2] * s; R[1 + 3 * 0] = nv[1] * nv[0] * oc + nv[2] * s;
        R[0 + 3 * 2] = nv[0] * nv[2] * oc + nv[1] * s; R[2 + 3 * 0] = nv[2] * nv[0] * oc - nv[1] * s;
        R[1 + 3 * 2] = nv[1] * nv[2] * oc - nv[0] * s; R[2 + 3 * 1] = nv[2] * nv[1] * oc + nv[0] * s;
    };
    const double xv[3] = {1, 0, 0}, zv[3] = {0, 0, 1};
    double Rth[9], Rph[9];
    rotmat(xv, th_inc, Rth);
    rotmat(zv, ph_az, Rph);
    ImNodeArgs na;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double s = 0.0;
            for (int k = 0; k < 3; k++) s += Rph[i + 3 * k] * Rth[k + 3 * j];
            na.R[i + 3 * j] = s;
        }
    // device buffers
    DevBuf<double> xyz_r, pops_d, vel_d, nrm2;
    DevBuf<int> jl;
    DevBuf<float4> cellv, cellb, coef;
    DevBuf<float> outd;
    DevBuf<int> stat;
    const size_t cube = (size_t)nrays * nch * nlines;
    if (xyz_r.reserve(3 * (size_t)N) || nrm2.reserve(N) || cellv.reserve(N) || cellb.reserve(N) ||
        coef.reserve((size_t)nlines * N) || jl.reserve(nlev) || stat.reserve((size_t)(nrays > 0 ? nrays : 1)))
        return set_err(c, PORTAL_ERR_NOMEM, "image buffers");
    const double *pops_src = c->pops.p;
    if (pol_pops) {
        if (pops_d.reserve((size_t)N * 2 * nlev)) return set_err(c, PORTAL_ERR_NOMEM, "pol_pops");
        PCHECK(c, cudaMemcpyAsync(pops_d.p, pol_pops, (size_t)N * 2 * nlev * sizeof(double),
                                  cudaMemcpyHostToDevice, c->stream));
        pops_src = pops_d.p;
    }
    PCHECK(c, cudaMemcpyAsync(jl.p, c->j_lev.data(), nlev * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    na.N = N; na.bulk = c->bulk; na.nlev = nlev; na.nlines = nlines; na.tdx = c->tx * dx;
    na.xyz = c->pos64.p; na.vel = c->vel64.p; na.bvec = c->bvec64.p; na.b = c->b64.p;
    na.tdust = c->tdust.p; na.levp = c->levp.p; na.pops_in = pops_src; na.j_lev = jl.p;
    na.xyz_r = xyz_r.p; na.nrm2 = nrm2.p; na.cellv = cellv.p; na.cellb = cellb.p; na.coef = coef.p;
    timer_start(c, T_EMCOEF);
    k_im_nodes<<<(N + 127) / 128, 128, 0, c->stream>>>(na);
    timer_stop(c, T_EMCOEF);
    PCHECK(c, cudaGetLastError());
    // outputs on the device
    int nout = 0;
    for (int q = 0; q < 8; q++) nout += dout[q] ? 1 : 0;
    if (outd.reserve(cube * (nout ? nout : 1))) return set_err(c, PORTAL_ERR_NOMEM, "image outputs");
    ImArgs ia;
    ia.N = N; ia.npx = npx; ia.im_pix = im_pix; ia.nlines = nlines; ia.nvel = nvel; ia.nch = nch;
    ia.mode = mode; ia.nrays = nrays;
    // star mode: R_star / tx (para_finish.f90:187) and the star's position rotated with the
    // nodes (rotate_all_save miscellaneous.f90:899-904), used unscaled as the reference does
    ia.star = c->star_mode;
    ia.Rs = c->star_mode ? c->R_star() : 0.0;
    {
        double sp[3] = {0.0, 0.0, 0.0};
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++) sp[j] = sp[j] + na.R[j + 3 * k] * c->X_star[k];
        ia.sx = sp[0]; ia.sy = sp[1]; ia.sz = sp[2];
    }
    ia.n_depth = n_depth_rt; ia.im_size = im_size; ia.dx = dx; ia.tdx = c->tx * dx; ia.alpha = alpha; ia.dvel = dvel; ia.v0 = v0;
    ia.xyz = xyz_r.p; ia.nrm2 = nrm2.p; ia.off = c->nb_off.p; ia.idx = c->nb_idx.p; ia.cellv = cellv.p; ia.cellb = cellb.p;
    ia.coef = coef.p; ia.dust_p = c->dustp.p; ia.tdust = c->tdust.p; ia.status = stat.p;
    {
        int q2 = 0;
        for (int q = 0; q < 8; q++) ia.out[q] = dout[q] ? outd.p + cube * (q2++) : nullptr;
    }
    int grid = c->sm_count * 4;
    size_t nslots = (size_t)grid * 4;
    if (c->walk.reserve(nslots * 32 * (size_t)n_depth_rt) != cudaSuccess)
        return set_err(c, PORTAL_ERR_NOMEM, "image walk scratch");
    ia.walk = c->walk.p;
    ia.counters = c->counters.p;
    PCHECK(c, cudaMemsetAsync(c->counters.p, 0, sizeof(unsigned long long), c->stream));
    timer_start(c, T_IMWALK);
    if (nch <= 32) k_image<1><<<grid, 128, 0, c->stream>>>(ia);
    else if (nch <= 64) k_image<2><<<grid, 128, 0, c->stream>>>(ia);
    else if (nch <= 96) k_image<3><<<grid, 128, 0, c->stream>>>(ia);
    else if (nch <= 160) k_image<5><<<grid, 128, 0, c->stream>>>(ia);
    else k_image<9><<<grid, 128, 0, c->stream>>>(ia);
    timer_stop(c, T_IMWALK);
    PCHECK(c, cudaGetLastError());
    for (int q = 0; q < 8; q++)
        if (dout[q])
            PCHECK(c, cudaMemcpyAsync(dout[q], ia.out[q], cube * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    std::vector<int> sth((size_t)nrays);
    std::vector<double> xyz_h;
    if (xy) {
        xyz_h.resize(3 * (size_t)N);
        PCHECK(c, cudaMemcpyAsync(xyz_h.data(), xyz_r.p, xyz_h.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                  c->stream));
    }
    PCHECK(c, cudaMemcpyAsync(sth.data(), stat.p, sth.size() * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    PCHECK(c, cudaStreamSynchronize(c->stream));
    timer_collect(c, T_EMCOEF);
    timer_collect(c, T_IMWALK);
    if (status) std::copy(sth.begin(), sth.end(), status);
    if (xy)  // the rows of inc%02d-xy.dat (para_finish.f90:269-271)
        for (int n = 0; n < nrays; n++) {
            xy[2 * (size_t)n] = c->tx * xyz_h[3 * (size_t)n];
            xy[2 * (size_t)n + 1] = c->tx * xyz_h[3 * (size_t)n + 1];
        }
    for (size_t i = 0; i < sth.size(); i++)
        if (sth[i] == 1)
            return set_err(c, PORTAL_ERR_DEPTH, std::string("node_count > n_depth_rt for ") +
                                                    (mode ? "node " : "pixel ") + std::to_string(i + 1));
    return PORTAL_OK;
}

extern "C" int portal_image(portal_ctx *c, const double *pol_pops, int nlines, const int *l1,
                            const int *l2, double th_inc, double ph_az, int nvel, double dvel,
                            double v0, int im_pix, double im_size, double alpha, double dx,
                            int n_depth_rt, float *I, float *Q, float *U, float *tau, float *dust_I,
                            float *dust_Q, float *dust_U, float *dust_tau, int *status) {
    if (!c) return PORTAL_ERR_ARG;
    float *const out[8] = {I, Q, U, tau, dust_I, dust_Q, dust_U, dust_tau};
    return image_call(c, pol_pops, nlines, l1, l2, th_inc, ph_az, nvel, dvel, v0, 0, im_pix, im_size, alpha, dx,
                      n_depth_rt, nullptr, out, status);
}

extern "C" int portal_image_nodes(portal_ctx *c, const double *pol_pops, int nlines, const int *l1,
                                  const int *l2, double th_inc, double ph_az, int nvel, double dvel,
                                  double v0, double alpha, double dx, int n_depth_rt, double *xy, float *I,
                                  float *Q, float *U, float *tau, float *dust_I, float *dust_Q, float *dust_U,
                                  float *dust_tau, int *status) {
    if (!c) return PORTAL_ERR_ARG;
    float *const out[8] = {I, Q, U, tau, dust_I, dust_Q, dust_U, dust_tau};
    return image_call(c, pol_pops, nlines, l1, l2, th_inc, ph_az, nvel, dvel, v0, 1, 1, 0.5, alpha, dx,
                      n_depth_rt, xy, out, status);
}
