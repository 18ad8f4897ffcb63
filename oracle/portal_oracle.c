/*
 * portal_oracle.c -- FP64 CPU restatement of PORTAL's hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle).  It is imported by tests/, by
 * __graft_entry__.smoke() as the checker, and by bench.py's CPU-baseline
 * leg.  The product library never links it.
 *
 * Each function follows the reference routine cited beside it (paths are
 * relative to the PORTAL source tree).  Loop nesting, operation order and the
 * reference's REAL*4 literals are kept so that this is the reference's own
 * arithmetic in FP64; the few places where it cannot be (LAPACK's DGETRI,
 * wigxjpf, uninitialised variables) say so in place.
 */
#include "portal_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#if defined(__x86_64__) || defined(__i386__)
#include <quadmath.h>
typedef __float128 qreal;
#else
/* aarch64 and most other LP64 targets: long double is IEEE binary128 */
typedef long double qreal;
#endif

/* REAL*4 literals the reference assigns to / multiplies with FP64 values */
#define F4(x) ((double)(float)(x))

/* ------------------------------------------------------------------------ */
/* numerics                                                                  */
/* ------------------------------------------------------------------------ */

/* black_body miscellaneous.f90:263-285 */
double orc_black_body(double T, double nu0)
{
    if (T == 0.0) return 0.0;
    double c1 = 1.4744995e-50;      /* 2h/c^2 */
    double c2 = 4.79924e-11 / T;    /* h/(k_B T) */
    return c1 * pow(nu0, 3.0) * pow(exp(c2 * nu0) - 1.0, -1.0);
}

/* Gauss-Legendre knots/weights on (-1,1), ascending knots.  The reference
 * calls IQPACK's cdgqf (legendre_rule.f90:1-84, kind=1); this is the
 * textbook Newton iteration on P_n, which yields the same rule to the last
 * few ulps (pinned against numpy.polynomial.legendre.leggauss). */
void orc_gauss_legendre(int n, double *x, double *w)
{
    const double pi = acos(-1.0);
    for (int i = 0; i < n; i++) {
        long double z = cosl((long double)pi * (i + 0.75L) / (n + 0.5L));
        long double pp = 0.0L;
        for (int it = 0; it < 100; it++) {
            long double p0 = 1.0L, p1 = z;
            for (int k = 2; k <= n; k++) {
                long double p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
                p0 = p1; p1 = p2;
            }
            if (n == 1) { p1 = z; p0 = 1.0L; }
            pp = n * (z * p1 - p0) / (z * z - 1.0L);
            long double dz = p1 / pp;
            z -= dz;
            if (fabsl(dz) < 1e-19L) break;
        }
        {
            long double p0 = 1.0L, p1 = z;
            for (int k = 2; k <= n; k++) {
                long double p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
                p0 = p1; p1 = p2;
            }
            pp = n * (z * p1 - p0) / (z * z - 1.0L);
        }
        /* i-th root counted from +1 downwards: store ascending */
        x[n - 1 - i] = (double)z;
        w[n - 1 - i] = (double)(2.0L / ((1.0L - z * z) * pp * pp));
    }
}

/* legendre_all miscellaneous.f90:1100-1137 */
int orc_legendre_all(int nth, int nph, double *xth)
{
    double pi = acos(-1.0);
    double *x_th = (double *)malloc(sizeof(double) * nth);
    double *w_th = (double *)malloc(sizeof(double) * nth);
    orc_gauss_legendre(nth, x_th, w_th);
    int n_sphere = 0;
    for (int i = 0; i < nth; i++) {
        int np = (int)ceil(nph * sin(acos(x_th[i])));
        double w_ph = 2.0 * pi / np;
        double ww = w_ph * w_th[i];
        for (int j = 1; j <= np; j++) {
            xth[3 * n_sphere + 0] = x_th[i];
            xth[3 * n_sphere + 1] = (j - 1) * w_ph;
            xth[3 * n_sphere + 2] = ww / (4.0 * pi);
            n_sphere++;
        }
    }
    free(x_th);
    free(w_th);
    return n_sphere;
}

/* Wigner symbols.  The reference calls wigxjpf's fwig3jj/fwig6jj (exact
 * multi-word arithmetic, result rounded to double; library not vendored,
 * version unpinned).  Here: Racah's closed forms with the alternating sums
 * carried in binary128 so that cancellation leaves > 15 correct digits for
 * the angular momenta PORTAL's rotors use (pinned against sympy's exact
 * values in tests/golden/wigner.json).  Arguments are 2j, 2m like fwig*jj. */
static qreal q_fact(int n)
{
    static qreal tab[256];
    static int init = 0;
    if (!init) {
        tab[0] = 1;
        for (int i = 1; i < 256; i++) tab[i] = tab[i - 1] * (qreal)i;
        init = 1; /* benign race: every thread writes identical values */
    }
    return (n < 0 || n > 255) ? (qreal)0 : tab[n];
}

static int tri_ok(int ta, int tb, int tc)
{
    if ((ta + tb + tc) & 1) return 0;
    if (tc > ta + tb || tc < abs(ta - tb)) return 0;
    return 1;
}

static qreal q_delta(int ta, int tb, int tc) /* Delta(abc), args doubled */
{
    return q_fact((ta + tb - tc) / 2) * q_fact((ta - tb + tc) / 2) *
           q_fact((-ta + tb + tc) / 2) / q_fact((ta + tb + tc) / 2 + 1);
}

double orc_wigner3j(int tj1, int tj2, int tj3, int tm1, int tm2, int tm3)
{
    if (tm1 + tm2 + tm3 != 0) return 0.0;
    if (!tri_ok(tj1, tj2, tj3)) return 0.0;
    if (abs(tm1) > tj1 || abs(tm2) > tj2 || abs(tm3) > tj3) return 0.0;
    if (((tj1 + tm1) & 1) || ((tj2 + tm2) & 1) || ((tj3 + tm3) & 1)) return 0.0;
    int a = tj1, b = tj2, c = tj3;
    /* integer combinations (all halves) */
    int j1pm1 = (a + tm1) / 2, j1mm1 = (a - tm1) / 2;
    int j2pm2 = (b + tm2) / 2, j2mm2 = (b - tm2) / 2;
    int j3pm3 = (c + tm3) / 2, j3mm3 = (c - tm3) / 2;
    int k1 = (c - b + tm1) / 2;   /* j3 - j2 + m1 */
    int k2 = (c - a - tm2) / 2;   /* j3 - j1 - m2 */
    int k3 = (a + b - c) / 2;     /* j1 + j2 - j3 */
    int k4 = (a - tm1) / 2;       /* j1 - m1      */
    int k5 = (b + tm2) / 2;       /* j2 + m2      */
    int tmin = 0;
    if (-k1 > tmin) tmin = -k1;
    if (-k2 > tmin) tmin = -k2;
    int tmax = k3;
    if (k4 < tmax) tmax = k4;
    if (k5 < tmax) tmax = k5;
    qreal sum = 0;
    for (int t = tmin; t <= tmax; t++) {
        qreal den = q_fact(t) * q_fact(k1 + t) * q_fact(k2 + t) * q_fact(k3 - t) *
                    q_fact(k4 - t) * q_fact(k5 - t);
        qreal term = (qreal)1 / den;
        sum += (t & 1) ? -term : term;
    }
    qreal pre = q_delta(a, b, c) * q_fact(j1pm1) * q_fact(j1mm1) * q_fact(j2pm2) *
                q_fact(j2mm2) * q_fact(j3pm3) * q_fact(j3mm3);
    int ph = (a - b - tm3) / 2;   /* j1 - j2 - m3 */
    double r = (double)sum * sqrt((double)pre);
    if (ph & 1) r = -r;
    return r;
}

double orc_wigner6j(int tj1, int tj2, int tj3, int tj4, int tj5, int tj6)
{
    if (!tri_ok(tj1, tj2, tj3) || !tri_ok(tj1, tj5, tj6) || !tri_ok(tj4, tj2, tj6) ||
        !tri_ok(tj4, tj5, tj3))
        return 0.0;
    int a1 = (tj1 + tj2 + tj3) / 2, a2 = (tj1 + tj5 + tj6) / 2;
    int a3 = (tj4 + tj2 + tj6) / 2, a4 = (tj4 + tj5 + tj3) / 2;
    int b1 = (tj1 + tj2 + tj4 + tj5) / 2, b2 = (tj2 + tj3 + tj5 + tj6) / 2;
    int b3 = (tj3 + tj1 + tj6 + tj4) / 2;
    int tmin = a1;
    if (a2 > tmin) tmin = a2;
    if (a3 > tmin) tmin = a3;
    if (a4 > tmin) tmin = a4;
    int tmax = b1;
    if (b2 < tmax) tmax = b2;
    if (b3 < tmax) tmax = b3;
    qreal sum = 0;
    for (int t = tmin; t <= tmax; t++) {
        qreal den = q_fact(t - a1) * q_fact(t - a2) * q_fact(t - a3) * q_fact(t - a4) *
                    q_fact(b1 - t) * q_fact(b2 - t) * q_fact(b3 - t);
        qreal term = q_fact(t + 1) / den;
        sum += (t & 1) ? -term : term;
    }
    qreal pre = q_delta(tj1, tj2, tj3) * q_delta(tj1, tj5, tj6) * q_delta(tj4, tj2, tj6) *
                q_delta(tj4, tj5, tj3);
    return (double)sum * sqrt((double)pre);
}

/* rotmat miscellaneous.f90:146-181 (R stored column-major R[i + 3 j]) */
static void rotmat(const double *nv, double th, double *R)
{
    double cth = cos(th), octh = 1.0 - cth, sth = sin(th);
    for (int i = 0; i < 3; i++) R[i + 3 * i] = cth + octh * nv[i] * nv[i];
    R[0 + 3 * 1] = nv[0] * nv[1] * octh - nv[2] * sth;
    R[1 + 3 * 0] = nv[1] * nv[0] * octh + nv[2] * sth;
    R[0 + 3 * 2] = nv[0] * nv[2] * octh + nv[1] * sth;
    R[2 + 3 * 0] = nv[2] * nv[0] * octh - nv[1] * sth;
    R[1 + 3 * 2] = nv[1] * nv[2] * octh - nv[0] * sth;
    R[2 + 3 * 1] = nv[2] * nv[1] * octh + nv[0] * sth;
}

/* find_dir miscellaneous.f90:48-82 with two_mat_vec_prod :183-204 */
void orc_find_dir(const double *bvec, const double *gvec, double th, double ph, double *dir)
{
    double xv[3], Rth[9], Rph[9];
    xv[0] = bvec[1] * gvec[2] - bvec[2] * gvec[1];
    xv[1] = bvec[2] * gvec[0] - bvec[0] * gvec[2];
    xv[2] = bvec[0] * gvec[1] - bvec[1] * gvec[0];
    double xn = sqrt(xv[0] * xv[0] + xv[1] * xv[1] + xv[2] * xv[2]);
    for (int i = 0; i < 3; i++) xv[i] /= xn;
    rotmat(xv, th, Rth);
    rotmat(bvec, ph, Rph);
    for (int i = 0; i < 3; i++) {
        double d = 0.0;
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++) d = d + Rph[i + 3 * j] * Rth[j + 3 * k] * bvec[k];
        dir[i] = d;
    }
}

static double norm2_3(const double *v)
{
    return sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
}

/* find_angles miscellaneous.f90:86-134: (th, ph) of dir in the frame of
 * find_dir (z = bvec, x = bvec x gvec normalised) */
static void find_angles(const double *b, const double *g, const double *dir, double *th, double *ph)
{
    double xv[3] = {b[1] * g[2] - b[2] * g[1], b[2] * g[0] - b[0] * g[2], b[0] * g[1] - b[1] * g[0]};
    double xn = sqrt(xv[0] * xv[0] + xv[1] * xv[1] + xv[2] * xv[2]);
    for (int k = 0; k < 3; k++) xv[k] = xv[k] / xn;
    double bd = b[0] * dir[0] + b[1] * dir[1] + b[2] * dir[2];
    if (bd > 1.0) *th = acos(1.0);
    else if (bd < -1.0) *th = acos(-1.0);
    else *th = acos(bd);
    double cbd[3] = {b[1] * dir[2] - b[2] * dir[1], b[2] * dir[0] - b[0] * dir[2], b[0] * dir[1] - b[1] * dir[0]};
    *ph = atan2(xv[0] * dir[0] + xv[1] * dir[1] + xv[2] * dir[2], xv[0] * cbd[0] + xv[1] * cbd[1] + xv[2] * cbd[2]);
}

/* circle_points miscellaneous.f90:1228-1265: n points on the star's cap of
 * half-angle th_s, x(3,n) = (cos th, ph, weight).  One point keeps the
 * reference's x(1:2,1) = cos(1): polar angle 1 rad, azimuth cos(1). */
static void circle_points(int n, double th_s, double dth_s, double *x)
{
    const double pi = acos(-1.0);
    if (n == 1) {
        x[0] = cos(1.0);
        x[1] = cos(1.0);
        x[2] = 2.0 * pi * dth_s;
    } else if (n < 10) {
        double wph = 2.0 * pi / n, ww = wph * dth_s, xx = cos(th_s / 2.0);
        for (int i = 1; i <= n; i++) {
            x[3 * (i - 1)] = xx;
            x[3 * (i - 1) + 1] = (i - 1) * wph;
            x[3 * (i - 1) + 2] = ww;
        }
    } else {  /* Vogel's spiral, golden angle */
        double ga = pi * (3.0 - sqrt(5.0)), ww = dth_s * 2.0 * pi / n;
        for (int i = 1; i <= n; i++) {
            x[3 * (i - 1)] = cos(th_s * sqrt(1.0 * i / n));
            x[3 * (i - 1) + 1] = i * ga;
            x[3 * (i - 1) + 2] = ww;
        }
    }
}

int orc_star_all(int nth, int nph, const double *kvec, const double *gvec, const double *bvec,
                 double dOm_star, int *n_star_out, double *xth)
{
    const double pi = acos(-1.0);
    double dth_star = dOm_star / (2.0 * pi);
    double th_star = acos(1 - dth_star);
    double dOm_max = 4.0 * pi / (nth * nph);
    int n_star = (int)ceil(dOm_star / dOm_max);
    if (n_star > nth * nph) return -1;
    circle_points(n_star, th_star, dth_star, xth);
    for (int i = 0; i < n_star; i++) xth[3 * i + 2] = xth[3 * i + 2] / (4.0 * pi);
    int n_sphere = n_star;
    double dth_rest = (pi - th_star) / nth;
    double th_i = th_star + dth_rest / 2.0;
    for (int i = 1; i <= nth; i++) {
        double th = (i - 1) * dth_rest + th_i, wth;
        if (i == 1) {
            double th_u = (i - 0.5) * dth_rest + th_i;
            wth = cos(th_star) - cos(th_u);
        } else if (i == nth) {
            double th_l = (i - 1.5) * dth_rest + th_i;
            wth = cos(th_l) + 1.0;
        } else {
            double th_u = (i - 0.5) * dth_rest + th_i;
            double th_l = (i - 1.5) * dth_rest + th_i;
            wth = cos(th_l) - cos(th_u);
        }
        int np = (int)ceil(nph * sin(th));
        double wph = 2.0 * pi / np, xx = cos(th);
        for (int j = 1; j <= np; j++) {
            n_sphere++;
            if (n_sphere > nph * nth) return -1;
            xth[3 * (n_sphere - 1)] = xx;
            xth[3 * (n_sphere - 1) + 1] = (j - 1) * wph;
            xth[3 * (n_sphere - 1) + 2] = wth * wph / (4.0 * pi);
        }
    }
    for (int i = 0; i < n_sphere; i++) {
        double dir[3], th, ph;
        orc_find_dir(kvec, gvec, acos(xth[3 * i]), xth[3 * i + 1], dir);
        find_angles(bvec, gvec, dir, &th, &ph);
        xth[3 * i] = cos(th);
        xth[3 * i + 1] = ph;
    }
    *n_star_out = n_star;
    return n_sphere;
}

/* ------------------------------------------------------------------------ */
/* radiation field                                                           */
/* ------------------------------------------------------------------------ */

/* pos_quadratic miscellaneous.f90:1078-1098 ; x1 is left untouched when the
 * discriminant is not positive, as in the reference */
static int pos_quadratic(double a, double b, double c, double *x1)
{
    double dis = b * b - 4.0 * a * c;
    if (dis > 0) {
        double r1 = (-b + sqrt(dis)) / (2.0 * a);
        double r2 = (-b - sqrt(dis)) / (2.0 * a);
        if (r2 > 0) r1 = r2;
        *x1 = r1;
        return 0;
    }
    return 1;
}

/* check_neigh_fast miscellaneous.f90:1017-1076; star != 0 for a ray aimed
 * at the star (trace_out's mode 1): the star's surface ends the step and
 * the ray when it comes first */
static void check_neigh_fast(const orc_cloud *c, double *X_phot, const double *dir, int node,
                             int star, double *delta_x, int *next)
{
    const double *X_node = c->xyz + 3 * (node - 1);
    double nd = norm2_3(dir);
    double np = norm2_3(X_phot);
    pos_quadratic(nd * nd, 2.0 * (X_phot[0] * dir[0] + X_phot[1] * dir[1] + X_phot[2] * dir[2]),
                  np * np - 1.0, delta_x);
    *next = 0;
    double d0[3] = {X_node[0] - X_phot[0], X_node[1] - X_phot[1], X_node[2] - X_phot[2]};
    double n4 = norm2_3(d0);
    double q4 = n4 * n4;
    double q5 = d0[0] * dir[0] + d0[1] * dir[1] + d0[2] * dir[2];
    int nn = c->del_num_ne[node - 1];
    const double thr = F4(1e-10);
    for (int i = 0; i < nn; i++) {
        int nb = c->del_ne[(size_t)(node - 1) + (size_t)c->node_num * i];
        const double *Xn = c->xyz + 3 * (nb - 1);
        double d1[3] = {Xn[0] - X_phot[0], Xn[1] - X_phot[1], Xn[2] - X_phot[2]};
        double n1 = norm2_3(d1);
        double q1 = n1 * n1;
        double q2 = d1[0] * dir[0] + d1[1] * dir[1] + d1[2] * dir[2];
        double new_x = 0.5 * (q1 - q4) / (q2 - q5);
        if (new_x > *delta_x || new_x <= thr) continue;
        *delta_x = new_x;
        *next = nb;
    }
    if (star) {
        double ds[3] = {X_phot[0] - c->X_star[0], X_phot[1] - c->X_star[1], X_phot[2] - c->X_star[2]};
        double nds = norm2_3(ds), sx = 0.0;
        if (pos_quadratic(nd * nd, 2.0 * (ds[0] * dir[0] + ds[1] * dir[1] + ds[2] * dir[2]),
                          nds * nds - c->R_star * c->R_star, &sx) == 0 &&
            sx < *delta_x && sx > 0.0) {
            *delta_x = sx;
            *next = 0;
        }
    }
    for (int k = 0; k < 3; k++) X_phot[k] = X_phot[k] + *delta_x * dir[k];
}

/* trace_out inverse_rt.f90:139-214.  depth_list is (2, n_depth+1) with
 * column k = (cell id, cumulative steps).  Unlike the reference (which
 * writes past n_depth before it stops), the walk stops writing at n_depth
 * and returns ORC_ERR_DEPTH. */
static int trace_out(const orc_cloud *c, int node, const double *dir, double dx, int n_depth,
                     int star, int *depth_list, int *node_count);

int orc_trace_out(const orc_cloud *c, int node, const double *dir, double dx, int n_depth,
                  int *depth_list, int *node_count)
{
    return trace_out(c, node, dir, dx, n_depth, 0, depth_list, node_count);
}

static int trace_out(const orc_cloud *c, int node, const double *dir, double dx, int n_depth,
                     int star, int *depth_list, int *node_count)
{
    double X_phot[3];
    int cur = node, nc = 0;
    double delta_x = 0.0;
    memcpy(X_phot, c->xyz + 3 * (node - 1), sizeof X_phot);
    depth_list[0] = node;
    for (;;) {
        int next;
        check_neigh_fast(c, X_phot, dir, cur, star, &delta_x, &next);
        nc++;
        if (nc > n_depth) { *node_count = nc; return ORC_ERR_DEPTH; }
        depth_list[2 * (nc - 1) + 1] = (int)lround(delta_x / dx);  /* nint */
        depth_list[2 * nc + 0] = next;
        cur = next;
        if (next == 0) break;
    }
    for (int i = 1; i < nc; i++) depth_list[2 * i + 1] += depth_list[2 * (i - 1) + 1];
    *node_count = nc;
    return ORC_OK;
}

/* ray_in inverse_rt.f90:217-344 (gathered cell lists passed as in the
 * call at inverse_rt.f90:121-124).  When I_eff / lam are given (an
 * extension without reference counterpart: the split of the accelerated
 * Lambda iteration), the channel sum is also formed without the node's own
 * line emission, sum phi (I e^-tau + S_dust (1 - e^-tau)) dv, and for the
 * derivative with respect to the node's line source function,
 * sum phi (kv phi / kappa) (1 - e^-tau) dv. */
static double ray_in(const orc_cloud *c, const int *depth_list, int node_count, int node,
                     double vel_node, const double *vel_ray, int l1, int l2, double kd,
                     int nvel, double dx, double nu0, double Aji, double Bij, int g1, int g2,
                     double I_in, double *I_eff, double *lam)
{
    const int nlev = c->nlev;
    double c1 = 2.2102191e-42 * nu0;   /* h nu0 / c      */
    double c2 = 5.272859e-35 * nu0;    /* h nu0 / 4 pi   */
    double cnu = 299792458.0 / nu0;
    double temp_node = c->b_all[node - 1];
    double p1_node = c->lev_p[(size_t)nlev * (node - 1) + (l1 - 1)];
    double p2_node = c->lev_p[(size_t)nlev * (node - 1) + (l2 - 1)];
    double dust_node = c->dust_p[node - 1];
    double bb_node = c->t_dust[node - 1];
    double I_tot = 0.0, Ie_tot = 0.0, lam_tot = 0.0;
    double d_v = 2.0 * temp_node / nvel;
    double spi = sqrt(acos(-1.0));
    double kv, ev, I_bb, alpha_v, j_v, phi_v, tau_v, Sv, e_tau, I_out;

    for (int nv = -nvel; nv <= nvel; nv++) {
        double v0 = (2.0 * temp_node) * nv / nvel;
        double r = v0 / temp_node;
        double phi_v0 = (1.0 / (spi * temp_node)) * exp(-(r * r));
        v0 = v0 + vel_node;
        double Iv = I_in;
        for (int i = node_count; i >= 2; i--) {
            int cell = depth_list[2 * (i - 1)];
            double p1 = c->lev_p[(size_t)nlev * (cell - 1) + (l1 - 1)];
            double p2 = c->lev_p[(size_t)nlev * (cell - 1) + (l2 - 1)];
            kv = c1 * Bij * (p1 - (1.0 * g1) * p2 / (1.0 * g2));
            ev = c2 * Aji * p2;
            I_bb = orc_black_body(c->t_dust[cell - 1], nu0);
            alpha_v = kd * c->dust_p[cell - 1];
            j_v = alpha_v * I_bb;
            double bt = c->b_all[cell - 1];
            double q = (v0 - vel_ray[i - 1]) / bt;
            phi_v = cnu * (1.0 / (spi * bt)) * exp(-(q * q));
            tau_v = (kv * phi_v + alpha_v) * dx *
                    (double)(depth_list[2 * (i - 1) + 1] - depth_list[2 * (i - 2) + 1]);
            if (tau_v > 1e-30) {
                Sv = (ev * phi_v + j_v) / (kv * phi_v + alpha_v);
                e_tau = exp(-tau_v);
                Iv = Iv * e_tau + Sv * (1.0 - e_tau);
            }
        }
        kv = c1 * Bij * (p1_node - (1.0 * g1) * p2_node / (1.0 * g2));
        ev = c2 * Aji * p2_node;
        I_bb = orc_black_body(bb_node, nu0);
        alpha_v = kd * dust_node;
        j_v = alpha_v * I_bb;
        phi_v = phi_v0 * cnu;
        Sv = (ev * phi_v + j_v) / (kv * phi_v + alpha_v);
        tau_v = (kv * phi_v + alpha_v) * dx * (double)depth_list[1];
        e_tau = exp(-tau_v);
        I_out = Iv * e_tau + Sv * (1.0 - e_tau);
        I_tot = I_tot + phi_v0 * I_out * d_v;
        if (I_eff) {
            double kap = kv * phi_v + alpha_v;
            Ie_tot += phi_v0 * (Iv * e_tau + (j_v / kap) * (1.0 - e_tau)) * d_v;
            lam_tot += phi_v0 * (kv * phi_v / kap) * (1.0 - e_tau) * d_v;
        }
    }
    if (I_eff) { *I_eff = Ie_tot; *lam = lam_tot; }
    return I_tot;
}

/* inverse_rt inverse_rt.f90:1-137.  dx here is the trace step
 * (main_para.f90:135); ray_in receives tx*dx.  The first n_star rays are
 * star rays (star mode): traced in mode 1 and started from B(T_star). */
static int inverse_rt(const orc_cloud *c, const orc_molecule *m, int node, const double *xth,
                      int n_sphere, int n_star, const double *gvec, int nvel, double dx, int n_depth,
                      double *J0, double *J2, double *JE, double *LS, int64_t *n_segments)
{
    int t_num = m->r_num;
    int *depth_list = (int *)malloc(sizeof(int) * 2 * (size_t)(n_depth + 2));
    double *vel_ray = (double *)malloc(sizeof(double) * (size_t)(n_depth + 2));
    const double *bvec = c->bvec + 3 * (node - 1);
    const double *vn = c->vel + 3 * (node - 1);
    int st = ORC_OK;
    int64_t nseg = 0;
    for (int k = 0; k < t_num; k++) { J0[k] = 0.0; J2[k] = 0.0; }
    if (JE)
        for (int k = 0; k < t_num; k++) { JE[k] = 0.0; LS[k] = 0.0; }
    for (int i = 0; i < n_sphere; i++) {
        double mu = xth[3 * i], ph = xth[3 * i + 1], w = xth[3 * i + 2];
        double c_in = (3.0 * mu * mu - 1.0) / 2.0;
        double dir[3];
        orc_find_dir(bvec, gvec, acos(mu), ph, dir);
        int node_count;
        const int star_ray = (c->star_mod == 1 && i < n_star);
        st = trace_out(c, node, dir, dx, n_depth, star_ray, depth_list, &node_count);
        if (st != ORC_OK) break;
        nseg += node_count;
        double vel_node = vn[0] * dir[0] + vn[1] * dir[1] + vn[2] * dir[2];
        for (int l = 0; l < node_count; l++) {
            const double *vt = c->vel + 3 * (depth_list[2 * l] - 1);
            vel_ray[l] = vt[0] * dir[0] + vt[1] * dir[1] + vt[2] * dir[2];
        }
        for (int k = 0; k < t_num; k++) {
            double nu0 = m->nu[k];
            int l1 = m->r_trans[2 * k], l2 = m->r_trans[2 * k + 1];
            double I_in = star_ray ? orc_black_body(c->T_star, nu0) : orc_black_body(2.73, nu0);
            double Ie = 0.0, lam = 0.0;
            double I_out = ray_in(c, depth_list, node_count, node, vel_node, vel_ray, l1, l2,
                                  m->kd_v[k], nvel, c->tx * dx, nu0, m->A[k], m->Bij[k],
                                  2 * m->j_lev[l1 - 1] + 1, 2 * m->j_lev[l2 - 1] + 1, I_in,
                                  JE ? &Ie : NULL, JE ? &lam : NULL);
            J0[k] = J0[k] + I_out * w;
            J2[k] = J2[k] + I_out * w * c_in / sqrt(2.0);
            if (JE) {
                JE[k] += Ie * w;
                LS[k] += lam * w;
            }
        }
    }
    free(depth_list);
    free(vel_ray);
    if (n_segments) *n_segments = nseg;
    return st;
}

int orc_inverse_rt(const orc_cloud *c, const orc_molecule *m, int node, const double *xth,
                   int n_sphere, const double *gvec, int nvel, double dx, int n_depth,
                   double *J0, double *J2, int64_t *n_segments)
{
    return inverse_rt(c, m, node, xth, n_sphere, 0, gvec, nvel, dx, n_depth, J0, J2, NULL, NULL,
                      n_segments);
}

/* Star mode: is the node inside the star, which the node loop skips
 * (main_para.f90:232 compares |X| with R_star, the star taken as centred) */
static int inside_star(const orc_cloud *c, int node)
{
    return c->star_mod == 1 && !(norm2_3(c->xyz + 3 * (node - 1)) > c->R_star);
}

/* One node of the node loop main_para.f90:210-257, radiation field half of
 * trace_node (main_sub.f90:56-85; star mode: the node's own ray set from
 * star_all).  Returns the node's status; adds its segments to *ns. */
static int rf_node(const orc_cloud *c, const orc_molecule *m, int nth, int nph, int nvel,
                   const double *gvec, double dx, int n_depth, const double *xth, int n_sphere,
                   int node, double *J0, double *J2, double *JE, double *LS, int64_t *ns)
{
    const int t_num = m->r_num;
    double *j0 = J0 + (size_t)t_num * (node - 1);
    double *j2 = J2 + (size_t)t_num * (node - 1);
    double *je = JE ? JE + (size_t)t_num * (node - 1) : NULL;
    double *ls = JE ? LS + (size_t)t_num * (node - 1) : NULL;
    int st = ORC_OK;
    if (c->ab_all[node - 1] > 0.0 && c->star_mod == 1 && !inside_star(c, node)) {
        const double *X = c->xyz + 3 * (node - 1);
        double kv[3] = {c->X_star[0] - X[0], c->X_star[1] - X[1], c->X_star[2] - X[2]};
        double d = norm2_3(kv);
        double q = c->R_star / d;
        double dOm = acos(-1.0) * (q * q);
        for (int k = 0; k < 3; k++) kv[k] = kv[k] / d;
        double *xs = (double *)malloc(sizeof(double) * 3 * (size_t)nth * nph);
        int n_star = 0;
        int n_var = orc_star_all(nth, nph, kv, gvec, c->bvec + 3 * (node - 1), dOm, &n_star, xs);
        if (n_var < 0) {
            st = ORC_ERR_ARG;
            for (int k = 0; k < t_num; k++) { j0[k] = 0.0; j2[k] = 0.0; }
        } else {
            st = inverse_rt(c, m, node, xs, n_var, n_star, gvec, nvel, dx, n_depth, j0, j2, je, ls, ns);
        }
        free(xs);
    } else if (c->ab_all[node - 1] > 0.0 && c->star_mod != 1) {
        st = inverse_rt(c, m, node, xth, n_sphere, 0, gvec, nvel, dx, n_depth, j0, j2, je, ls, ns);
    } else {
        for (int k = 0; k < t_num; k++) { j0[k] = 0.0; j2[k] = 0.0; }
        if (je)
            for (int k = 0; k < t_num; k++) { je[k] = 0.0; ls[k] = 0.0; }
    }
    return st;
}

/* The node loop main_para.f90:210-257 over nodes node_lo..node_hi. */
int orc_radiation_field_split(const orc_cloud *c, const orc_molecule *m, int nth, int nph,
                              int nvel, const double *gvec, double dx, int n_depth, int node_lo,
                              int node_hi, int nthreads, double *J0, double *J2, double *JE,
                              double *LS, int *status, int64_t *n_segments)
{
    double *xth = (double *)malloc(sizeof(double) * 3 * (size_t)nth * nph);
    int n_sphere = orc_legendre_all(nth, nph, xth);
    int nfail = 0;
    int64_t nseg = 0;
    if (node_lo < 1) node_lo = 1;
    if (node_hi > c->bulk_node_num) node_hi = c->bulk_node_num;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(static) reduction(+ : nfail, nseg)
    for (int node = node_lo; node <= node_hi; node++) {
        int64_t ns = 0;
        int st = rf_node(c, m, nth, nph, nvel, gvec, dx, n_depth, xth, n_sphere, node, J0, J2, JE, LS, &ns);
        if (status) status[node - 1] = st;
        if (st != ORC_OK) nfail++;
        nseg += ns;
    }
    free(xth);
    if (n_segments) *n_segments = nseg;
    return nfail;
}

/* The same node loop over an arbitrary list of bulk nodes (1-based ids; a
 * sample of a cloud too large to restate whole).  Nodes vary widely in cost,
 * so the threads take them one at a time.  seg_per_node (n_nodes) or NULL
 * receives each listed node's segment count. */
int orc_radiation_field_nodes(const orc_cloud *c, const orc_molecule *m, int nth, int nph, int nvel,
                              const double *gvec, double dx, int n_depth, const int *nodes,
                              int n_nodes, int nthreads, double *J0, double *J2, double *JE,
                              double *LS, int *status, int64_t *seg_per_node)
{
    double *xth = (double *)malloc(sizeof(double) * 3 * (size_t)nth * nph);
    int n_sphere = orc_legendre_all(nth, nph, xth);
    int nfail = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : nfail)
    for (int i = 0; i < n_nodes; i++) {
        const int node = nodes[i];
        int64_t ns = 0;
        int st = ORC_ERR_ARG;
        if (node >= 1 && node <= c->bulk_node_num)
            st = rf_node(c, m, nth, nph, nvel, gvec, dx, n_depth, xth, n_sphere, node, J0, J2, JE, LS, &ns);
        if (status) status[i] = st;
        if (seg_per_node) seg_per_node[i] = ns;
        if (st != ORC_OK) nfail++;
    }
    free(xth);
    return nfail;
}

int orc_radiation_field(const orc_cloud *c, const orc_molecule *m, int nth, int nph, int nvel,
                        const double *gvec, double dx, int n_depth, int node_lo, int node_hi,
                        int nthreads, double *J0, double *J2, int *status,
                        int64_t *n_segments)
{
    return orc_radiation_field_split(c, m, nth, nph, nvel, gvec, dx, n_depth, node_lo, node_hi,
                                     nthreads, J0, J2, NULL, NULL, status, n_segments);
}

/* ------------------------------------------------------------------------ */
/* statistical equilibrium                                                   */
/* ------------------------------------------------------------------------ */

/* setup_count_array miscellaneous.f90:206-239; returns c_dim */
int orc_setup_count_array(const int *j_lev, int nlev, int kmax, int *count_array)
{
    int i_count = 0;
    count_array[0] = 0;
    for (int i = 0; i < nlev - 1; i++) {
        int j = j_lev[i];
        int kk = 2 * j < kmax ? 2 * j : kmax;
        for (int k = 0; k <= kk; k += 2) i_count++;
        count_array[i + 1] = i_count;
    }
    int j = j_lev[nlev - 1];
    int kk = 2 * j < kmax ? 2 * j : kmax;
    for (int k = 0; k <= kk; k += 2) i_count++;
    return i_count;
}

/* all_transitions miscellaneous.f90:394-460; returns n_trans */
int orc_all_transitions(const orc_molecule *m, int *all_trans)
{
    int nL = m->nlev;
    int *T = (int *)calloc((size_t)nL * nL, sizeof(int));
    for (int i = 0; i < m->r_num; i++) {
        int j = m->r_trans[2 * i], k = m->r_trans[2 * i + 1];
        if (m->e_levs[k - 1] > m->e_levs[j - 1]) T[(j - 1) + nL * (k - 1)] = 1;
        else T[(k - 1) + nL * (j - 1)] = 1;
    }
    for (int i = 0; i < m->c_num; i++) {
        int j = m->c_trans[2 * i], k = m->c_trans[2 * i + 1];
        if (m->e_levs[k - 1] > m->e_levs[j - 1]) T[(j - 1) + nL * (k - 1)] = 1;
        else T[(k - 1) + nL * (j - 1)] = 1;
    }
    int n = 0;
    for (int i = 1; i <= nL; i++)
        for (int j = 1; j <= nL; j++)
            if (T[(i - 1) + nL * (j - 1)]) {
                all_trans[2 * n] = i;
                all_trans[2 * n + 1] = j;
                n++;
            }
    free(T);
    return n;
}

/* make_AC miscellaneous.f90:288-392.  C_r is zero-initialised where the
 * reference leaves it undefined (Temp above the last table temperature). */
void orc_make_AC(const orc_molecule *m, double nH2, double Temp, int n_trans,
                 const int *all_trans, const double *J0, const double *J2, double *AC)
{
    int nT = m->c_temp, nC = m->c_num, nP = m->c_par;
    const double *C = m->C;
#define CIDX(t, c, p) ((size_t)(t) + (size_t)nT * ((size_t)(c) + (size_t)nC * (size_t)(p)))
    double *C_r = (double *)calloc((size_t)(nC > 0 ? nC : 1), sizeof(double));
    if (Temp <= m->col_temps[0] && nP == 1)
        for (int j = 0; j < nC; j++) C_r[j] = C[CIDX(0, j, 0)];
    if (Temp <= m->col_temps[0] && nP == 2)
        for (int j = 0; j < nC; j++) C_r[j] = 0.25 * C[CIDX(0, j, 0)] + 0.75 * C[CIDX(0, j, 1)];
    for (int i = 1; i < nT; i++) {
        if (m->col_temps[i] > Temp) {
            double ddT = (Temp - m->col_temps[i - 1]) / (m->col_temps[i] - m->col_temps[i - 1]);
            for (int j = 0; j < nC; j++) {
                if (nP == 1) {
                    double f1 = C[CIDX(i - 1, j, 0)], f2 = C[CIDX(i, j, 0)];
                    C_r[j] = f1 + ddT * (f2 - f1);
                } else if (nP == 2) {
                    double f1 = C[CIDX(i - 1, j, 0)], f2 = C[CIDX(i, j, 0)];
                    double f3 = C[CIDX(i - 1, j, 1)], f4 = C[CIDX(i, j, 1)];
                    double ff1 = f1 + ddT * (f2 - f1), ff2 = f3 + ddT * (f4 - f3);
                    C_r[j] = 0.25 * ff1 + 0.75 * ff2;
                }
            }
            break;
        }
    }
#undef CIDX
    for (int j = 0; j < nC; j++) C_r[j] = C_r[j] * nH2 * 1e-6;
    memset(AC, 0, sizeof(double) * 5 * (size_t)n_trans);
    for (int i = 0; i < n_trans; i++) {
        int lo = all_trans[2 * i], up = all_trans[2 * i + 1];
        AC[5 * i + 2] = m->e_levs[up - 1] - m->e_levs[lo - 1];
        for (int j = 0; j < m->r_num; j++)
            if (m->r_trans[2 * j] == lo && m->r_trans[2 * j + 1] == up) {
                AC[5 * i + 0] = m->A[j];
                AC[5 * i + 3] = J0[j];
                AC[5 * i + 4] = J2[j];
                break;
            }
        for (int j = 0; j < nC; j++)
            if (m->c_trans[2 * j] == lo && m->c_trans[2 * j + 1] == up) {
                AC[5 * i + 1] = C_r[j];
                break;
            }
    }
    free(C_r);
}

#define W3(a, b, c, d, e, f) orc_wigner3j(2 * (a), 2 * (b), 2 * (c), 2 * (d), 2 * (e), 2 * (f))
#define SGN(p) (((p) % 2 == 0) ? 1.0 : -1.0)   /* (-1.d0)**p for integral p */

/* t_abs_const pop_eqs.f90:1-78 */
static void t_abs_const(int j, int k, int jl, int kl, double *t0, double *t2)
{
    int dj = jl - j, dk = kl - k;
    *t0 = 0.0; *t2 = 0.0;
    if (abs(dj) <= 1) {
        double ljl = 2.0 * jl + 1.0;
        double fac1 = sqrt(3.0 * (2.0 * k + 1.0) * (2.0 * kl + 1.0));
        double fas = SGN(abs(1 - dj));
        double fac = ljl * fac1 * fas;
        if (dk == 0 || abs(dk) == 2) {
            for (int m = -j; m <= j; m++)
                for (int q = -1; q <= 1; q++) {
                    int ml = q + m;
                    double w1 = W3(j, j, k, m, -m, 0);
                    double w2 = W3(jl, jl, kl, ml, -ml, 0);
                    double w3 = W3(j, jl, 1, -m, ml, -q);
                    double w40 = W3(1, 1, 0, q, -q, 0);
                    double w42 = W3(1, 1, 2, q, -q, 0);
                    double ww = w1 * w2 * w3 * w3;
                    if (dk == 0) *t0 = *t0 + ww * w40;
                    *t2 = *t2 + ww * w42;
                }
            *t0 = *t0 * fac;
            *t2 = *t2 * sqrt(5.0) * fac;
        }
    }
}

/* t_stim_const pop_eqs.f90:80-156 */
static void t_stim_const(int j, int k, int ju, int ku, double *t0, double *t2)
{
    int dj = ju - j, dk = ku - k;
    *t0 = 0.0; *t2 = 0.0;
    if (abs(dj) <= 1) {
        double lju = 2.0 * ju + 1.0;
        double fac1 = sqrt(3.0 * (2.0 * k + 1.0) * (2.0 * ku + 1.0));
        double fas = SGN(abs(1 - dj));
        double fac = lju * fac1 * fas;
        if (dk == 0 || abs(dk) == 2) {
            for (int m = -j; m <= j; m++)
                for (int q = -1; q <= 1; q++) {
                    int mu = m - q;
                    double w1 = W3(j, j, k, m, -m, 0);
                    double w2 = W3(ju, ju, ku, mu, -mu, 0);
                    double w3 = W3(ju, j, 1, -mu, m, -q);
                    double w40 = W3(1, 1, 0, q, -q, 0);
                    double w42 = W3(1, 1, 2, q, -q, 0);
                    double ww = w1 * w2 * w3 * w3;
                    if (dk == 0) *t0 = *t0 + ww * w40;
                    *t2 = *t2 + ww * w42;
                }
            *t0 = *t0 * fac;
            *t2 = *t2 * sqrt(5.0) * fac;
        }
    }
}

/* t_spont_const pop_eqs.f90:158-201 */
static void t_spont_const(int j, int k, int ju, int ku, double *t0)
{
    int dj = ju - j, dk = ku - k;
    *t0 = 0.0;
    if (abs(dj) <= 1 && dk == 0) {
        double lju = 2.0 * ju + 1.0;
        double fas = SGN(abs(1 + j + ju + k));
        double w1 = orc_wigner6j(2 * ju, 2 * ju, 2 * k, 2 * j, 2 * j, 2);
        *t0 = lju * fas * w1;
    }
}

/* r_abs_const pop_eqs.f90:204-281 */
static void r_abs_const(int j, int k, int ju, int kp, double *r0, double *r2)
{
    int dj = ju - j, dk = kp - k;
    *r0 = 0.0; *r2 = 0.0;
    if (abs(dj) <= 1) {
        double lj = 2.0 * j + 1.0;
        double fac1 = sqrt(3.0 * (2.0 * k + 1.0) * (2.0 * kp + 1.0));
        if (dk == 0 || abs(dk) == 2) {
            for (int m = -j; m <= j; m++)
                for (int q = -1; q <= 1; q++) {
                    int mu = m - q;
                    double fas = SGN(abs(1 + q));
                    double fac = lj * fac1 * fas;
                    double w1 = W3(j, j, k, m, -m, 0);
                    double w2 = W3(j, j, kp, m, -m, 0);
                    double w3 = W3(ju, j, 1, -mu, m, -q);
                    double w40 = W3(1, 1, 0, q, -q, 0);
                    double w42 = W3(1, 1, 2, q, -q, 0);
                    double ww = w1 * w2 * w3 * w3;
                    if (dk == 0) *r0 = *r0 + fac * ww * w40;
                    *r2 = *r2 + fac * ww * w42;
                }
            *r2 = *r2 * sqrt(5.0);
        }
    }
}

/* r_stim_const pop_eqs.f90:283-359 */
static void r_stim_const(int j, int k, int jl, int kp, double *r0, double *r2)
{
    int dj = jl - j, dk = kp - k;
    *r0 = 0.0; *r2 = 0.0;
    if (abs(dj) <= 1) {
        double lj = 2.0 * j + 1.0;
        double fac1 = sqrt(3.0 * (2.0 * k + 1.0) * (2.0 * kp + 1.0));
        if (dk == 0 || abs(dk) == 2) {
            for (int m = -j; m <= j; m++)
                for (int q = -1; q <= 1; q++) {
                    int ml = m + q;
                    double fas = SGN(abs(1 - q));
                    double fac = lj * fac1 * fas;
                    double w1 = W3(j, j, k, m, -m, 0);
                    double w2 = W3(j, j, kp, m, -m, 0);
                    double w3 = W3(j, jl, 1, -m, ml, -q);
                    double w40 = W3(1, 1, 0, q, -q, 0);
                    double w42 = W3(1, 1, 2, q, -q, 0);
                    double ww = w1 * w2 * w3 * w3;
                    if (dk == 0) *r0 = *r0 + fac * ww * w40;
                    *r2 = *r2 + fac * ww * w42;
                }
            *r2 = *r2 * sqrt(5.0);
        }
    }
}

/* Exported for the tests that pin the coupling constants. */
void orc_coupling_constants(int which, int j, int k, int j2, int k2, double *c0, double *c2)
{
    *c0 = 0.0; *c2 = 0.0;
    switch (which) {
    case 0: t_abs_const(j, k, j2, k2, c0, c2); break;
    case 1: t_stim_const(j, k, j2, k2, c0, c2); break;
    case 2: t_spont_const(j, k, j2, k2, c0); break;
    case 3: r_abs_const(j, k, j2, k2, c0, c2); break;
    case 4: r_stim_const(j, k, j2, k2, c0, c2); break;
    default: break;
    }
}

/* de_polarization depol.f90:242-317 (Morris 1985 Eq. B11 in the form of
 * L&L04 Eq. 7.102).  C_j0 takes the rates of the collisional transitions
 * whose lower level is level 1, indexed by their upper level; the sum runs
 * over m = 1..2J with C_j0(:,m) -- level m, whose rate from level 1 is set
 * for m >= 2 and never for m = 1 (the reference leaves C_j0(:,1) unset; 0
 * here), and for m > nlev reads past the array (0 here).  The first
 * partner's rates (t_Cji(:,:,1)) are used. */
int orc_de_polarization(const orc_molecule *m, int kmax, double *D0_all)
{
    const int nlev = m->nlev, nT = m->c_temp, nk = kmax / 2;
    for (int i = 0; i < nlev; i++)
        if (m->j_lev[i] != i) return -1;   /* "only works if j_lev(i) = i-1" */
    double *Cj0 = (double *)calloc((size_t)nT * nlev, sizeof(double));
    for (int i = 0; i < m->c_num; i++)
        if (m->c_trans[2 * i] == 1) {
            int up = m->c_trans[2 * i + 1];
            for (int l = 0; l < nT; l++) Cj0[l + (size_t)nT * (up - 1)] = m->C[l + (size_t)nT * i];
        }
    for (size_t q = 0; q < (size_t)nT * nlev * (nk > 0 ? nk : 1); q++) D0_all[q] = 0.0;
#define D0A(l, i, k) D0_all[(size_t)(l) + (size_t)nT * ((size_t)(i - 1) + (size_t)nlev * (size_t)((k) / 2 - 1))]
    for (int i = 2; i <= nlev; i++) {
        int j = i - 1;
        double lj2 = pow(2.0 * j + 1.0, 2.0);
        for (int k = 2; k <= (2 * j < kmax ? 2 * j : kmax); k += 2) {
            for (int l = 0; l < nT; l++) {
                D0A(l, i, k) = 0.0;
                for (int mm = 1; mm <= 2 * j; mm++) {
                    double fac = pow(-1.0, mm) * (2.0 * mm + 1.0);
                    double w1 = orc_wigner3j(2 * j, 2 * j, 2 * mm, 0, 0, 0);
                    double w2 = orc_wigner6j(2 * j, 2 * j, 2 * mm, 2 * j, 2 * j, 0);
                    double w3 = orc_wigner6j(2 * j, 2 * j, 2 * mm, 2 * j, 2 * j, 2 * k);
                    double fac2 = w2 - w3;
                    /* m runs to 2J, past the nlev columns of C_j0 for the upper half
                     * of the levels (the reference reads beyond the array there); a
                     * level that does not exist has no rate: 0 */
                    double cj = (mm <= nlev) ? Cj0[l + (size_t)nT * (mm - 1)] : 0.0;
                    D0A(l, i, k) = D0A(l, i, k) + lj2 * fac * w1 * w1 * fac2 * cj;
                }
            }
        }
    }
#undef D0A
    free(Cj0);
    return 0;
}

/* make_depolarization_temp depol.f90:319-360.  Its loop over the table has
 * no exit: every bracket (i-1, i) with col_temps(i) > T overwrites D0, so
 * the last one, (nT-1, nT), sets it -- linear in that bracket, extrapolated
 * below it -- whenever T < col_temps(nT).  At or above col_temps(nT) the
 * reference leaves D0 unset (0 here). */
void orc_make_depolarization_temp(const double *D0_all, int nlev, int nT, int kmax,
                                  const double *col_temps, double T, double nH2, double *D0)
{
    const int nk = kmax / 2;
    for (int q = 0; q < nlev * nk; q++) D0[q] = 0.0;
    if (T <= col_temps[0])
        for (int q = 0; q < nlev * nk; q++) D0[q] = D0_all[(size_t)nT * q];
    for (int i = 2; i <= nT; i++) {
        if (col_temps[i - 1] > T) {
            double ddT = (T - col_temps[i - 2]) / (col_temps[i - 1] - col_temps[i - 2]);
            for (int q = 0; q < nlev * nk; q++) {
                double f1 = D0_all[(size_t)(i - 2) + (size_t)nT * q];
                double f2 = D0_all[(size_t)(i - 1) + (size_t)nT * q];
                D0[q] = f1 + ddT * (f2 - f1);
            }
        }
    }
    for (int q = 0; q < nlev * nk; q++) D0[q] = D0[q] * nH2 * 1e-6;
}

/* setup_stateq pop_eqs.f90:361-653.  Matrices column-major (c_dim,c_dim).
 * col_dep (pop_eqs.f90:642-648) is assigned D0(i1,k1) at the K = K' >= 2
 * diagonal entries and read by every entry's Amat; the reference never
 * initialises it (0 here) and passes D0 = 0 (main_sub.f90:96).  depol = 1
 * applies D0 only where it is assigned; depol = 2 keeps the last assigned
 * value in the later entries too, as the reference's code reads it. */
void orc_setup_stateq(int c_dim, const int *count_array, int nlev, const int *j_lev,
                      const int *trans, int ntrans, int kmax, const double *AC, double Temp,
                      const double *D0, int depol, double *Amat, double *A_mat, double *B_mat,
                      double *C_mat)
{
    const double a_to_b = 6.781962e49;
    size_t nn = (size_t)c_dim * c_dim;
#define M(X, r, cc) X[(size_t)((r) - 1) + (size_t)c_dim * (size_t)((cc) - 1)]
    memset(Amat, 0, sizeof(double) * nn);
    memset(A_mat, 0, sizeof(double) * nn);
    memset(B_mat, 0, sizeof(double) * nn);
    memset(C_mat, 0, sizeof(double) * nn);
    int *up = (int *)malloc(sizeof(int) * (ntrans + 1));
    int *dn = (int *)malloc(sizeof(int) * (ntrans + 1));
    double *ACu = (double *)malloc(sizeof(double) * 5 * (ntrans + 1));
    double *ACd = (double *)malloc(sizeof(double) * 5 * (ntrans + 1));
    double col_dep = 0.0;
    for (int i1 = 1; i1 <= nlev; i1++) {
        int cu = 0, cd = 0;
        for (int i2 = 1; i2 <= nlev; i2++)
            for (int q = 0; q < ntrans; q++) {
                if (trans[2 * q] == i1 && trans[2 * q + 1] == i2) {
                    up[cu] = i2;
                    memcpy(ACu + 5 * cu, AC + 5 * q, 5 * sizeof(double));
                    cu++;
                }
                if (trans[2 * q] == i2 && trans[2 * q + 1] == i1) {
                    dn[cd] = i2;
                    memcpy(ACd + 5 * cd, AC + 5 * q, 5 * sizeof(double));
                    cd++;
                }
            }
        int j1 = j_lev[i1 - 1];
        double g1 = 2.0 * j1 + 1.0;
        int k1max = 2 * j1 < kmax ? 2 * j1 : kmax;
        /* excitations i1 -> i2 (pop_eqs.f90:467-515) */
        for (int t = 0; t < cu; t++) {
            int i2 = up[t], j2 = j_lev[i2 - 1];
            double g2 = 2.0 * j2 + 1.0;
            double A21 = ACu[5 * t], C21 = ACu[5 * t + 1], nu0 = ACu[5 * t + 2];
            double JR0 = ACu[5 * t + 3], JR2 = ACu[5 * t + 4];
            double B21 = a_to_b * A21 / pow(nu0, 3.0);
            int k2max = 2 * j2 < kmax ? 2 * j2 : kmax;
            int c1 = count_array[i1 - 1];
            for (int k1 = 0; k1 <= k1max; k1 += 2) {
                c1++;
                int c2 = count_array[i2 - 1];
                for (int k2 = 0; k2 <= k2max; k2 += 2) {
                    c2++;
                    double ts0, ts2, te0;
                    t_stim_const(j1, k1, j2, k2, &ts0, &ts2);
                    t_spont_const(j1, k1, j2, k2, &te0);
                    double t_rad = B21 * (ts0 * JR0 + ts2 * JR2) + A21 * te0;
                    double t_col = 0.0;
                    if (k1 == k2 && k1 == 0) t_col = sqrt(g2 / g1) * C21;
                    M(Amat, c1, c2) = t_rad + t_col;
                    M(A_mat, c1, c2) = M(A_mat, c1, c2) + A21 * te0;
                    M(B_mat, c1, c2) = M(B_mat, c1, c2) + B21 * (ts0 * JR0 + ts2 * JR2);
                    M(C_mat, c1, c2) = M(C_mat, c1, c2) + t_col;
                }
            }
        }
        /* de-excitations i1 -> i2 (pop_eqs.f90:518-562) */
        for (int t = 0; t < cd; t++) {
            int i2 = dn[t], j2 = j_lev[i2 - 1];
            double g2 = 2.0 * j2 + 1.0;
            double A21 = ACd[5 * t], C21 = ACd[5 * t + 1], nu0 = ACd[5 * t + 2];
            double JR0 = ACd[5 * t + 3], JR2 = ACd[5 * t + 4];
            double B21 = a_to_b * A21 / pow(nu0, 3.0);
            double B12 = B21 * g1 / g2;
            double C12 = C21 * g1 * exp(-4.79924e-11 * nu0 / Temp) / g2;
            int k2max = 2 * j2 < kmax ? 2 * j2 : kmax;
            int c1 = count_array[i1 - 1];
            for (int k1 = 0; k1 <= k1max; k1 += 2) {
                c1++;
                int c2 = count_array[i2 - 1];
                for (int k2 = 0; k2 <= k2max; k2 += 2) {
                    c2++;
                    double ta0, ta2;
                    t_abs_const(j1, k1, j2, k2, &ta0, &ta2);
                    double t_rad = B12 * (ta0 * JR0 + ta2 * JR2);
                    double t_col = 0.0;
                    if (k1 == k2 && k1 == 0) t_col = sqrt(g2 / g1) * C12;
                    M(Amat, c1, c2) = t_rad + t_col;
                    M(B_mat, c1, c2) = M(B_mat, c1, c2) + t_rad;
                    M(C_mat, c1, c2) = M(C_mat, c1, c2) + t_col;
                }
            }
        }
        /* diagonal block (pop_eqs.f90:564-650) */
        {
            int c1 = count_array[i1 - 1];
            for (int k1 = 0; k1 <= k1max; k1 += 2) {
                c1++;
                int c2 = count_array[i1 - 1];
                for (int k2 = 0; k2 <= k1max; k2 += 2) {
                    c2++;
                    double rad_abs = 0.0, col_abs = 0.0, rad_stim = 0.0, col_stim = 0.0;
                    for (int t = 0; t < cu; t++) {
                        int i3 = up[t], j3 = j_lev[i3 - 1];
                        double g3 = 2.0 * j3 + 1.0;
                        double A21 = ACu[5 * t], C21 = ACu[5 * t + 1], nu0 = ACu[5 * t + 2];
                        double JR0 = ACu[5 * t + 3], JR2 = ACu[5 * t + 4];
                        double B21 = a_to_b * A21 / pow(nu0, 3.0);
                        double B12 = B21 * g3 / g1;
                        double C12 = C21 * g3 * exp(-4.79924e-11 * nu0 / Temp) / g1;
                        double r0, r2;
                        r_abs_const(j1, k1, j3, k2, &r0, &r2);
                        rad_abs = rad_abs + B12 * (JR0 * r0 + JR2 * r2);
                        M(B_mat, c1, c2) = M(B_mat, c1, c2) - B12 * (JR0 * r0 + JR2 * r2);
                        if (k1 == k2) {
                            col_abs = col_abs + C12;
                            M(C_mat, c1, c2) = M(C_mat, c1, c2) - C12;
                        }
                    }
                    for (int t = 0; t < cd; t++) {
                        int i3 = dn[t], j3 = j_lev[i3 - 1];
                        double A21 = ACd[5 * t], C21 = ACd[5 * t + 1], nu0 = ACd[5 * t + 2];
                        double JR0 = ACd[5 * t + 3], JR2 = ACd[5 * t + 4];
                        double B21 = a_to_b * A21 / pow(nu0, 3.0);
                        double r0, r2;
                        r_stim_const(j1, k1, j3, k2, &r0, &r2);
                        rad_stim = rad_stim + B21 * (JR0 * r0 + JR2 * r2);
                        M(B_mat, c1, c2) = M(B_mat, c1, c2) - B21 * (JR0 * r0 + JR2 * r2);
                        if (k1 == k2) {
                            rad_stim = rad_stim + A21;
                            col_stim = col_stim + C21;
                            M(A_mat, c1, c2) = M(A_mat, c1, c2) - A21;
                            M(C_mat, c1, c2) = M(C_mat, c1, c2) - C21;
                        }
                    }
                    if (depol == 1) col_dep = 0.0;
                    if (k1 == k2 && k2 >= 2) {
                        col_dep = (D0 && depol) ? D0[(i1 - 1) + nlev * (k1 / 2 - 1)] : 0.0;
                        M(C_mat, c1, c2) = M(C_mat, c1, c2) - col_dep;
                    }
                    M(Amat, c1, c2) = -1.0 * (rad_abs + rad_stim + col_abs + col_stim + col_dep);
                }
            }
        }
    }
#undef M
    free(up); free(dn); free(ACu); free(ACd);
}

/* LU with partial pivoting in the manner of LAPACK DGETRF (pivot = first
 * entry of largest modulus in the column), then the solve A x = e_1.
 * The reference forms inv(A) with DGETRI and keeps its first column
 * (em_coefs.f90:169-186); solving for e_1 gives the same vector up to
 * rounding (pinned against scipy's dgetrf/dgetri in the tests). */
static int lu_solve_e1(int n, double *A, double *x)
{
    int *piv = (int *)malloc(sizeof(int) * n);
#define A_(r, cc) A[(size_t)(r) + (size_t)n * (size_t)(cc)]
    for (int k = 0; k < n; k++) {
        int p = k;
        double amax = fabs(A_(k, k));
        for (int i = k + 1; i < n; i++)
            if (fabs(A_(i, k)) > amax) { amax = fabs(A_(i, k)); p = i; }
        piv[k] = p;
        if (A_(p, k) == 0.0) { free(piv); return ORC_ERR_LU; }
        if (p != k)
            for (int cc = 0; cc < n; cc++) { double t = A_(k, cc); A_(k, cc) = A_(p, cc); A_(p, cc) = t; }
        double r = 1.0 / A_(k, k);
        for (int i = k + 1; i < n; i++) A_(i, k) *= r;
        for (int cc = k + 1; cc < n; cc++) {
            double akc = A_(k, cc);
            if (akc != 0.0)
                for (int i = k + 1; i < n; i++) A_(i, cc) -= A_(i, k) * akc;
        }
    }
    for (int i = 0; i < n; i++) x[i] = 0.0;
    x[0] = 1.0;
    for (int k = 0; k < n; k++) if (piv[k] != k) { double t = x[k]; x[k] = x[piv[k]]; x[piv[k]] = t; }
    for (int i = 0; i < n; i++) for (int k = 0; k < i; k++) x[i] -= A_(i, k) * x[k];
    for (int i = n - 1; i >= 0; i--) {
        for (int k = i + 1; k < n; k++) x[i] -= A_(i, k) * x[k];
        x[i] /= A_(i, i);
    }
#undef A_
    free(piv);
    return ORC_OK;
}

/* get_rhovec em_coefs.f90:115-201 */
int orc_get_rhovec(int c_dim, const int *count_array, int nlev, const int *j_lev, int ntrans,
                   const int *trans, const double *AC, int kmax, double Temp, const double *D0,
                   int depol, double *rhovec, double *rates)
{
    size_t nn = (size_t)c_dim * c_dim;
    double *Amat = (double *)malloc(sizeof(double) * nn * 4);
    double *R_mat = Amat + nn, *B_mat = Amat + 2 * nn, *C_mat = Amat + 3 * nn;
    orc_setup_stateq(c_dim, count_array, nlev, j_lev, trans, ntrans, kmax, AC, Temp, D0, depol, Amat,
                     R_mat, B_mat, C_mat);
    for (int cc = 0; cc < c_dim; cc++) Amat[(size_t)c_dim * cc] = 0.0;
    for (int i = 0; i < nlev; i++) {
        int ic = count_array[i];
        Amat[(size_t)c_dim * ic] = sqrt(2.0 * j_lev[i] + 1.0);
    }
    int st = lu_solve_e1(c_dim, Amat, rhovec);
    if (st == ORC_OK && rates) {
        for (int i = 0; i < 3 * c_dim; i++) rates[i] = 0.0;
        for (int i = 0; i < c_dim; i++)
            for (int j = 0; j < c_dim; j++) {
                rates[3 * i + 0] += fabs(R_mat[i + (size_t)c_dim * j]) * rhovec[j];
                rates[3 * i + 1] += fabs(B_mat[i + (size_t)c_dim * j]) * rhovec[j];
                rates[3 * i + 2] += fabs(C_mat[i + (size_t)c_dim * j]) * rhovec[j];
            }
    }
    free(Amat);
    return st;
}

int orc_node_matrix(const orc_cloud *c, const orc_molecule *m, int kmax, int node,
                    const double *J0, const double *J2, double *Amat, int *c_dim_out)
{
    int nlev = m->nlev;
    int *count_array = (int *)malloc(sizeof(int) * nlev);
    int c_dim = orc_setup_count_array(m->j_lev, nlev, kmax, count_array);
    int *all_trans = (int *)malloc(sizeof(int) * 2 * (m->r_num + m->c_num + 1));
    int n_trans = orc_all_transitions(m, all_trans);
    double *AC = (double *)malloc(sizeof(double) * 5 * (n_trans + 1));
    orc_make_AC(m, c->h2_dens[node - 1], c->t_kin[node - 1], n_trans, all_trans,
                J0 + (size_t)m->r_num * (node - 1), J2 + (size_t)m->r_num * (node - 1), AC);
    size_t nn = (size_t)c_dim * c_dim;
    double *scr = (double *)malloc(sizeof(double) * nn * 3);
    double *D0_all = NULL, *D0 = NULL;
    if (m->depol && kmax >= 2) {
        D0_all = (double *)malloc(sizeof(double) * (size_t)m->c_temp * nlev * (kmax / 2));
        D0 = (double *)malloc(sizeof(double) * (size_t)nlev * (kmax / 2));
        if (orc_de_polarization(m, kmax, D0_all) == 0)
            orc_make_depolarization_temp(D0_all, nlev, m->c_temp, kmax, m->col_temps, c->t_kin[node - 1],
                                         c->h2_dens[node - 1], D0);
        else
            memset(D0, 0, sizeof(double) * (size_t)nlev * (kmax / 2));
    }
    orc_setup_stateq(c_dim, count_array, nlev, m->j_lev, all_trans, n_trans, kmax, AC,
                     c->t_kin[node - 1], D0, m->depol, Amat, scr, scr + nn, scr + 2 * nn);
    free(D0_all); free(D0);
    *c_dim_out = c_dim;
    free(scr); free(AC); free(all_trans); free(count_array);
    return ORC_OK;
}

/* SE half of trace_node main_sub.f90:93-137 over nodes node_lo..node_hi of
 * the bulk, in the node loop of main_para.f90:210-257. */
/* trace_node's SE half (main_sub.f90:93-137) for one node: pol_pops
 * (node_num, 2*nlev) column-major, rates (node_num,3,2*nlev) or NULL; AC,
 * rhovec and rt are the thread's work arrays.  Returns the node's status. */
static int se_node(const orc_cloud *c, const orc_molecule *m, int kmax, const double *J0,
                   const double *J2, int c_dim, const int *count_array, int n_trans,
                   const int *all_trans, const double *D0_all, int node, double *AC, double *D0,
                   double *rhovec, double *rt, double *pol_pops, double *rates)
{
    int nlev = m->nlev, N = c->node_num;
    int st = ORC_OK;
    if (c->ab_all[node - 1] > 0.0 && !inside_star(c, node)) {
        orc_make_AC(m, c->h2_dens[node - 1], c->t_kin[node - 1], n_trans, all_trans,
                    J0 + (size_t)m->r_num * (node - 1), J2 + (size_t)m->r_num * (node - 1), AC);
        if (D0_all)
            orc_make_depolarization_temp(D0_all, nlev, m->c_temp, kmax, m->col_temps, c->t_kin[node - 1],
                                         c->h2_dens[node - 1], D0);
        st = orc_get_rhovec(c_dim, count_array, nlev, m->j_lev, n_trans, all_trans, AC, kmax,
                            c->t_kin[node - 1], D0_all ? D0 : NULL, m->depol, rhovec, rates ? rt : NULL);
        if (st != ORC_OK) {
            for (int i = 0; i < c_dim; i++) rhovec[i] = NAN;
            for (int i = 0; i < 3 * c_dim; i++) rt[i] = 0.0;
        }
        for (int i = 0; i < nlev; i++) {
            size_t p0 = (size_t)(node - 1) + (size_t)N * (2 * i);
            size_t p1 = p0 + N;
            int ca = count_array[i];
            pol_pops[p0] = rhovec[ca];
            /* with kmax = 0 the reference reads the next level's rho^0_0 here,
             * and past the end of rhovec for the last level (0 here) */
            pol_pops[p1] = (m->j_lev[i] != 0 && ca + 1 < c_dim) ? rhovec[ca + 1] : 0.0;
            if (rates) {
                for (int q = 0; q < 3; q++) {
                    size_t r0 = (size_t)(node - 1) + (size_t)N * (q + 3 * (size_t)(2 * i));
                    size_t r1 = (size_t)(node - 1) + (size_t)N * (q + 3 * (size_t)(2 * i + 1));
                    rates[r0] = rt[3 * ca + q];
                    rates[r1] = (m->j_lev[i] != 0 && ca + 1 < c_dim) ? rt[3 * (ca + 1) + q] : 0.0;
                }
            }
            /* main_sub.f90:131-136 (the reference zeroes the same
             * rates entry twice; the restatement keeps that) */
            if (isnan(pol_pops[p0])) {
                pol_pops[p0] = 0.0;
                pol_pops[p1] = 0.0;
                if (rates)
                    for (int q = 0; q < 3; q++)
                        rates[(size_t)(node - 1) + (size_t)N * (q + 3 * (size_t)(2 * i + 1))] = 0.0;
            }
        }
    }
    return st;
}

/* The SE half of the node loop over nodes node_lo..node_hi (node_list NULL)
 * or over the n_list 1-based bulk nodes of node_list (status then per list
 * entry). */
static int solve_se_impl(const orc_cloud *c, const orc_molecule *m, int kmax, const double *J0,
                         const double *J2, int node_lo, int node_hi, const int *node_list,
                         int n_list, int nthreads, double *pol_pops, double *rates, int *status)
{
    int nlev = m->nlev;
    int *count_array = (int *)malloc(sizeof(int) * nlev);
    int c_dim = orc_setup_count_array(m->j_lev, nlev, kmax, count_array);
    int *all_trans = (int *)malloc(sizeof(int) * 2 * (m->r_num + m->c_num + 1));
    int n_trans = orc_all_transitions(m, all_trans);
    int nfail = 0;
    if (node_lo < 1) node_lo = 1;
    if (node_hi > c->bulk_node_num) node_hi = c->bulk_node_num;
    const int n_items = node_list ? n_list : (node_hi >= node_lo ? node_hi - node_lo + 1 : 0);
    double *D0_all = NULL;
    if (m->depol && kmax >= 2) {
        D0_all = (double *)malloc(sizeof(double) * (size_t)m->c_temp * nlev * (kmax / 2));
        if (orc_de_polarization(m, kmax, D0_all) != 0) {
            free(D0_all); free(count_array); free(all_trans);
            return -1;
        }
    }
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel reduction(+ : nfail)
    {
        double *AC = (double *)malloc(sizeof(double) * 5 * (n_trans + 1));
        double *rhovec = (double *)malloc(sizeof(double) * c_dim);
        double *rt = (double *)malloc(sizeof(double) * 3 * c_dim);
        double *D0 = (double *)malloc(sizeof(double) * (size_t)nlev * (kmax / 2 + 1));
#pragma omp for schedule(static)
        for (int it = 0; it < n_items; it++) {
            const int node = node_list ? node_list[it] : node_lo + it;
            int st = ORC_ERR_ARG;
            if (node >= 1 && node <= c->bulk_node_num)
                st = se_node(c, m, kmax, J0, J2, c_dim, count_array, n_trans, all_trans, D0_all, node, AC, D0,
                             rhovec, rt, pol_pops, rates);
            if (status) status[node_list ? it : node - 1] = st;
            if (st != ORC_OK) nfail++;
        }
        free(AC); free(rhovec); free(rt); free(D0);
    }
    free(count_array); free(all_trans); free(D0_all);
    return nfail;
}

int orc_solve_se(const orc_cloud *c, const orc_molecule *m, int kmax, const double *J0,
                 const double *J2, int node_lo, int node_hi, int nthreads, double *pol_pops,
                 double *rates, int *status)
{
    return solve_se_impl(c, m, kmax, J0, J2, node_lo, node_hi, NULL, 0, nthreads, pol_pops, rates, status);
}

int orc_solve_se_nodes(const orc_cloud *c, const orc_molecule *m, int kmax, const double *J0,
                       const double *J2, const int *nodes, int n_nodes, int nthreads,
                       double *pol_pops, double *rates, int *status)
{
    return solve_se_impl(c, m, kmax, J0, J2, 1, c->bulk_node_num, nodes, n_nodes, nthreads, pol_pops, rates,
                         status);
}

/* ------------------------------------------------------------------------ */
/* Stokes image                                                              */
/* ------------------------------------------------------------------------ */

/* comp_emcoefs em_coefs.f90:1-113 */
void orc_comp_emcoefs(double r1_0, double r2_0, double r1_2, double r2_2, int j1, int j2,
                      double th, double nu0, double Aji, double *nsI_tot, double *nsQ_tot,
                      double *es_I, double *es_Q)
{
    double fas = SGN(abs(1 + j1 + j2));
    double fac1 = sqrt(3.0 * (2.0 * j1 + 1.0));
    double fac2 = sqrt(3.0 * (2.0 * j2 + 1.0));
    double w6_1 = orc_wigner6j(2, 2, 4, 2 * j1, 2 * j1, 2 * j2);
    double w6_2 = orc_wigner6j(2, 2, 4, 2 * j2, 2 * j2, 2 * j1);
    double wjj2_1 = fas * fac1 * w6_1;
    double wjj2_2 = fas * fac2 * w6_2;
    double g1 = 2.0 * j1 + 1.0, g2 = 2.0 * j2 + 1.0;
    double ct = cos(th), st = sin(th);
    double tki = (3.0 * ct * ct - 1.0) / (2.0 * sqrt(2.0));
    double tkq = -3.0 * st * st / (2.0 * sqrt(2.0));
    double na_I = 1.0 + wjj2_1 * (r1_2 / r1_0) * tki;
    double na_Q = wjj2_1 * (r1_2 / r1_0) * tkq;
    double ns_I = 1.0 + wjj2_2 * (r2_2 / r2_0) * tki;
    double ns_Q = wjj2_2 * (r2_2 / r2_0) * tkq;
    double a_to_b = 6.781962e49;
    double b_to_a = pow(nu0, 3.0) / a_to_b;
    double Bji = Aji / b_to_a;
    double eI = ns_I, eQ = ns_Q;
    double nI = sqrt(g1) * r1_0 * na_I - sqrt(g2) * r2_0 * ns_I * g1 / g2;
    double nQ = sqrt(g1) * r1_0 * na_Q - sqrt(g2) * r2_0 * ns_Q * g1 / g2;
    double hv_fac = 5.273e-35 * nu0;
    *es_I = hv_fac * Aji * eI * sqrt(g2) * r2_0;
    *es_Q = hv_fac * Aji * eQ * sqrt(g2) * r2_0;
    *nsI_tot = hv_fac * (g2 / g1) * Bji * nI;
    *nsQ_tot = hv_fac * (g2 / g1) * Bji * nQ;
}

/* rotate_all_save miscellaneous.f90:844-907 (star coordinates omitted) */
void orc_rotate_all_save(int node_num, double th_inc, double ph_az, const double *vel,
                         const double *bvec, const double *xyz, double *vel_new,
                         double *bvec_new, double *xyz_new)
{
    double xv[3] = {1, 0, 0}, zv[3] = {0, 0, 1}, Rth[9], Rph[9], R[9];
    rotmat(xv, th_inc, Rth);
    rotmat(zv, ph_az, Rph);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double s = 0.0;
            for (int k = 0; k < 3; k++) s += Rph[i + 3 * k] * Rth[k + 3 * j];
            R[i + 3 * j] = s;
        }
    for (int n = 0; n < node_num; n++)
        for (int j = 0; j < 3; j++) {
            double sv = 0.0, sb = 0.0, sx = 0.0;
            for (int k = 0; k < 3; k++) {
                sv = sv + R[j + 3 * k] * vel[3 * n + k];
                sb = sb + R[j + 3 * k] * bvec[3 * n + k];
                sx = sx + R[j + 3 * k] * xyz[3 * n + k];
            }
            vel_new[3 * n + j] = sv;
            bvec_new[3 * n + j] = sb;
            xyz_new[3 * n + j] = sx;
        }
}

/* check_neigh miscellaneous.f90:1-46 */
static int check_neigh(const double *X_phot, int node, const double *xyz, const int *del_ne,
                       const int *del_num_ne, int node_num)
{
    const double *Xc = xyz + 3 * (node - 1);
    double x0[3] = {X_phot[0] - Xc[0], X_phot[1] - Xc[1], X_phot[2] - Xc[2]};
    double dis_0 = x0[0] * x0[0] + x0[1] * x0[1] + x0[2] * x0[2];
    int new_node = node;
    int nn = del_num_ne[node - 1];
    for (int i = 0; i < nn; i++) {
        int nb = del_ne[(size_t)(node - 1) + (size_t)node_num * i];
        const double *Xn = xyz + 3 * (nb - 1);
        double xn[3] = {X_phot[0] - Xn[0], X_phot[1] - Xn[1], X_phot[2] - Xn[2]};
        double dis = xn[0] * xn[0] + xn[1] * xn[1] + xn[2] * xn[2];
        if (dis < dis_0) { dis_0 = dis; new_node = nb; }
    }
    return new_node;
}

/* trace_out_raytrace raytrace.f90:58-177 (dir = +z).
 * depth_list is (2, n_depth_rt) = (cell id, step index). */
static int trace_out_raytrace(double x_co, double y_co, int node_num, const double *xyz,
                              const int *del_ne, const int *del_num_ne, double dx, int n_depth_rt,
                              int star_mod, double R_star, const double *XYZ_star, int *from_star,
                              int *depth_list, int *node_count);

int orc_trace_out_raytrace(double x_co, double y_co, int node_num, const double *xyz,
                           const int *del_ne, const int *del_num_ne, int maxne, double dx,
                           int n_depth_rt, int *depth_list, int *node_count)
{
    (void)maxne;
    int from_star = 0;
    return trace_out_raytrace(x_co, y_co, node_num, xyz, del_ne, del_num_ne, dx, n_depth_rt, 0, 0.0, NULL,
                              &from_star, depth_list, node_count);
}

/* trace_out_raytrace raytrace.f90:58-177.  Star mode (:103-115): a start
 * point within R_star of the star's sky position starts at the star's
 * front, z = z_star + R_star, and *from_star tells the caller to start
 * from B(T_star). */
static int trace_out_raytrace(double x_co, double y_co, int node_num, const double *xyz,
                              const int *del_ne, const int *del_num_ne, double dx, int n_depth_rt,
                              int star_mod, double R_star, const double *XYZ_star, int *from_star,
                              int *depth_list, int *node_count)
{
    double z_co = -1.0 * sqrt(1.0 - x_co * x_co - y_co * y_co);
    *from_star = 0;
    if (star_mod == 1) {
        double xc = x_co - XYZ_star[0], yc = y_co - XYZ_star[1];
        double rc = sqrt(xc * xc + yc * yc);
        if (rc < R_star) {
            z_co = XYZ_star[2] + R_star;
            *from_star = 1;
        }
    }
    double start[3] = {x_co, y_co, z_co};
    int k_cur = 0, nc = 0, node = 0;
    double rsave = 10.0;
    for (int i = 1; i <= node_num; i++) {
        const double *X = xyz + 3 * (i - 1);
        double d[3] = {start[0] - X[0], start[1] - X[1], start[2] - X[2]};
        double r = norm2_3(d);
        if (r < rsave) { rsave = r; node = i; }
    }
    if (node == 0) { *node_count = 0; return ORC_ERR_ARG; }
    double X_phot[3] = {start[0], start[1], start[2]};
    const double dir[3] = {0.0, 0.0, 1.0};
    int in_sim = 0;
    while (in_sim == 0) {
        for (int k = 0; k < 3; k++) X_phot[k] = X_phot[k] + dx * dir[k];
        k_cur++;
        if (norm2_3(X_phot) > 1.0) {
            nc++;
            in_sim = 1;
            if (nc > n_depth_rt) { *node_count = nc; return ORC_ERR_DEPTH; }
            depth_list[2 * (nc - 1) + 1] = k_cur;
            depth_list[2 * (nc - 1)] = node;
        }
        int new_node = check_neigh(X_phot, node, xyz, del_ne, del_num_ne, node_num);
        if (new_node != node) {
            nc++;
            if (nc > n_depth_rt) { *node_count = nc; return ORC_ERR_DEPTH; }
            depth_list[2 * (nc - 1) + 1] = k_cur;
            depth_list[2 * (nc - 1)] = new_node;
            node = new_node;
        }
    }
    *node_count = nc;
    return ORC_OK;
}

/* polarize_prop raytrace.f90:1-56 */
void orc_polarize_prop(double eta_I, double eta_Q, double eps_I, double eps_Q, double ds,
                       double *I, double *Q, double *U)
{
    double I0 = *I, Q0 = *Q;
    double shQ = sinh(eta_Q * ds);
    double chQ = cosh(eta_Q * ds);
    double e_tau = exp(-eta_I * ds);
    double fac = pow(eta_I * eta_I - eta_Q * eta_Q, -1.0);
    double o11 = fac * eta_I * (1.0 - (chQ + (eta_Q / eta_I) * shQ) * e_tau);
    double o12 = -fac * eta_Q * (1.0 - (chQ + (eta_I / eta_Q) * shQ) * e_tau);
    *I = o11 * eps_I + o12 * eps_Q + e_tau * (chQ * I0 - shQ * Q0);
    *Q = o12 * eps_I + o11 * eps_Q + e_tau * (-shQ * I0 + chQ * Q0);
    *U = *U * e_tau;
}

/* rot_stokes / rot_stokes_back miscellaneous.f90:463-551 */
static double stokes_alpha(const double *b)
{
    double chi0 = b[0], chi1 = b[1];
    double n = sqrt(chi0 * chi0 + chi1 * chi1);
    chi0 /= n;
    chi1 /= n;
    double alpha = acos(chi1);
    if (chi0 > 0.0) alpha = -alpha;
    return alpha;
}

/* ray_in_raytrace raytrace.f90:179-323 */
void orc_ray_in_raytrace(double vel_obs, int node_count, const int *depth_list,
                         const double *pol_rayt, int nlines, int line, const double *b_all,
                         const double *bvec, const double *dust_p, double alpha, double kd,
                         const double *t_dust, const double *vel_z, double dx, double nu0,
                         double I_in, double *out)
{
    double cnu = F4(2.99792e8) / nu0;
    double I_out = I_in, Q_in = 0.0, U_in = 0.0, Q_out = 0.0, U_out = 0.0, tau = 0.0;
    double tau_dust_tot = 0.0, I_dust = I_in, sig0 = 0.0, sig2 = 0.0, Qd = 0.0, Ud = 0.0;
    const double spi = sqrt(acos(-1.0));
    for (int i = 1; i <= node_count - 1; i++) {
        int cell = depth_list[2 * (i - 1)];
        const double *pr = pol_rayt + (size_t)nlines * 4 * (cell - 1) + line;
        const double *b = bvec + 3 * (cell - 1);
        double bl = b_all[cell - 1];
        double dv = vel_obs - vel_z[cell - 1];
        double v_corr = (1.0 / (bl * spi)) * exp((-(dv * dv)) / (bl * bl));
        double al = stokes_alpha(b);
        Q_out = Q_in * cos(2.0 * al) + U_in * sin(2.0 * al);
        U_out = U_in * cos(2.0 * al) - Q_in * sin(2.0 * al);
        double mu = b[2];
        double mu2 = 1.0 - mu * mu;
        double eta_I = cnu * v_corr * pr[0];
        double eta_Q = cnu * v_corr * pr[nlines];
        double eps_I = cnu * v_corr * pr[2 * nlines];
        double eps_Q = cnu * v_corr * pr[3 * nlines];
        double delta_x = dx * (double)(depth_list[2 * i + 1] - depth_list[2 * (i - 1) + 1]);
        if (delta_x * eta_I > 1e-30) {
            orc_polarize_prop(eta_I, eta_Q, eps_I, eps_Q, delta_x, &I_out, &Q_out, &U_out);
            tau = tau + eta_I * delta_x;
        }
        double tau_dust = kd * dust_p[cell - 1] * delta_x;
        if (tau_dust > 1e-30) {
            double I_bb = orc_black_body(t_dust[cell - 1], nu0);
            double e_dust = exp(-tau_dust);
            double sI = 0.5 * alpha * (mu2 - 2.0 / 3.0);
            double sQ = alpha * mu2;
            I_dust = I_dust * e_dust + I_bb * (1 - e_dust);
            sig0 = sig0 * e_dust + I_bb * (1 - e_dust);
            sig2 = sig2 * e_dust + sI * I_bb * (1 - e_dust);
            double phi = acos(b[1] / sqrt(b[0] * b[0] + b[1] * b[1]));
            if (b[0] < 0.0) phi = -phi;
            Qd = Qd * e_dust + sQ * I_bb * (1 - e_dust) * cos(2.0 * phi);
            Ud = Ud * e_dust + sQ * I_bb * (1 - e_dust) * sin(2.0 * phi);
            tau_dust_tot = tau_dust_tot + tau_dust;
        }
        Q_in = Q_out * cos(2.0 * al) - U_out * sin(2.0 * al);
        U_in = U_out * cos(2.0 * al) + Q_out * sin(2.0 * al);
    }
    double I_corr = orc_black_body(2.73, nu0);
    I_out = I_out - I_corr;
    Q_out = Q_in;
    U_out = U_in;
    I_dust = I_dust - I_corr;
    double Q_dust, U_dust, tau_d;
    if (I_dust == 0.0) {
        Q_dust = 0.0; U_dust = 0.0; tau_d = 0.0;
    } else {
        Q_dust = I_dust * Qd / (sig0 - sig2);
        U_dust = I_dust * Ud / (sig0 - sig2);
        tau_d = tau_dust_tot;
    }
    out[0] = I_out; out[1] = Q_out; out[2] = U_out; out[3] = tau;
    out[4] = I_dust; out[5] = Q_dust; out[6] = U_dust; out[7] = tau_d;
}

/* Both modes of finish_portal.x for one inclination: para_finish.f90:170-185
 * (line data, including the nu0_all whole-array assignment of :173-175),
 * :222-240 (population read-back), then either the pixel mode (:369-376 pixel
 * grid, :382-448 loops; node_mode 0) or the per-node mode (:261-320; node_mode
 * 1: one ray per bulk node from its rotated (x, y), the emission coefficients
 * with t_Aji(l1(j)) as the Einstein A, :303). */
static int image_impl(const orc_cloud *c, const orc_molecule *m, int nlines, const int *l1,
                      const int *l2, const double *pol_pops_in, double th_inc, double ph_az,
                      int nvel, double dvel, double v0, int node_mode, int im_pix, double im_size,
                      double alpha, int n_depth_rt, int pix_lo, int pix_hi, int nthreads,
                      double *xy, double *out, int *status)
{
    int N = c->node_num, nlev = c->nlev;
    int npx = 2 * im_pix + 1, nchan = 2 * nvel + 1;
    int n_rt = node_mode ? c->bulk_node_num : npx * npx;
    double *nu0_all = (double *)malloc(sizeof(double) * nlines);
    double *Aji_all = (double *)calloc(nlines, sizeof(double));
    double *kd_all = (double *)calloc(nlines, sizeof(double));
    for (int i = 0; i < nlines; i++)
        for (int j = 0; j < nlines; j++)
            nu0_all[j] = m->e_levs[l2[i] - 1] - m->e_levs[l1[i] - 1];
    for (int i = 0; i < nlines; i++)
        for (int j = 0; j < m->r_num; j++)
            if (l2[i] == m->r_trans[2 * j + 1] && l1[i] == m->r_trans[2 * j]) {
                Aji_all[i] = m->A[j];
                kd_all[i] = m->kd_v[j];
                break;
            }
    if (node_mode)  /* para_finish.f90:303 passes t_Aji(l1(j)) */
        for (int i = 0; i < nlines; i++) Aji_all[i] = (l1[i] <= m->r_num) ? m->A[l1[i] - 1] : 0.0;
    /* population read-back para_finish.f90:226-239 */
    double *pp = (double *)malloc(sizeof(double) * (size_t)N * 2 * nlev);
    memcpy(pp, pol_pops_in, sizeof(double) * (size_t)N * 2 * nlev);
    for (int node = 0; node < N; node++) {
#define PP(n, col) pp[(size_t)(n) + (size_t)N * (size_t)((col) - 1)]
#define LP(l, n) c->lev_p[(size_t)nlev * (size_t)(n) + (size_t)((l) - 1)]
        PP(node, 1) = LP(1, node) / sqrt(1.0 * (2 * m->j_lev[0] + 1));
        for (int i = 2; i <= nlev; i++) {
            double g = 1.0 * (2 * m->j_lev[i - 1] + 1);
            double rat = PP(node, (i - 1) * 2 + 2) / PP(node, (i - 1) * 2 + 1);
            PP(node, (i - 1) * 2 + 2) = rat * LP(i, node) / sqrt(g);
            PP(node, (i - 1) * 2 + 1) = LP(i, node) / sqrt(g);
        }
    }
    double *vel_inc = (double *)malloc(sizeof(double) * 3 * (size_t)N);
    double *bvec_inc = (double *)malloc(sizeof(double) * 3 * (size_t)N);
    double *xyz_inc = (double *)malloc(sizeof(double) * 3 * (size_t)N);
    orc_rotate_all_save(N, th_inc, ph_az, c->vel, c->bvec, c->xyz, vel_inc, bvec_inc, xyz_inc);
    /* the star's position rotated with the nodes (miscellaneous.f90:899-904) */
    double star_inc[3] = {0.0, 0.0, 0.0};
    if (c->star_mod == 1) {
        double xv[3] = {1, 0, 0}, zv[3] = {0, 0, 1}, Rth[9], Rph[9], R[9];
        rotmat(xv, th_inc, Rth);
        rotmat(zv, ph_az, Rph);
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double sm = 0.0;
                for (int k = 0; k < 3; k++) sm += Rph[i + 3 * k] * Rth[k + 3 * j];
                R[i + 3 * j] = sm;
            }
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++) star_inc[j] = star_inc[j] + R[j + 3 * k] * c->X_star[k];
    }
    double *velz = (double *)malloc(sizeof(double) * (size_t)N);
    for (int n = 0; n < N; n++) velz[n] = vel_inc[3 * n + 2];
    double *pol_rayt = (double *)calloc((size_t)nlines * 4 * N, sizeof(double));
    for (int node = 0; node < c->bulk_node_num; node++) {
        if (PP(node, 1) != 0.0) {
            for (int j = 0; j < nlines; j++) {
                double *pr = pol_rayt + (size_t)nlines * 4 * node + j;
                orc_comp_emcoefs(PP(node, (l1[j] - 1) * 2 + 1), PP(node, (l2[j] - 1) * 2 + 1),
                                 PP(node, (l1[j] - 1) * 2 + 2), PP(node, (l2[j] - 1) * 2 + 2),
                                 m->j_lev[l1[j] - 1], m->j_lev[l2[j] - 1],
                                 acos(bvec_inc[3 * node + 2]), nu0_all[j], Aji_all[j], &pr[0],
                                 &pr[nlines], &pr[2 * nlines], &pr[3 * nlines]);
            }
        }
    }
#undef PP
#undef LP
    if (node_mode && xy)  /* the rows of inc%02d-xy.dat, para_finish.f90:269-271 */
        for (int n = 0; n < n_rt; n++) {
            xy[2 * n] = c->tx * xyz_inc[3 * n];
            xy[2 * n + 1] = c->tx * xyz_inc[3 * n + 1];
        }
    double dx = F4(1e-4);
    int nfail = 0;
    if (pix_lo < 0) pix_lo = 0;
    if (pix_hi > n_rt - 1) pix_hi = n_rt - 1;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel reduction(+ : nfail)
    {
        int *dl = (int *)malloc(sizeof(int) * 2 * (size_t)(n_depth_rt + 2));
#pragma omp for schedule(static)
        for (int p = pix_lo; p <= pix_hi; p++) {
            double x, y;
            if (node_mode) {
                x = xyz_inc[3 * p];
                y = xyz_inc[3 * p + 1];
            } else {
                int i = p / npx - im_pix, j = p % npx - im_pix;
                x = i * im_size / im_pix;
                y = j * im_size / im_pix;
            }
            int nc = 0, from_star = 0;
            int st = trace_out_raytrace(x, y, N, xyz_inc, c->del_ne, c->del_num_ne, dx, n_depth_rt,
                                        c->star_mod, c->R_star, star_inc, &from_star, dl, &nc);
            if (status) status[p] = st;
            if (st != ORC_OK) { nfail++; continue; }
            for (int jl = 0; jl < nlines; jl++) {
                double I_in = orc_black_body(from_star ? c->T_star : 2.73, nu0_all[jl]);
                for (int k = -nvel; k <= nvel; k++) {
                    double o[8];
                    orc_ray_in_raytrace(k * dvel + v0, nc, dl, pol_rayt, nlines, jl, c->b_all,
                                        bvec_inc, c->dust_p, alpha, kd_all[jl], c->t_dust, velz,
                                        c->tx * dx, nu0_all[jl], I_in, o);
                    for (int q = 0; q < 8; q++)
                        out[(((size_t)q * n_rt + p) * nlines + jl) * nchan + (k + nvel)] = o[q];
                }
            }
        }
        free(dl);
    }
    free(nu0_all); free(Aji_all); free(kd_all); free(pp); free(vel_inc); free(bvec_inc);
    free(xyz_inc); free(velz); free(pol_rayt);
    return nfail;
}

int orc_image(const orc_cloud *c, const orc_molecule *m, int nlines, const int *l1,
              const int *l2, const double *pol_pops_in, double th_inc, double ph_az, int nvel,
              double dvel, double v0, int im_pix, double im_size, double alpha, int n_depth_rt,
              int pix_lo, int pix_hi, int nthreads, double *out, int *status)
{
    return image_impl(c, m, nlines, l1, l2, pol_pops_in, th_inc, ph_az, nvel, dvel, v0, 0, im_pix,
                      im_size, alpha, n_depth_rt, pix_lo, pix_hi, nthreads, NULL, out, status);
}

int orc_image_nodes(const orc_cloud *c, const orc_molecule *m, int nlines, const int *l1,
                    const int *l2, const double *pol_pops_in, double th_inc, double ph_az,
                    int nvel, double dvel, double v0, double alpha, int n_depth_rt, int node_lo,
                    int node_hi, int nthreads, double *xy, double *out, int *status)
{
    return image_impl(c, m, nlines, l1, l2, pol_pops_in, th_inc, ph_az, nvel, dvel, v0, 1, 1, 0.0,
                      alpha, n_depth_rt, node_lo, node_hi, nthreads, xy, out, status);
}
