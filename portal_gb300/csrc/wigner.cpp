// Wigner 3j / 6j symbols and the polarized SE coupling constants, host FP64.
//
// PORTAL evaluates these through wigxjpf (fwig3jj / fwig6jj, exact
// multi-word arithmetic) inside the per-node SE assembly (pop_eqs.f90:1-359,
// em_coefs.f90:42-46).  They do not depend on the node, so this library
// evaluates them once per molecule into tables that the device kernels read.
//
// Method: Racah's single-sum formulas with every term kept as a product of
// prime powers.  The alternating sum is carried out exactly in big-integer
// arithmetic over the common prime factor of the terms; only the final
// square root and the scaling by that common factor are rounded, so the
// result carries a few ulps of error regardless of cancellation.
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <vector>

namespace portal {
namespace {

const std::vector<int> &primes() {
    static std::vector<int> p;
    if (p.empty())
        for (int n = 2; n < 400; n++) {
            bool ok = true;
            for (int q : p)
                if (q * q > n) break;
                else if (n % q == 0) { ok = false; break; }
            if (ok) p.push_back(n);
        }
    return p;
}

// exponents of n! over the prime table (Legendre's formula)
void add_fact(std::vector<int> &e, int n, int sign) {
    const auto &P = primes();
    for (size_t i = 0; i < P.size() && P[i] <= n; i++) {
        int c = 0;
        for (long long q = P[i]; q <= n; q *= P[i]) c += (int)(n / q);
        e[i] += sign * c;
    }
}

// unsigned big integer, base 2^32, little endian
struct Big {
    std::vector<uint32_t> d;
    void mul_small(uint32_t m) {
        uint64_t carry = 0;
        for (auto &x : d) {
            uint64_t v = (uint64_t)x * m + carry;
            x = (uint32_t)v;
            carry = v >> 32;
        }
        if (carry) d.push_back((uint32_t)carry);
    }
    int cmp(const Big &o) const {
        if (d.size() != o.d.size()) return d.size() < o.d.size() ? -1 : 1;
        for (size_t i = d.size(); i-- > 0;)
            if (d[i] != o.d[i]) return d[i] < o.d[i] ? -1 : 1;
        return 0;
    }
    void add(const Big &o) {
        uint64_t carry = 0;
        if (d.size() < o.d.size()) d.resize(o.d.size(), 0);
        for (size_t i = 0; i < d.size(); i++) {
            uint64_t v = (uint64_t)d[i] + (i < o.d.size() ? o.d[i] : 0) + carry;
            d[i] = (uint32_t)v;
            carry = v >> 32;
        }
        if (carry) d.push_back((uint32_t)carry);
    }
    void sub(const Big &o) {  // requires *this >= o
        int64_t borrow = 0;
        for (size_t i = 0; i < d.size(); i++) {
            int64_t v = (int64_t)d[i] - (i < o.d.size() ? o.d[i] : 0) - borrow;
            borrow = v < 0;
            if (v < 0) v += (int64_t)1 << 32;
            d[i] = (uint32_t)v;
        }
        while (!d.empty() && d.back() == 0) d.pop_back();
    }
    // value = mant * 2^exp2 with mant in double
    double to_double(int &exp2) const {
        if (d.empty()) { exp2 = 0; return 0.0; }
        size_t n = d.size();
        long double v = 0.0L;
        size_t lo = n > 3 ? n - 3 : 0;
        for (size_t i = n; i-- > lo;) v = v * 4294967296.0L + d[i];
        exp2 = (int)(32 * lo);
        return (double)v;  // rounded once (64-bit mantissa -> 53)
    }
};

struct Signed {
    Big mag;
    bool neg = false;
    void accumulate(const Big &t, bool tneg) {
        if (tneg == neg) { mag.add(t); return; }
        if (mag.cmp(t) >= 0) mag.sub(t);
        else {
            Big r = t;
            r.sub(mag);
            mag = r;
            neg = tneg;
        }
    }
};

// sum_t sign_t * prod p^(e_t) -> value (as double) times prod p^(pre)/2
// (the square-root prefactor).  terms: exponent vectors; signs.
double racah_sum(const std::vector<std::vector<int>> &terms, const std::vector<int> &signs,
                 const std::vector<int> &pre_sq) {
    const auto &P = primes();
    const size_t np = P.size();
    if (terms.empty()) return 0.0;
    std::vector<int> emin(np, 1 << 30);
    for (const auto &e : terms)
        for (size_t i = 0; i < np; i++) emin[i] = std::min(emin[i], e[i]);
    Signed S;
    for (size_t t = 0; t < terms.size(); t++) {
        Big b;
        b.d.push_back(1);
        for (size_t i = 0; i < np; i++)
            for (int k = 0; k < terms[t][i] - emin[i]; k++) b.mul_small((uint32_t)P[i]);
        S.accumulate(b, signs[t] < 0);
    }
    if (S.mag.d.empty()) return 0.0;
    int e2 = 0;
    double m = S.mag.to_double(e2);
    // log of the remaining factor: prod p^emin * sqrt(prod p^pre_sq)
    long double lg = (long double)e2 * logl(2.0L);
    for (size_t i = 0; i < np; i++) {
        long double ex = (long double)emin[i] + 0.5L * pre_sq[i];
        if (ex != 0.0L) lg += ex * logl((long double)P[i]);
    }
    long double v = (long double)m * expl(lg);
    return (double)(S.neg ? -v : v);
}

bool tri(int ta, int tb, int tc) {
    if ((ta + tb + tc) & 1) return false;
    return tc <= ta + tb && tc >= std::abs(ta - tb);
}

void delta_pre(std::vector<int> &pre, int ta, int tb, int tc) {
    add_fact(pre, (ta + tb - tc) / 2, 1);
    add_fact(pre, (ta - tb + tc) / 2, 1);
    add_fact(pre, (-ta + tb + tc) / 2, 1);
    add_fact(pre, (ta + tb + tc) / 2 + 1, -1);
}

}  // namespace

// arguments are doubled angular momenta / projections, like fwig3jj
double wigner3j(int tj1, int tj2, int tj3, int tm1, int tm2, int tm3) {
    if (tm1 + tm2 + tm3 != 0 || !tri(tj1, tj2, tj3)) return 0.0;
    if (std::abs(tm1) > tj1 || std::abs(tm2) > tj2 || std::abs(tm3) > tj3) return 0.0;
    if (((tj1 + tm1) & 1) || ((tj2 + tm2) & 1) || ((tj3 + tm3) & 1)) return 0.0;
    const size_t np = primes().size();
    std::vector<int> pre(np, 0);
    delta_pre(pre, tj1, tj2, tj3);
    add_fact(pre, (tj1 + tm1) / 2, 1);
    add_fact(pre, (tj1 - tm1) / 2, 1);
    add_fact(pre, (tj2 + tm2) / 2, 1);
    add_fact(pre, (tj2 - tm2) / 2, 1);
    add_fact(pre, (tj3 + tm3) / 2, 1);
    add_fact(pre, (tj3 - tm3) / 2, 1);
    int k1 = (tj3 - tj2 + tm1) / 2, k2 = (tj3 - tj1 - tm2) / 2, k3 = (tj1 + tj2 - tj3) / 2;
    int k4 = (tj1 - tm1) / 2, k5 = (tj2 + tm2) / 2;
    int tmin = std::max(0, std::max(-k1, -k2)), tmax = std::min(k3, std::min(k4, k5));
    std::vector<std::vector<int>> terms;
    std::vector<int> signs;
    for (int t = tmin; t <= tmax; t++) {
        std::vector<int> e(np, 0);
        add_fact(e, t, -1);
        add_fact(e, k1 + t, -1);
        add_fact(e, k2 + t, -1);
        add_fact(e, k3 - t, -1);
        add_fact(e, k4 - t, -1);
        add_fact(e, k5 - t, -1);
        terms.push_back(e);
        signs.push_back((t & 1) ? -1 : 1);
    }
    double r = racah_sum(terms, signs, pre);
    int ph = (tj1 - tj2 - tm3) / 2;
    return (ph & 1) ? -r : r;
}

double wigner6j(int tj1, int tj2, int tj3, int tj4, int tj5, int tj6) {
    if (!tri(tj1, tj2, tj3) || !tri(tj1, tj5, tj6) || !tri(tj4, tj2, tj6) || !tri(tj4, tj5, tj3))
        return 0.0;
    const size_t np = primes().size();
    std::vector<int> pre(np, 0);
    delta_pre(pre, tj1, tj2, tj3);
    delta_pre(pre, tj1, tj5, tj6);
    delta_pre(pre, tj4, tj2, tj6);
    delta_pre(pre, tj4, tj5, tj3);
    int a1 = (tj1 + tj2 + tj3) / 2, a2 = (tj1 + tj5 + tj6) / 2;
    int a3 = (tj4 + tj2 + tj6) / 2, a4 = (tj4 + tj5 + tj3) / 2;
    int b1 = (tj1 + tj2 + tj4 + tj5) / 2, b2 = (tj2 + tj3 + tj5 + tj6) / 2;
    int b3 = (tj3 + tj1 + tj6 + tj4) / 2;
    int tmin = std::max(std::max(a1, a2), std::max(a3, a4));
    int tmax = std::min(b1, std::min(b2, b3));
    std::vector<std::vector<int>> terms;
    std::vector<int> signs;
    for (int t = tmin; t <= tmax; t++) {
        std::vector<int> e(np, 0);
        add_fact(e, t + 1, 1);
        add_fact(e, t - a1, -1);
        add_fact(e, t - a2, -1);
        add_fact(e, t - a3, -1);
        add_fact(e, t - a4, -1);
        add_fact(e, b1 - t, -1);
        add_fact(e, b2 - t, -1);
        add_fact(e, b3 - t, -1);
        terms.push_back(e);
        signs.push_back((t & 1) ? -1 : 1);
    }
    return racah_sum(terms, signs, pre);
}

// ---- coupling constants of L&L04 Eqs. 7.20 (pop_eqs.f90:1-359) ----------
namespace {
inline double W3(int a, int b, int c, int d, int e, int f) {
    return wigner3j(2 * a, 2 * b, 2 * c, 2 * d, 2 * e, 2 * f);
}
inline double sgn(int p) { return (std::abs(p) % 2 == 0) ? 1.0 : -1.0; }
}  // namespace

// which: 0 t_A (pop_eqs.f90:1-78), 1 t_S (:80-156), 2 t_E (:158-201, c0 only),
//        3 r_A (:204-281), 4 r_S (:283-359)
void coupling_constants(int which, int j, int k, int j2, int k2, double *c0, double *c2) {
    *c0 = 0.0;
    *c2 = 0.0;
    int dj = j2 - j, dk = k2 - k;
    if (std::abs(dj) > 1) return;
    if (which == 2) {
        if (dk != 0) return;
        *c0 = (2.0 * j2 + 1.0) * sgn(1 + j + j2 + k) *
              wigner6j(2 * j2, 2 * j2, 2 * k, 2 * j, 2 * j, 2);
        return;
    }
    if (!(dk == 0 || std::abs(dk) == 2)) return;
    const double fac1 = std::sqrt(3.0 * (2.0 * k + 1.0) * (2.0 * k2 + 1.0));
    double s0 = 0.0, s2 = 0.0;
    for (int m = -j; m <= j; m++)
        for (int q = -1; q <= 1; q++) {
            double w1, w2, w3, fac = 1.0;
            const double w40 = W3(1, 1, 0, q, -q, 0), w42 = W3(1, 1, 2, q, -q, 0);
            if (which == 0) {           // t_abs
                int ml = q + m;
                w1 = W3(j, j, k, m, -m, 0);
                w2 = W3(j2, j2, k2, ml, -ml, 0);
                w3 = W3(j, j2, 1, -m, ml, -q);
            } else if (which == 1) {    // t_stim
                int mu = m - q;
                w1 = W3(j, j, k, m, -m, 0);
                w2 = W3(j2, j2, k2, mu, -mu, 0);
                w3 = W3(j2, j, 1, -mu, m, -q);
            } else if (which == 3) {    // r_abs
                int mu = m - q;
                fac = (2.0 * j + 1.0) * fac1 * sgn(1 + q);
                w1 = W3(j, j, k, m, -m, 0);
                w2 = W3(j, j, k2, m, -m, 0);
                w3 = W3(j2, j, 1, -mu, m, -q);
            } else {                    // r_stim
                int ml = m + q;
                fac = (2.0 * j + 1.0) * fac1 * sgn(1 - q);
                w1 = W3(j, j, k, m, -m, 0);
                w2 = W3(j, j, k2, m, -m, 0);
                w3 = W3(j, j2, 1, -m, ml, -q);
            }
            double ww = w1 * w2 * w3 * w3;
            if (dk == 0) s0 += fac * ww * w40;
            s2 += fac * ww * w42;
        }
    if (which == 0 || which == 1) {
        const double fac = (2.0 * j2 + 1.0) * fac1 * sgn(1 - dj);
        *c0 = s0 * fac;
        *c2 = s2 * std::sqrt(5.0) * fac;
    } else {
        *c0 = s0;
        *c2 = s2 * std::sqrt(5.0);
    }
}

}  // namespace portal

extern "C" double portal_wigner3j(int tj1, int tj2, int tj3, int tm1, int tm2, int tm3) {
    return portal::wigner3j(tj1, tj2, tj3, tm1, tm2, tm3);
}
extern "C" double portal_wigner6j(int tj1, int tj2, int tj3, int tj4, int tj5, int tj6) {
    return portal::wigner6j(tj1, tj2, tj3, tj4, tj5, tj6);
}
extern "C" void portal_coupling_constant(int which, int j, int k, int j2, int k2, double *c0,
                                         double *c2) {
    portal::coupling_constants(which, j, k, j2, k2, c0, c2);
}
