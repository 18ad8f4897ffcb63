// Readers and writers of PORTAL's files.  Each reader mirrors the read
// statements of the reference routine named beside it.
#include "portal_io.h"

#include <algorithm>
#include <cctype>
#include <charconv>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <sys/stat.h>
#include <fstream>
#include <random>
#include <sstream>
#include <thread>
#include <type_traits>

namespace portal_io {

static double f4(double x) { return (double)(float)x; }  // REAL*4 literal promoted to FP64

// ---------------------------------------------------------------------------
// list-directed input
// ---------------------------------------------------------------------------

ListReader::ListReader(const std::string &path) : path_(path) {
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) return;
    fseek(f, 0, SEEK_END);
    const long sz = ftell(f);
    fseek(f, 0, SEEK_SET);
    buf_.resize(sz > 0 ? (size_t)sz : 0);
    const size_t got = sz > 0 ? fread(&buf_[0], 1, (size_t)sz, f) : 0;
    fclose(f);
    buf_.resize(got);
    size_t b = 0;
    while (b < buf_.size()) {
        const void *nl = memchr(buf_.data() + b, '\n', buf_.size() - b);
        size_t e = nl ? (size_t)((const char *)nl - buf_.data()) : buf_.size();
        size_t ee = e;
        if (ee > b && buf_[ee - 1] == '\r') ee--;
        lbeg_.push_back(b);
        lend_.push_back(ee);
        b = e + 1;
    }
    ok_ = true;
}

int io_threads() {
    if (const char *e = getenv("PORTAL_THREADS")) {
        const int t = atoi(e);
        if (t > 0) return t;
    }
    const unsigned h = std::thread::hardware_concurrency();
    return h ? (int)std::min(h, 64u) : 1;
}

static void tokenize(const char *line, size_t len, std::vector<std::string> &toks) {
    toks.clear();
    std::string cur;
    auto flush = [&]() {
        if (cur.empty()) return;
        // r*c repeat count
        size_t star = cur.find('*');
        if (star != std::string::npos && star > 0 &&
            std::all_of(cur.begin(), cur.begin() + star, [](char ch) { return ch >= '0' && ch <= '9'; })) {
            int r = atoi(cur.substr(0, star).c_str());
            std::string v = cur.substr(star + 1);
            for (int i = 0; i < r; i++) toks.push_back(v);
        } else {
            toks.push_back(cur);
        }
        cur.clear();
    };
    bool quote = false;
    char qc = 0;
    for (size_t i = 0; i < len; i++) {
        const char ch = line[i];
        if (quote) {
            if (ch == qc) { quote = false; flush(); }
            else cur.push_back(ch);
            continue;
        }
        if (ch == '\'' || ch == '"') { flush(); quote = true; qc = ch; continue; }
        if (ch == '/') { flush(); toks.push_back("/"); break; }  // value separator that ends the list
        if (ch == ' ' || ch == '\t' || ch == ',') { flush(); continue; }
        cur.push_back(ch);
    }
    flush();
}

bool ListReader::next_record() {
    if (line_ >= lbeg_.size()) return false;
    tokenize(buf_.data() + lbeg_[line_], lend_[line_] - lbeg_[line_], toks_);
    line_++;
    pos_ = 0;
    return true;
}

namespace {

inline bool is_sep(char ch) { return ch == ' ' || ch == '\t' || ch == ','; }

// One line of exactly n plain numbers (no repeat counts, quotes, slashes or
// D exponents: those take the general path) into out; false otherwise.
template <typename T>
bool parse_plain_line(const char *p, const char *end, size_t n, T *out) {
    size_t k = 0;
    char tmp[64];
    while (true) {
        while (p < end && is_sep(*p)) p++;
        if (p >= end) break;
        const char *q = p;
        while (q < end && !is_sep(*q)) {
            const char ch = *q;
            if (ch == '*' || ch == '/' || ch == '\'' || ch == '"' || ch == 'd' || ch == 'D') return false;
            q++;
        }
        if (k >= n || (size_t)(q - p) >= sizeof tmp) return false;
        memcpy(tmp, p, (size_t)(q - p));
        tmp[q - p] = 0;
        char *ep = nullptr;
        if (std::is_floating_point<T>::value) {
            out[k] = (T)strtod(tmp, &ep);
        } else {
            out[k] = (T)strtol(tmp, &ep, 10);
        }
        if (ep != tmp + (q - p)) return false;  // the general path's token conversion would differ
        k++;
        p = q;
    }
    return k == n;
}

}  // namespace

template <typename T>
size_t ListReader::read_block(T *out, size_t n_rec, size_t n, int threads) {
    const size_t avail = lbeg_.size() > line_ ? lbeg_.size() - line_ : 0;
    const size_t m = std::min(n_rec, avail);
    bool fast = m > 0;
    if (fast) {
        const int nt = (int)std::max<size_t>(1, std::min<size_t>((size_t)std::max(threads, 1), m / 4096 + 1));
        std::vector<char> okv(nt, 1);
        std::vector<std::thread> th;
        auto work = [&](int t) {
            const size_t r0 = m * t / nt, r1 = m * (t + 1) / nt;
            for (size_t r = r0; r < r1; r++) {
                const size_t L = line_ + r;
                if (!parse_plain_line<T>(buf_.data() + lbeg_[L], buf_.data() + lend_[L], n, out + r * n)) {
                    okv[t] = 0;
                    return;
                }
            }
        };
        for (int t = 1; t < nt; t++) th.emplace_back(work, t);
        work(0);
        for (auto &x : th) x.join();
        for (char v : okv) fast = fast && v;
    }
    if (fast) {
        line_ += m;
        return m;
    }
    // the general list-directed path, record by record
    std::vector<std::string> t;
    size_t r = 0;
    for (; r < n_rec; r++) {
        if (!read(t, n)) break;
        for (size_t k = 0; k < n; k++)
            out[r * n + k] = std::is_floating_point<T>::value ? (T)to_double(t[k]) : (T)to_int(t[k]);
    }
    return r;
}

size_t ListReader::read_block_doubles(double *out, size_t n_rec, size_t n, int threads) {
    return read_block<double>(out, n_rec, n, threads);
}
size_t ListReader::read_block_ints(int *out, size_t n_rec, size_t n, int threads) {
    return read_block<int>(out, n_rec, n, threads);
}

bool ListReader::skip() { return next_record(); }

bool ListReader::read(std::vector<std::string> &out, size_t n) {
    out.clear();
    if (!next_record()) return false;
    while (out.size() < n) {
        if (pos_ >= toks_.size()) {
            if (!next_record()) return false;
            continue;
        }
        if (toks_[pos_] == "/") return false;  // the reference would leave the rest unset
        out.push_back(toks_[pos_++]);
    }
    return true;
}

// Fortran's list-directed READ stops the program on an item that is not a
// number; the readers here fail the same way: to_double / to_int remember
// the first token they cannot read whole, and every reader checks it.
namespace {
thread_local std::string g_bad;
}

double to_double(const std::string &tok) {
    std::string t = tok;
    for (auto &ch : t)
        if (ch == 'd' || ch == 'D') ch = 'e';
    char *ep = nullptr;
    double v = strtod(t.c_str(), &ep);
    if (ep == t.c_str() || *ep != 0) {
        // numeric input also takes an exponent given by its sign alone (1.5+3 = 1.5e3)
        const size_t s = t.find_last_of("+-");
        if (s != std::string::npos && s > 0 && (isdigit((unsigned char)t[s - 1]) || t[s - 1] == '.')) {
            const std::string u = t.substr(0, s) + "e" + t.substr(s);
            char *eu = nullptr;
            const double w = strtod(u.c_str(), &eu);
            if (eu != u.c_str() && *eu == 0) return w;
        }
        if (g_bad.empty()) g_bad = tok;
    }
    return v;
}

int to_int(const std::string &tok) {
    char *ep = nullptr;
    const long v = strtol(tok.c_str(), &ep, 10);
    if ((ep == tok.c_str() || *ep != 0) && g_bad.empty()) g_bad = tok;
    return (int)v;
}

// false (with the message) when a token of `path` was not a number
static bool numbers_ok(const std::string &path, std::string &err) {
    if (g_bad.empty()) return true;
    err = path + ": not a number: '" + g_bad + "'";
    g_bad.clear();
    return false;
}

bool ListReader::read_doubles(std::vector<double> &out, size_t n) {
    std::vector<std::string> t;
    if (!read(t, n)) return false;
    out.resize(n);
    for (size_t i = 0; i < n; i++) out[i] = to_double(t[i]);
    return true;
}

bool ListReader::read_ints(std::vector<int> &out, size_t n) {
    std::vector<std::string> t;
    if (!read(t, n)) return false;
    out.resize(n);
    for (size_t i = 0; i < n; i++) out[i] = to_int(t[i]);
    return true;
}

// ---------------------------------------------------------------------------
// input files
// ---------------------------------------------------------------------------

bool read_main_input(const std::string &path, MainInput &in, std::string &err) {
    g_bad.clear();
    ListReader r(path);
    if (!r.ok()) { err = "cannot open " + path; return false; }
    std::vector<std::string> t;
    // main_para.f90:74-79 (the line holding dust_ii_gas is read as x1, and
    // x2, x3, x_dip then continue on the field line, as list-directed input does)
    if (!r.skip() || !r.read(t, 6)) { err = path + ": star line"; return false; }
    in.star_mod = to_int(t[0]); in.T_star = to_double(t[1]); in.R_star = to_double(t[2]);
    for (int k = 0; k < 3; k++) in.XYZ_star[k] = to_double(t[3 + k]);
    if (!r.read(t, 3)) { err = path + ": nth nph nvel"; return false; }
    in.nth = to_int(t[0]); in.nph = to_int(t[1]); in.nvel = to_int(t[2]);
    if (!r.read(t, 4)) { err = path + ": field line"; return false; }
    in.x1 = to_double(t[0]); in.x2 = to_double(t[1]); in.x3 = to_double(t[2]); in.x_dip = to_double(t[3]);
    if (!r.read(t, 2)) { err = path + ": kmax extra_info"; return false; }
    in.kmax = to_int(t[0]); in.extra_info = to_int(t[1]);
    if (!r.read(t, 2)) { err = path + ": max_ne_temp n_depth"; return false; }
    in.max_ne_temp = to_int(t[0]); in.n_depth = to_int(t[1]);
    return numbers_ok(path, err);
}

bool read_finish_input(const std::string &path, FinishInput &in, std::string &err) {
    g_bad.clear();
    ListReader r(path);
    if (!r.ok()) { err = "cannot open " + path; return false; }
    std::vector<std::string> t;
    std::vector<int> vi;
    std::vector<double> vd;
    // para_finish.f90:89-121
    if (!r.skip() || !r.read(t, 1)) { err = path + ": nlevels"; return false; }
    in.nlevels = to_int(t[0]);
    if (in.nlevels < 1) { err = path + ": nlevels < 1"; return false; }
    if (!r.read_ints(in.l1, in.nlevels) || !r.read_ints(in.l2, in.nlevels)) { err = path + ": l1/l2"; return false; }
    if (!r.skip() || !r.read(t, 1)) { err = path + ": nincs"; return false; }
    in.nincs = to_int(t[0]);
    if (in.nincs < 1) { err = path + ": nincs < 1"; return false; }
    if (!r.read_doubles(in.th_inc, in.nincs) || !r.read_doubles(in.ph_az, in.nincs)) { err = path + ": angles"; return false; }
    if (!r.skip() || !r.read(t, 3)) { err = path + ": nvel dvel v0"; return false; }
    in.nvel = to_int(t[0]); in.dvel = to_double(t[1]); in.v0 = to_double(t[2]);
    if (!r.skip() || !r.read(t, 6)) { err = path + ": star line"; return false; }
    in.star_mod = to_int(t[0]); in.T_star = to_double(t[1]); in.R_star = to_double(t[2]);
    for (int k = 0; k < 3; k++) in.XYZ_star[k] = to_double(t[3 + k]);
    if (!r.read(t, 4)) { err = path + ": field line"; return false; }
    in.x1 = to_double(t[0]); in.x2 = to_double(t[1]); in.x3 = to_double(t[2]); in.x_dip = to_double(t[3]);
    if (!r.read(t, 2)) { err = path + ": kmax extra_info"; return false; }
    in.kmax = to_int(t[0]); in.extra_info = to_int(t[1]);
    if (!r.read(t, 3)) { err = path + ": pix im_pix im_size"; return false; }
    in.pix = to_int(t[0]); in.im_pix = to_int(t[1]); in.im_size = to_double(t[2]);
    if (!r.read(t, 2)) { err = path + ": fits distance"; return false; }
    in.fits = to_int(t[0]); in.distance = to_double(t[1]);
    if (!r.read(t, 2)) { err = path + ": max_ne_temp n_depth_rt"; return false; }
    in.max_ne_temp = to_int(t[0]); in.n_depth_rt = to_int(t[1]);
    return numbers_ok(path, err);
}

// ---------------------------------------------------------------------------
// LIME / LAMDA / dust
// ---------------------------------------------------------------------------

// adj_list_no_delaunay miscellaneous.f90:910-1015 on the host: each
// tetrahedron gives its vertices the other three; SortUnique then sorts and
// de-duplicates.  Built as a CSR: incidence counts, offsets, the raw lists
// (filled in tetrahedron order per thread range, so the per-node lists are
// the same multiset whatever the thread count), then a per-node sort +
// unique.  cells: nc records of (4, v0..v3), 0-based vertices.
static bool host_neighbours(int N, const std::vector<int> &cells, size_t nc, int max_ne_temp, int nth, Cloud &c,
                            std::string &err) {
    std::vector<long long> roff((size_t)N + 1, 0);
    for (size_t q = 0; q < nc; q++)
        for (int k = 0; k < 4; k++) roff[(size_t)cells[5 * q + 1 + k] + 1] += 3;
    for (int i = 0; i < N; i++) roff[i + 1] += roff[i];
    for (int i = 0; i < N; i++)
        if (roff[i + 1] - roff[i] > max_ne_temp) {  // miscellaneous.f90:1000-1004
            err = "count_ne=" + std::to_string(roff[i + 1] - roff[i]) + " while max_ne_temp=" +
                  std::to_string(max_ne_temp) + "; adjust max_ne_temp parameter! Make it bigger.";
            return false;
        }
    std::vector<int> raw((size_t)roff[N]);
    {
        std::vector<long long> fill(roff.begin(), roff.end() - 1);
        for (size_t q = 0; q < nc; q++)
            for (int k = 0; k < 4; k++) {
                const int a = cells[5 * q + 1 + k];
                for (int k2 = 0; k2 < 4; k2++)
                    if (k2 != k) raw[(size_t)fill[a]++] = cells[5 * q + 1 + k2] + 1;
            }
    }
    c.del_num_ne.assign(N, 0);
    {
        std::vector<std::thread> th;
        auto work = [&](int t) {
            const int i0 = (int)((long long)N * t / nth), i1 = (int)((long long)N * (t + 1) / nth);
            for (int i = i0; i < i1; i++) {
                int *b = raw.data() + roff[i], *e = raw.data() + roff[i + 1];
                std::sort(b, e);
                c.del_num_ne[i] = (int)(std::unique(b, e) - b);
            }
        };
        for (int t = 1; t < nth; t++) th.emplace_back(work, t);
        work(0);
        for (auto &x : th) x.join();
    }
    int maxne = 0;
    for (int i = 0; i < N; i++) maxne = std::max(maxne, c.del_num_ne[i]);
    c.maxne = maxne;
    c.del_ne.assign((size_t)N * maxne, 0);  // main_para.f90:124-128
    for (int i = 0; i < N; i++)
        for (int s2 = 0; s2 < c.del_num_ne[i]; s2++) c.del_ne[(size_t)i + (size_t)N * s2] = raw[(size_t)roff[i] + s2];
    return true;
}

bool read_lime(const std::string &pop, const std::string &grid, const std::string &mol,
               const std::string &dust, double dust_ii_gas, int max_ne_temp, Molecule &m, Cloud &c,
               std::string &err, const NeighbourBuilder *build_neighbours) {
    (void)dust_ii_gas;  // the per-node gas-to-dust column of the .pop is what eat_lime uses
    std::vector<std::string> t;
    std::vector<double> vd;
    g_bad.clear();
    // ---- grid.vtk: points (eat_lime_dim eat_lime.f90:21-34, :124-136) ----
    ListReader g(grid);
    if (!g.ok()) { err = "cannot open " + grid; return false; }
    for (int k = 0; k < 4; k++) g.skip();
    if (!g.read(t, 2)) { err = grid + ": POINTS line"; return false; }
    const int N = to_int(t[1]);
    if (N < 1) { err = grid + ": no points"; return false; }
    c.node_num = N;
    c.xyz.resize(3 * (size_t)N);
    const int nth = io_threads();
    const size_t np = g.read_block_doubles(c.xyz.data(), (size_t)N, 3, nth);
    if (np < (size_t)N) { err = grid + ": point " + std::to_string(np + 1); return false; }
    g.skip();
    if (!g.read(t, 2)) { err = grid + ": CELLS line"; return false; }
    const int ntet = to_int(t[1]);
    std::vector<int> cells(5 * (size_t)std::max(ntet, 0));
    const size_t nc = g.read_block_ints(cells.data(), (size_t)std::max(ntet, 0), 5, nth);
    if (nc < (size_t)std::max(ntet, 0)) { err = grid + ": cell " + std::to_string(nc + 1); return false; }
    for (size_t q = 0; q < nc; q++)
        for (int k = 0; k < 4; k++) {
            const int v = cells[5 * q + 1 + k] + 1;
            if (v < 1 || v > N) { err = grid + ": cell vertex out of range"; return false; }
        }
    if (build_neighbours) {
        std::vector<int> tets(4 * nc);
        for (size_t q = 0; q < nc; q++)
            for (int k = 0; k < 4; k++) tets[4 * q + k] = cells[5 * q + 1 + k];
        if (!(*build_neighbours)(N, tets, max_ne_temp, c, err)) return false;
    } else if (!host_neighbours(N, cells, nc, max_ne_temp, nth, c, err)) {
        return false;
    }

    if (!numbers_ok(grid, err)) return false;
    // ---- LAMDA (eat_lime_dim :38-62, eat_lime_no_delaunay :151-196) ----
    ListReader f(mol);
    if (!f.ok()) { err = "cannot open " + mol; return false; }
    for (int k = 0; k < 3; k++) f.skip();
    if (!f.read_doubles(vd, 1)) { err = mol + ": molecular weight"; return false; }
    m.mass = vd[0];
    f.skip();
    if (!f.read(t, 1)) { err = mol + ": number of levels"; return false; }
    m.nlev = to_int(t[0]);
    f.skip();
    m.e_levs.resize(m.nlev);
    m.j_lev.resize(m.nlev);
    for (int i = 0; i < m.nlev; i++) {
        if (!f.read(t, 3)) { err = mol + ": level " + std::to_string(i + 1); return false; }
        m.e_levs[i] = to_double(t[1]);
        const double g1 = to_double(t[2]);
        m.j_lev[i] = (int)std::lround((g1 - 1.0) / 2.0);  // nint
    }
    f.skip();
    if (!f.read(t, 1)) { err = mol + ": number of radiative transitions"; return false; }
    m.r_num = to_int(t[0]);
    f.skip();
    m.r_trans.resize(2 * (size_t)m.r_num);
    m.A.resize(m.r_num);
    m.nu.resize(m.r_num);
    for (int i = 0; i < m.r_num; i++) {
        if (!f.read(t, 5)) { err = mol + ": radiative transition " + std::to_string(i + 1); return false; }
        m.r_trans[2 * i + 1] = to_int(t[1]);  // upper
        m.r_trans[2 * i] = to_int(t[2]);      // lower
        m.A[i] = to_double(t[3]);
        m.nu[i] = to_double(t[4]);
    }
    f.skip();
    if (!f.read(t, 1)) { err = mol + ": number of collision partners"; return false; }
    m.c_par = to_int(t[0]);
    if (m.c_par < 1 || m.c_par > 2) { err = mol + ": 1 or 2 collision partners"; return false; }
    for (int k = 0; k < 3; k++) f.skip();
    if (!f.read(t, 1)) { err = mol + ": number of collisional transitions"; return false; }
    m.c_num = to_int(t[0]);
    f.skip();
    if (!f.read(t, 1)) { err = mol + ": number of collision temperatures"; return false; }
    m.c_temp = to_int(t[0]);
    f.skip();
    if (!f.read_doubles(m.col_temps, m.c_temp)) { err = mol + ": collision temperatures"; return false; }
    f.skip();
    m.c_trans.resize(2 * (size_t)m.c_num);
    m.C.assign((size_t)m.c_temp * m.c_num * m.c_par, 0.0);
    for (int i = 0; i < m.c_num; i++) {
        if (!f.read(t, 3 + (size_t)m.c_temp)) { err = mol + ": collisional transition " + std::to_string(i + 1); return false; }
        m.c_trans[2 * i + 1] = to_int(t[1]);
        m.c_trans[2 * i] = to_int(t[2]);
        for (int k = 0; k < m.c_temp; k++) m.C[(size_t)k + (size_t)m.c_temp * i] = to_double(t[3 + k]);
    }
    if (m.c_par == 2) {
        // eat_lime.f90:184-195: five records skipped, then the partner's
        // temperature count is read as its transition count
        for (int k = 0; k < 5; k++) f.skip();
        if (!f.read(t, 1)) { err = mol + ": second partner"; return false; }
        const int c2 = to_int(t[0]);
        for (int k = 0; k < 3; k++) f.skip();
        for (int i = 0; i < c2 && i < m.c_num; i++) {
            if (!f.read(t, 3 + (size_t)m.c_temp)) { err = mol + ": second partner rates"; return false; }
            for (int k = 0; k < m.c_temp; k++)
                m.C[(size_t)k + (size_t)m.c_temp * (i + (size_t)m.c_num)] = to_double(t[3 + k]);
        }
    }
    if (!numbers_ok(mol, err)) return false;
    // ---- .pop rows (eat_lime.f90:207-224) ----
    ListReader p(pop);
    if (!p.ok()) { err = "cannot open " + pop; return false; }
    p.skip();
    const int nl = m.nlev;
    c.nlev = nl;
    c.vel.assign(3 * (size_t)N, 0.0);
    c.h2_dens.assign(N, 1.0);
    c.temp_all.assign(2 * (size_t)N, 0.0);
    c.b_all.assign(N, 200.0);
    c.ab_all.assign(N, 1e-3);
    c.lev_p.assign((size_t)nl * N, 0.0);
    std::vector<double> g2d(N, 0.0);
    const size_t nv = 13 + (size_t)nl;
    std::vector<double> rows((size_t)N * nv);
    const int bulk = (int)p.read_block_doubles(rows.data(), (size_t)N, nv, nth);
    for (int i = 0; i < bulk; i++) {
        const double *r = rows.data() + (size_t)i * nv;
        for (int k = 0; k < 3; k++) c.vel[3 * (size_t)i + k] = r[3 + k];
        c.h2_dens[i] = r[6];
        c.temp_all[2 * (size_t)i] = r[7];
        c.temp_all[2 * (size_t)i + 1] = r[8];
        c.b_all[i] = r[9];
        c.ab_all[i] = r[10];
        g2d[i] = r[11];
        for (int l = 0; l < nl; l++) c.lev_p[(size_t)nl * i + l] = r[13 + l];
    }
    c.bulk_node_num = bulk;
    // surface nodes (eat_lime.f90:227-245)
    for (int j = bulk; j < N; j++) {
        double sp = 1.0;
        c.lev_p[(size_t)nl * j] = 1.0;
        for (int k = 1; k < nl; k++) {
            c.lev_p[(size_t)nl * j + k] = 1.0 * std::exp(-m.e_levs[k] * 0.527);
            sp += c.lev_p[(size_t)nl * j + k];
        }
        for (int k = 0; k < nl; k++) c.lev_p[(size_t)nl * j + k] /= sp;
    }
    for (int j = 0; j < N; j++) {  // :250-263
        const double b_therm = 2.0 * 8314.462 * c.temp_all[2 * (size_t)j] / m.mass;
        c.b_all[j] = std::sqrt(c.b_all[j] * c.b_all[j] + b_therm);
        for (int l = 0; l < nl; l++) c.lev_p[(size_t)nl * j + l] *= c.ab_all[j] * c.h2_dens[j];
    }
    double rmax = 0.0;  // :269-279
    for (int i = 0; i < N; i++) {
        const double *x = &c.xyz[3 * (size_t)i];
        rmax = std::max(rmax, std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]));
    }
    for (auto &v : c.xyz) v /= rmax;
    c.tx = rmax;
    if (!numbers_ok(pop, err)) return false;
    // ---- dust table (eat_lime.f90:285-298, dust_to_opacities miscellaneous.f90:643-700) ----
    ListReader d(dust);
    if (!d.ok()) { err = "cannot open " + dust; return false; }
    const int n_dt = 67;
    std::vector<double> lt(n_dt), lk(n_dt);
    for (int i = 0; i < n_dt; i++) {
        if (!d.read_doubles(vd, 2)) { err = dust + ": row " + std::to_string(i + 1); return false; }
        lt[i] = std::log10(vd[0]);
        lk[i] = std::log10(vd[1]);
    }
    m.kd_v.resize(m.r_num);
    for (int i = 0; i < m.r_num; i++) {
        const double nu_hz = m.nu[i] * f4(1e9);
        const double mu0 = std::log10(f4(2.998e14) / nu_hz);
        double kd_m = 0.0;
        for (int j = 0; j < n_dt - 1; j++)
            if (mu0 > lt[j] && mu0 < lt[j + 1]) {
                const double res = (mu0 - lt[j]) / (lt[j + 1] - lt[j]);
                kd_m = lk[j] + res * (lk[j + 1] - lk[j]);
                break;
            }
        if (mu0 > lt[n_dt - 1]) {
            const double res = (mu0 - lt[n_dt - 1]) / (lt[n_dt - 1] - lt[n_dt - 2]);
            kd_m = lk[n_dt - 1] + res * (lk[n_dt - 1] - lk[n_dt - 2]);
        }
        m.kd_v[i] = std::pow(10.0, kd_m) * f4(1e-1);
    }
    c.dust_p.assign(N, 0.0);  // :302-311
    for (int i = 0; i < N; i++)
        if (g2d[i] != 0.0) c.dust_p[i] = c.h2_dens[i] * f4(2.32e-27) / g2d[i];
    if (!numbers_ok(dust, err)) return false;
    // ---- main_para.f90:119-120, :178-185 ----
    for (auto &v : m.nu) v = f4(1e9) * v;
    for (auto &v : m.e_levs) v = f4(29.9792458e9) * v;
    m.Bij.resize(m.r_num);
    for (int i = 0; i < m.r_num; i++) {
        const double g1 = 2.0 * m.j_lev[m.r_trans[2 * i] - 1] + 1.0;
        const double g2 = 2.0 * m.j_lev[m.r_trans[2 * i + 1] - 1] + 1.0;
        m.Bij[i] = (g2 / g1) * m.A[i] * 1.6179542e57 / std::pow(m.nu[i], 3.0);
    }
    return true;
}

void magfield(const Cloud &c, double x1, double x2, double x3, double x_dip, std::vector<double> &bvec) {
    const int N = c.node_num;
    bvec.assign(3 * (size_t)N, 0.0);
    auto nrm = [](const double *v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); };
    for (int i = 0; i < N; i++) {
        const double *x = &c.xyz[3 * (size_t)i];
        double b[3];
        if (x_dip != 0.0) {  // dipole_magfield miscellaneous.f90:553-595
            double xv[3] = {x[0], x[1], x[2]};
            const double n = nrm(xv);
            for (auto &v : xv) v /= n;
            b[0] = 3.0 * xv[0] * xv[2];
            b[1] = 3.0 * xv[1] * xv[2];
            b[2] = 3.0 * xv[2] * xv[2] - 1.0;
        } else {  // global_magfield :597-641
            double rad[3] = {x[0], x[1], x[2]}, tor[3] = {x[1], -x[0], 0.0};
            double pol[3] = {x[2] * x[0], x[1] * x[2], -(x[1] * x[1] + x[0] * x[0])};
            const double nr = nrm(rad), nt = nrm(tor), np = nrm(pol);
            for (int k = 0; k < 3; k++) b[k] = x1 * rad[k] / nr + x2 * tor[k] / nt + x3 * pol[k] / np;
        }
        const double nb = nrm(b);
        for (int k = 0; k < 3; k++) bvec[3 * (size_t)i + k] = b[k] / nb;
    }
}

void gauge_vector(unsigned long long seed, double g[3]) {
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> u(0.0, 1.0);
    for (int k = 0; k < 3; k++) g[k] = u(rng);
    const double n = std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
    for (int k = 0; k < 3; k++) g[k] /= n;
}

// One value as printf's " %24.17E": std::to_chars in scientific notation
// with 17 digits is correctly rounded like glibc's printf, so the digits are
// the same; the exponent letter and inf / nan are upper-cased and the field
// right-aligned to 24 characters.  Returns the characters written (<= 40).
static size_t format_e17(char *p, double v) {
    char b[40];
    const auto r = std::to_chars(b, b + sizeof b, v, std::chars_format::scientific, 17);
    const size_t n = (size_t)(r.ptr - b);
    for (size_t i = 0; i < n; i++)
        if (b[i] >= 'a' && b[i] <= 'z') b[i] = (char)(b[i] - 'a' + 'A');
    const size_t pad = n < 24 ? 24 - n : 0;
    p[0] = ' ';
    memset(p + 1, ' ', pad);
    memcpy(p + 1 + pad, b, n);
    return 1 + pad + n;
}

bool write_rows(const std::string &path, const std::vector<double> &cm, int rows, int cols) {
    FILE *f = fopen(path.c_str(), "w");
    if (!f) return false;
    // rows formatted by all host threads into per-thread buffers, written in order
    const int nth = std::max(1, std::min(io_threads(), rows / 4096 + 1));
    std::vector<std::string> buf((size_t)nth);
    auto work = [&](int t) {
        const int r0 = (int)((long long)rows * t / nth), r1 = (int)((long long)rows * (t + 1) / nth);
        std::string &s = buf[(size_t)t];
        s.resize((size_t)(r1 - r0) * ((size_t)cols * 40 + 1));
        char *p = &s[0];
        for (int r = r0; r < r1; r++) {
            for (int k = 0; k < cols; k++) p += format_e17(p, cm[(size_t)r + (size_t)rows * k]);
            *p++ = '\n';
        }
        s.resize((size_t)(p - &s[0]));
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nth; t++) th.emplace_back(work, t);
    work(0);
    for (auto &x : th) x.join();
    bool ok = true;
    for (const auto &s : buf) ok = ok && fwrite(s.data(), 1, s.size(), f) == s.size();
    return (fclose(f) == 0) && ok;
}

bool read_rows(const std::string &path, std::vector<double> &cm, int rows, int cols, std::string &err) {
    g_bad.clear();
    ListReader r(path);
    if (!r.ok()) { err = "cannot open " + path; return false; }
    cm.assign((size_t)rows * cols, 0.0);
    std::vector<double> v((size_t)rows * cols);
    const size_t got = r.read_block_doubles(v.data(), (size_t)rows, (size_t)cols, io_threads());
    if (got < (size_t)rows) { err = path + ": row " + std::to_string(got + 1); return false; }
    if (!numbers_ok(path, err)) return false;
    for (int i = 0; i < rows; i++)  // para_finish.f90:226-227
        for (int k = 0; k < cols; k++) cm[(size_t)i + (size_t)rows * k] = v[(size_t)i * cols + k];
    return true;
}

bool write_sidecar(const std::string &path, const std::vector<double> &cm, int rows, int cols) {
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) return false;
    const int32_t shape[2] = {rows, cols};
    bool ok = fwrite("PORTALPP", 1, 8, f) == 8 && fwrite(shape, 4, 2, f) == 2 &&
              fwrite(cm.data(), 8, (size_t)rows * cols, f) == (size_t)rows * cols;
    return (fclose(f) == 0) && ok;
}

bool read_sidecar(const std::string &path, const std::string &text_path, std::vector<double> &cm, int rows,
                  int cols) {
    struct stat sb, st;
    if (stat(path.c_str(), &sb) != 0) return false;
    if (stat(text_path.c_str(), &st) == 0 &&
        (sb.st_mtim.tv_sec < st.st_mtim.tv_sec ||
         (sb.st_mtim.tv_sec == st.st_mtim.tv_sec && sb.st_mtim.tv_nsec < st.st_mtim.tv_nsec)))
        return false;  // the text file was written after the sidecar: it wins
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) return false;
    char magic[8];
    int32_t shape[2];
    std::vector<double> v((size_t)rows * cols);
    const bool ok = fread(magic, 1, 8, f) == 8 && memcmp(magic, "PORTALPP", 8) == 0 && fread(shape, 4, 2, f) == 2 &&
                    shape[0] == rows && shape[1] == cols && fread(v.data(), 8, v.size(), f) == v.size();
    fclose(f);
    if (ok) cm.swap(v);
    return ok;
}

// ---------------------------------------------------------------------------
// FITS
// ---------------------------------------------------------------------------

static std::string card_log(const char *k, bool v) {
    char b[81];
    snprintf(b, sizeof b, "%-8s= %20s", k, v ? "T" : "F");
    return b;
}
static std::string card_int(const char *k, long v) {
    char b[81];
    snprintf(b, sizeof b, "%-8s= %20ld", k, v);
    return b;
}
static std::string card_e(const char *k, float v) {  // ftpkye with 8 decimals
    char b[81];
    snprintf(b, sizeof b, "%-8s= %20.8E", k, (double)v);
    return b;
}
static std::string card_s(const char *k, const char *v) {
    char q[72];
    snprintf(q, sizeof q, "'%-8s'", v);
    char b[81];
    snprintf(b, sizeof b, "%-8s= %-20s", k, q);
    return b;
}

bool write_fits(const std::string &path, const float *a, int npix, int nvel, float restfreq, float cdelt1,
                float crpix1, float cdelt2, float crpix2, float cdelt3, float crpix3, float crval1,
                float crval2, float crval3) {
    std::vector<std::string> cards = {
        card_log("SIMPLE", true), card_int("BITPIX", -32), card_int("NAXIS", 3),
        card_int("NAXIS1", npix), card_int("NAXIS2", npix), card_int("NAXIS3", nvel),
        card_log("EXTEND", true), card_s("OBJECT", "PORTAL"), card_e("EPOCH", 2.0e3f),
        card_e("LONPOLE", 1.8e2f), card_e("EQUINOX", 2.0e3f), card_s("SPECSYS", "LSRK"),
        card_e("RESTFREQ", restfreq), card_int("VELREF", 257), card_s("CTYPE1", "RA---SIN"),
        card_e("CDELT1", cdelt1), card_e("CRPIX1", crpix1), card_e("CRVAL1", crval1),
        card_s("CUNIT1", "DEG"), card_s("CTYPE2", "DEC--SIN"), card_e("CDELT2", cdelt2),
        card_e("CRPIX2", crpix2), card_e("CRVAL2", crval2), card_s("CUNIT2", "DEG"),
        card_s("CTYPE3", "VELO-LSR"), card_e("CDELT3", cdelt3), card_e("CRPIX3", crpix3),
        card_e("CRVAL3", crval3), card_s("CUNIT3", "M/S"), card_e("BSCALE", 1.0f),
        card_e("BZERO", 0.0f), card_s("BUNIT", "K"), "END"};
    std::string hdr;
    for (auto &c : cards) {
        std::string x = c;
        x.resize(80, ' ');
        hdr += x;
    }
    hdr.resize((hdr.size() + 2879) / 2880 * 2880, ' ');
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) return false;
    fwrite(hdr.data(), 1, hdr.size(), f);
    const size_t n = (size_t)npix * npix * nvel;
    std::vector<unsigned char> buf(n * 4);
    for (size_t i = 0; i < n; i++) {
        uint32_t u;
        memcpy(&u, &a[i], 4);
        buf[4 * i] = (unsigned char)(u >> 24);
        buf[4 * i + 1] = (unsigned char)(u >> 16);
        buf[4 * i + 2] = (unsigned char)(u >> 8);
        buf[4 * i + 3] = (unsigned char)u;
    }
    fwrite(buf.data(), 1, buf.size(), f);
    const size_t pad = (2880 - (buf.size() % 2880)) % 2880;
    std::vector<unsigned char> z(pad, 0);
    if (pad) fwrite(z.data(), 1, pad, f);
    return fclose(f) == 0;
}

}  // namespace portal_io
