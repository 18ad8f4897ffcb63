// Radiation field of every node: the inverse_rt loop of main_portal.x.
//
// Reference: main_para.f90:210-257 -> trace_node main_sub.f90:82-84 ->
// inverse_rt inverse_rt.f90:1-137, trace_out :139-214 (with
// check_neigh_fast miscellaneous.f90:1017-1076, pos_quadratic :1078-1098),
// ray_in :217-344, find_dir miscellaneous.f90:48-82.
//
// Two kernels:
//   k_line_table   per (node, line): the opacity / emissivity factors that
//                  ray_in rebuilds for every (direction, channel, cell):
//                  A = kv * c/nu / (sqrt(pi) b) * tx*dx   (optical depth per
//                  trace step per unit Gaussian profile value), E the same
//                  for the emissivity, and the dust terms.  HBM-bound, tiny.
//   k_radiation_field  one warp per node (persistent warps, node queue);
//                  the directions of legendre_all in batches of 32 rays:
//                   (1) FP64 set-up, one lane per ray: the direction
//                       (find_dir's rotation in closed form) and the
//                       sphere-exit distance (pos_quadratic from the node,
//                       as trace_out's first step computes it);
//                   (2) the Voronoi walk, one lane per ray, 32 rays in
//                       flight per warp.  The photon is kept relative to the
//                       current node, so the face crossing
//                       t = (|e|^2/2 - e.r) / (e.d) is formed from the
//                       FP64-derived edge vectors without cancellation
//                       against absolute coordinates; the neighbour scan
//                       keeps check_neigh_fast's sequential tie rule.  The
//                       (cell, steps) list of each ray goes to a per-warp
//                       scratch slice in global memory (L2-resident);
//                   (3) the channel integration inward over the walk, lanes
//                       over channels, lines looped in registers, cell
//                       records staged in shared memory 32 cells at a time;
//                   (4) the profile-weighted channel sum (warp reduction)
//                       and the compensated accumulation of J^0_0, J^2_0
//                       over directions (fixed order: deterministic).
//                  On request it also splits J^0_0 = J_eff + L* S_line at
//                  the central cell: J_eff the field without the node's own
//                  line emission, L* = dJ^0_0/dS_line the diagonal of the
//                  Lambda operator (what the node's own cell contributes per
//                  unit source function) -- the inputs of the preconditioned
//                  SE of the accelerated Lambda iteration.
#include <cmath>
#include <cstdlib>

#include "rf_kernel.cuh"

using namespace portal;


namespace {

// upload per-line constants of the molecule into the context
int upload_lines(portal_ctx *c) {
    if (c->r_num > MAX_LINES)
        return set_err(c, PORTAL_ERR_ARG, "more than 64 radiative lines are not supported");
    std::vector<LineConst> h(c->r_num);
    std::vector<float> bb(c->r_num);
    for (int k = 0; k < c->r_num; k++) {
        int lo = c->r_trans[2 * k] - 1, up = c->r_trans[2 * k + 1] - 1;
        h[k].nu = c->nu[k];
        h[k].A = c->A[k];
        h[k].B = c->Bij[k];
        h[k].kd = c->kd_v[k];
        h[k].glo = 2.0 * c->j_lev[lo] + 1.0;
        h[k].gup = 2.0 * c->j_lev[up] + 1.0;
        // black_body(2.73, nu) miscellaneous.f90:263-285
        h[k].bb_cmb = 1.4744995e-50 * std::pow(c->nu[k], 3.0) *
                      std::pow(std::exp(4.79924e-11 / 2.73 * c->nu[k]) - 1.0, -1.0);
        h[k].lo = lo;
        h[k].up = up;
        bb[k] = (float)h[k].bb_cmb;
    }
    if (c->linebuf.reserve(sizeof(LineConst) * c->r_num) || c->bbcmb.reserve(c->r_num) ||
        c->bbstar.reserve(c->r_num))
        return set_err(c, PORTAL_ERR_NOMEM, "line constants");
    // star rays start from black_body(T_star) (inverse_rt.f90:113-115)
    std::vector<float> bs(c->r_num, 0.f);
    if (c->star_mode && c->T_star > 0.0)
        for (int k = 0; k < c->r_num; k++)
            bs[k] = (float)(1.4744995e-50 * std::pow(c->nu[k], 3.0) *
                            std::pow(std::exp(4.79924e-11 / c->T_star * c->nu[k]) - 1.0, -1.0));
    PCHECK(c, cudaMemcpyAsync(c->bbstar.p, bs.data(), sizeof(float) * c->r_num, cudaMemcpyHostToDevice,
                              c->stream));
    PCHECK(c, cudaMemcpyAsync(c->linebuf.p, h.data(), sizeof(LineConst) * c->r_num, cudaMemcpyHostToDevice,
                              c->stream));
    PCHECK(c, cudaMemcpyAsync(c->bbcmb.p, bb.data(), sizeof(float) * c->r_num, cudaMemcpyHostToDevice,
                              c->stream));
    return PORTAL_OK;
}

// Warps per block of the radiation-field kernel: 8, or PORTAL_RF_WARPS (4..8)
// -- fewer warps per block let a register-heavy variant keep two blocks on
// an SM.
inline int rf_warps() {
    const char *e = getenv("PORTAL_RF_WARPS");
    const int v = e ? atoi(e) : 8;
    return (v >= 4 && v <= 8) ? v : 8;
}

template <int NS, int NLG, bool DUST, int RT>
int launch_rf(portal_ctx *c, RFArgs &a, int n_depth) {
    auto kern = k_radiation_field<NS, NLG, DUST, false, RT>;
    const int wpb = rf_warps();
    // the remainder channel's (cell, line) tables, one per warp
    const size_t dyn = RT ? (size_t)wpb * 32 * rem_row_stride(a.L) * sizeof(float2) : 0;
    if (dyn) PCHECK(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
    int nb = 0;
    PCHECK(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, 32 * wpb, dyn));
    if (nb < 1) nb = 1;
    int grid = nb * c->sm_count;
    size_t nslots = (size_t)grid * wpb;
    if (c->walk.reserve(nslots * 32 * (size_t)n_depth) != cudaSuccess)
        return set_err(c, PORTAL_ERR_NOMEM, "walk scratch allocation failed");
    a.walk = c->walk.p;
    PCHECK(c, cudaMemsetAsync(c->counters.p, 0, 8 * sizeof(unsigned long long), c->stream));
    timer_start(c, T_RF);
    kern<<<grid, 32 * wpb, dyn, c->stream>>>(a, RFBatch{});
    timer_stop(c, T_RF);
    PCHECK(c, cudaGetLastError());
    return PORTAL_OK;
}

// Line-group width: lines whose intensities one lane keeps in registers at
// once.  Lines are padded to whole groups, and a padding line costs as much
// as a real one, so the width is the one of 5, 4, 3 with the fewest padded
// lines (the larger on ties: fewer passes over the walk lists); 10 saves
// profile evaluations but needs more than 128 registers (one block per SM).
// PORTAL_RF_LINE_GROUP=3|4|5|10 overrides the choice.
inline int line_group(int L) {
    const char *e = getenv("PORTAL_RF_LINE_GROUP");
    if (e) {
        const int v = atoi(e);
        if (v == 3 || v == 4 || v == 5 || v == 10) return v;
    }
    int best = 5, slots = 1 << 30;
    for (int g : {5, 4, 3}) {
        const int sl = ((L + g - 1) / g) * g;
        if (sl < slots) { slots = sl; best = g; }
    }
    return best;
}

template <int NS, int RT>
int dispatch_nlg(portal_ctx *c, RFArgs &a, int n_depth) {
    if (c->has_dust) {  // the dust variants: groups of 5 (or 10), whole slots
        return line_group(a.L) == 10 ? launch_rf<NS, 10, true, 0>(c, a, n_depth)
                                     : launch_rf<NS, 5, true, 0>(c, a, n_depth);
    }
    switch (line_group(a.L)) {
    case 3: return launch_rf<NS, 3, false, RT>(c, a, n_depth);
    case 4: return launch_rf<NS, 4, false, RT>(c, a, n_depth);
    case 10: return RT ? launch_rf<NS, 5, false, RT>(c, a, n_depth) : launch_rf<NS, 10, false, 0>(c, a, n_depth);
    default: return launch_rf<NS, 5, false, RT>(c, a, n_depth);
    }
}

// Star mode: the node loop through the batched kernel with one model.  Its
// instantiations carry the per-node star ray sets (star_all); the
// single-model kernel leaves that code out, which keeps its registers for the
// integration (1 % faster on the benchmark sphere).
int launch_rf_star(portal_ctx *c, RFArgs &a, int n_depth) {
    const int nlg = (c->has_dust && line_group(a.L) == 10) ? 10 : 5;
    int nb = 0;
    if (rf_batch_blocks_per_sm(a.nch, c->has_dust, nlg, a.L, &nb))
        return set_err(c, PORTAL_ERR_CUDA, "star mode: occupancy query failed");
    if (nb < 1) nb = 1;
    const int grid = nb * c->sm_count;
    if (c->walk.reserve((size_t)grid * 8 * 32 * (size_t)n_depth) != cudaSuccess)
        return set_err(c, PORTAL_ERR_NOMEM, "walk scratch allocation failed");
    if (c->star_model.reserve(sizeof(RFArgs)) || c->star_items.reserve(c->bulk > 0 ? c->bulk : 1))
        return set_err(c, PORTAL_ERR_NOMEM, "star-mode work items");
    if (c->star_items_n != c->bulk) {
        std::vector<int2> it((size_t)c->bulk);
        for (int n = 0; n < c->bulk; n++) it[n] = make_int2(0, n);
        PCHECK(c, cudaMemcpyAsync(c->star_items.p, it.data(), it.size() * sizeof(int2), cudaMemcpyHostToDevice,
                                  c->stream));
        PCHECK(c, cudaStreamSynchronize(c->stream));
        c->star_items_n = c->bulk;
    }
    a.walk = c->walk.p;
    PCHECK(c, cudaMemcpyAsync(c->star_model.p, &a, sizeof(RFArgs), cudaMemcpyHostToDevice, c->stream));
    PCHECK(c, cudaMemsetAsync(c->counters.p, 0, 8 * sizeof(unsigned long long), c->stream));
    RFBatch bw;
    bw.models = reinterpret_cast<const RFArgs *>(c->star_model.p);
    bw.items = c->star_items.p;
    bw.n_items = c->bulk;
    bw.queue = c->counters.p;  // [0] next item, [1] segments, as the single-model kernel's counters
    bw.walk = c->walk.p;
    bw.n_depth = n_depth;
    timer_start(c, T_RF);
    const int rc = rf_batch_launch(c->stream, grid, a.nch, c->has_dust, nlg, a.L, bw);
    timer_stop(c, T_RF);
    if (rc) return set_err(c, rc, std::string("star mode: ") + cudaGetErrorString(cudaGetLastError()));
    // the argument block is read by the kernel: keep it until the stream passes here
    PCHECK(c, cudaStreamSynchronize(c->stream));
    return PORTAL_OK;
}

int dispatch_rf(portal_ctx *c, RFArgs &a, int n_depth) {
    if (a.star) return launch_rf_star(c, a, n_depth);
    const ChanLayout cl = chan_layout(a.nch, c->has_dust, a.L);
    if (cl.rt) {
        switch (cl.ns) {
        case 1: return dispatch_nlg<1, 1>(c, a, n_depth);
        case 2: return dispatch_nlg<2, 1>(c, a, n_depth);
        case 4: return dispatch_nlg<4, 1>(c, a, n_depth);
        default: return dispatch_nlg<8, 1>(c, a, n_depth);
        }
    }
    switch (cl.ns) {
    case 1: return dispatch_nlg<1, 0>(c, a, n_depth);
    case 2: return dispatch_nlg<2, 0>(c, a, n_depth);
    case 3: return dispatch_nlg<3, 0>(c, a, n_depth);
    case 5: return dispatch_nlg<5, 0>(c, a, n_depth);
    default: return dispatch_nlg<9, 0>(c, a, n_depth);
    }
}

}  // namespace

namespace portal {

// Validates the call, uploads the molecule's line constants and the
// direction / channel tables, sizes the outputs and fills the kernel's
// argument block (walk scratch and counters are the launcher's).
int rf_prepare(portal_ctx *c, int nth, int nph, int nvel, const double *gvec, double dx, int n_depth,
               bool split, RFArgs *out) {
    if (!c->have_cloud || !c->have_mol) return set_err(c, PORTAL_ERR_STATE, "no cloud or molecule");
    if (c->nlev != (int)c->j_lev.size())
        return set_err(c, PORTAL_ERR_STATE, "cloud and molecule disagree on nlev");
    if (nth < 1 || nph < 1 || nvel < 1 || n_depth < 1 || !gvec || !(dx > 0.0) || 2 * nvel + 1 > 288)
        return set_err(c, PORTAL_ERR_ARG, "portal_radiation_field: bad nth/nph/nvel/n_depth/dx "
                                          "(at most 288 channels)");
    cudaSetDevice(c->device);
    int rc;
    if ((rc = upload_lines(c))) return rc;
    const int L = c->r_num, N = c->N;
    // direction table (legendre_all) and channel tables
    std::vector<double> xth;
    const int ndir = legendre_all(nth, nph, xth);
    std::vector<double> dt(6 * (size_t)ndir);
    for (int k = 0; k < ndir; k++) {
        double mu = xth[3 * k], ph = xth[3 * k + 1], w = xth[3 * k + 2];
        double th = std::acos(mu);
        double c_in = (3.0 * mu * mu - 1.0) / 2.0;
        dt[6 * k + 0] = std::cos(th);
        dt[6 * k + 1] = std::sin(th);
        dt[6 * k + 2] = std::cos(ph);
        dt[6 * k + 3] = std::sin(ph);
        dt[6 * k + 4] = w;
        dt[6 * k + 5] = w * c_in / std::sqrt(2.0);
    }
    const int nch = 2 * nvel + 1;
    std::vector<float> ct(2 * (size_t)nch);
    const double spi = std::sqrt(std::acos(-1.0));
    for (int i = 0; i < nch; i++) {
        int nv = i - nvel;
        double q0 = 2.0 * nv / nvel;
        ct[i] = (float)q0;
        // phi_v0 * d_v = exp(-q0^2)/(sqrt(pi) b) * 2 b / nvel
        ct[nch + i] = (float)(std::exp(-q0 * q0) * 2.0 / (spi * nvel));
    }
    if (c->dirtab.reserve(dt.size()) || c->chtab.reserve(ct.size()) ||
        c->ltab.reserve((size_t)L * N) || c->J0.reserve((size_t)L * N) || c->J2.reserve((size_t)L * N) ||
        c->nodeseg.reserve((size_t)N) || c->kmom.reserve((size_t)6 * N))
        return set_err(c, PORTAL_ERR_NOMEM, "radiation-field buffers");
    if (split && (c->JE.reserve((size_t)L * N) || c->LS.reserve((size_t)L * N)))
        return set_err(c, PORTAL_ERR_NOMEM, "split-field buffers");
    PCHECK(c, cudaMemcpyAsync(c->dirtab.p, dt.data(), dt.size() * sizeof(double),
                              cudaMemcpyHostToDevice, c->stream));
    PCHECK(c, cudaMemcpyAsync(c->chtab.p, ct.data(), ct.size() * sizeof(float),
                              cudaMemcpyHostToDevice, c->stream));
    // the host vectors go out of scope: the copies must have happened
    PCHECK(c, cudaStreamSynchronize(c->stream));
    RFArgs a;
    a.N = N; a.bulk = c->bulk; a.L = L; a.nvel = nvel; a.nch = nch; a.ndir = ndir; a.n_depth = n_depth;
    a.dx32 = (float)dx;
    a.pos = c->pos64.p; a.bvec = c->bvec64.p; a.ab = c->ab.p; a.cellv = c->cellv.p;
    a.off = c->nb_off.p; a.idx = c->nb_idx.p; a.edge = c->edge.p; a.ltab = c->ltab.p;
    a.dirs = c->dirtab.p; a.chq = c->chtab.p; a.chw = c->chtab.p + nch; a.bb = c->bbcmb.p;
    a.gx = gvec[0]; a.gy = gvec[1]; a.gz = gvec[2];
    a.ab = c->active_ab();
    a.star = c->star_mode; a.nth = nth; a.nph = nph;
    a.xs = c->X_star[0]; a.ys = c->X_star[1]; a.zs = c->X_star[2];
    a.Rs = c->star_mode ? c->R_star() : 0.0;
    a.bbs = c->bbstar.p;
    a.J0 = c->J0.p; a.J2 = c->J2.p; a.status = c->status.p; a.counters = c->counters.p;
    a.segs = c->nodeseg.p;
    a.kmom = c->kmom.p;
    a.JE = split ? c->JE.p : nullptr;
    a.LS = split ? c->LS.p : nullptr;
    a.walk = nullptr;
    // the line table's transfer step (main_para.f90:135 dx times r_max)
    c->rf_dxp = c->tx * dx;
    *out = a;
    return PORTAL_OK;
}

// The per-pass device work before the walk: zeroed outputs and the line
// table from the current populations.  Stream-ordered only (capturable).
int rf_pass(portal_ctx *c, const RFArgs &a, cudaStream_t s) {
    const int L = c->r_num, N = c->N;
    PCHECK(c, cudaMemsetAsync(c->J0.p, 0, (size_t)L * N * sizeof(double), s));
    PCHECK(c, cudaMemsetAsync(c->J2.p, 0, (size_t)L * N * sizeof(double), s));
    PCHECK(c, cudaMemsetAsync(c->status.p, 0, (size_t)N * sizeof(int), s));
    if (a.segs) PCHECK(c, cudaMemsetAsync(a.segs, 0, (size_t)N * sizeof(int), s));
    if (a.kmom) PCHECK(c, cudaMemsetAsync(a.kmom, 0, (size_t)6 * N * sizeof(float), s));
    if (a.JE) {
        PCHECK(c, cudaMemsetAsync(c->JE.p, 0, (size_t)L * N * sizeof(double), s));
        PCHECK(c, cudaMemsetAsync(c->LS.p, 0, (size_t)L * N * sizeof(double), s));
    }
    const long long tot = (long long)N * L;
    k_line_table<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(
        N, L, c->rf_dxp, reinterpret_cast<const LineConst *>(c->linebuf.p), c->levp.p, c->nlev, c->b64.p,
        c->dustp.p, c->tdust.p, c->ltab.p);
    PCHECK(c, cudaGetLastError());
    return PORTAL_OK;
}

// Runs the line table + radiation field on the device; J stays in c->J0/J2
// (and the split field in c->JE/LS when `split`).
int run_radiation_field(portal_ctx *c, int nth, int nph, int nvel, const double *gvec, double dx,
                        int n_depth, long long *n_segments, int *n_failed, bool split) {
    RFArgs a;
    int rc = rf_prepare(c, nth, nph, nvel, gvec, dx, n_depth, split, &a);
    if (rc) return rc;
    c->ali_valid = false;
    timer_start(c, T_LINETAB);
    if ((rc = rf_pass(c, a, c->stream))) return rc;
    timer_stop(c, T_LINETAB);
    if ((rc = dispatch_rf(c, a, n_depth))) return rc;
    unsigned long long cnt[8];
    PCHECK(c, cudaMemcpyAsync(cnt, c->counters.p, sizeof cnt, cudaMemcpyDeviceToHost, c->stream));
    PCHECK(c, cudaStreamSynchronize(c->stream));
    timer_collect(c, T_LINETAB);
    timer_collect(c, T_RF);
    if (n_segments) *n_segments = (long long)cnt[1];
    // failed nodes, counted on the host from the status array when asked (the
    // iterated node loop): a walk past n_depth or a star ray set past nth*nph
    // is an error, as the reference stops there
    if (n_failed) {
        std::vector<int> st((size_t)c->N);
        PCHECK(c, cudaMemcpyAsync(st.data(), c->status.p, st.size() * sizeof(int), cudaMemcpyDeviceToHost,
                                  c->stream));
        PCHECK(c, cudaStreamSynchronize(c->stream));
        int nf = 0, first = -1, bits = 0;
        for (int i = 0; i < c->N; i++)
            if (st[i] & (PORTAL_NODE_DEPTH | PORTAL_NODE_STAR)) {
                if (first < 0) first = i;
                bits |= st[i];
                nf++;
            }
        *n_failed = nf;
        if (nf)
            return set_err(c, (bits & PORTAL_NODE_DEPTH) ? PORTAL_ERR_DEPTH : PORTAL_ERR_ARG,
                           std::string((bits & PORTAL_NODE_DEPTH) ? "node_count > n_depth" : "star rays > nth*nph") +
                               " for " + std::to_string(nf) + " node(s), the first node " + std::to_string(first + 1));
    }
    c->j_valid = true;
    c->ali_valid = split;
    return PORTAL_OK;
}

}  // namespace portal

namespace {

int radiation_field_call(portal_ctx *c, int nth, int nph, int nvel, const double *gvec, double dx,
                         int n_depth, double *J0, double *J2, double *JE, double *LS, bool split, int *status,
                         long long *n_segments) {
    if (!c) return PORTAL_ERR_ARG;
    timers_reset(c);
    int rc = portal::run_radiation_field(c, nth, nph, nvel, gvec, dx, n_depth, n_segments, nullptr, split);
    if (rc) return rc;
    const size_t LN = (size_t)c->r_num * c->N;
    if (J0) PCHECK(c, cudaMemcpyAsync(J0, c->J0.p, LN * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if (J2) PCHECK(c, cudaMemcpyAsync(J2, c->J2.p, LN * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if (split && JE) PCHECK(c, cudaMemcpyAsync(JE, c->JE.p, LN * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if (split && LS) PCHECK(c, cudaMemcpyAsync(LS, c->LS.p, LN * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    std::vector<int> st_host;
    int *st = status;
    if (!st) { st_host.resize(c->N); st = st_host.data(); }
    PCHECK(c, cudaMemcpyAsync(st, c->status.p, (size_t)c->N * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    PCHECK(c, cudaStreamSynchronize(c->stream));
    for (int i = 0; i < c->N; i++) {
        if (st[i] & PORTAL_NODE_DEPTH)
            return set_err(c, PORTAL_ERR_DEPTH, "node_count > n_depth for node " + std::to_string(i + 1));
        if (st[i] & PORTAL_NODE_STAR)
            return set_err(c, PORTAL_ERR_ARG, "star mode: the star's rays exceed nth*nph for node " +
                                                  std::to_string(i + 1) + " (a node this close to the star "
                                                                          "stops the reference too)");
    }
    return PORTAL_OK;
}

}  // namespace

extern "C" int portal_radiation_field(portal_ctx *c, int nth, int nph, int nvel, const double *gvec,
                                      double dx, int n_depth, double *J0, double *J2, int *status,
                                      long long *n_segments) {
    return radiation_field_call(c, nth, nph, nvel, gvec, dx, n_depth, J0, J2, nullptr, nullptr, false, status,
                                n_segments);
}

extern "C" int portal_radiation_field_split(portal_ctx *c, int nth, int nph, int nvel, const double *gvec,
                                            double dx, int n_depth, double *J0, double *J2, double *J_eff,
                                            double *L_star, int *status, long long *n_segments) {
    return radiation_field_call(c, nth, nph, nvel, gvec, dx, n_depth, J0, J2, J_eff, L_star, true, status,
                                n_segments);
}

extern "C" int portal_node_segments(portal_ctx *c, int *segments) {
    if (!c || !segments) return PORTAL_ERR_ARG;
    if (!c->j_valid || !c->nodeseg.p) return set_err(c, PORTAL_ERR_STATE, "no radiation field computed");
    PCHECK(c, cudaMemcpyAsync(segments, c->nodeseg.p, (size_t)c->N * sizeof(int), cudaMemcpyDeviceToHost,
                              c->stream));
    PCHECK(c, cudaStreamSynchronize(c->stream));
    return PORTAL_OK;
}

extern "C" int portal_field_moments(portal_ctx *c, double *moments) {
    if (!c || !moments) return PORTAL_ERR_ARG;
    if (!c->j_valid || !c->kmom.p) return set_err(c, PORTAL_ERR_STATE, "no radiation field computed");
    std::vector<float> h((size_t)6 * c->N);
    PCHECK(c, cudaMemcpyAsync(h.data(), c->kmom.p, h.size() * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    PCHECK(c, cudaStreamSynchronize(c->stream));
    for (int n = 0; n < c->N; n++)
        for (int k = 0; k < 6; k++) moments[6 * (size_t)n + k] = (double)h[(size_t)k * c->N + n];
    return PORTAL_OK;
}
