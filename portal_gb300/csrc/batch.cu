// Many models in one launch: the node loop of every model of a batch as one
// persistent radiation-field launch and one SE launch over all models' nodes,
// captured once into a CUDA graph and replayed, with the launch shapes
// picked by timing candidates on a sample of the work.
//
// No reference counterpart: PORTAL post-processes one LIME model per run.
// Each model keeps its own context (cloud, molecule, device results); the
// batch only orders their work.  Work items are (model, node) pairs; the
// radiation-field kernel takes them from a global queue (dynamic balance of
// uneven models), the SE kernel strides over them.  Items are ordered by
// the models' estimated cost per node, largest first, so the queue's tail
// holds the cheapest nodes.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "internal.cuh"

using namespace portal;

struct portal_batch {
    int device = 0, sm_count = 0;
    cudaStream_t stream = nullptr;
    std::vector<portal_ctx *> models;
    std::string err;

    bool prepared = false;
    int nch = 0, n_depth = 0, kmax = 0, max_lines = 0;
    bool dust = false;
    std::vector<RFArgs> rf;
    std::vector<SEArgs> se;
    DevBuf<RFArgs> d_rf;
    DevBuf<SEArgs> d_se;
    DevBuf<int2> items, sample;
    long long n_items = 0, n_sample = 0;
    size_t se_wb = 0;
    size_t se_a64_stride = 0;           // largest model's c_dim^2
    DevBuf<double> se_a64;              // FP64 SE matrices, one per resident warp
    DevBuf<int2> walk;
    DevBuf<unsigned long long> queue;   // [0] next item, [1] segments

    // launch shapes (the tuner's choice)
    int nlg = 5, rf_bps = 1, se_warps = 8, se_bps = 1;
    std::vector<double> tune;           // candidate timings, ms: (nlg, bps, ms) ... then (warps, bps, ms)

    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

namespace {

int bfail(portal_batch *b, int code, const std::string &m) {
    if (b) b->err = m;
    return code;
}

#define BCHECK(b, call)                                                                                  \
    do {                                                                                                 \
        cudaError_t _e = (call);                                                                         \
        if (_e != cudaSuccess) return bfail((b), PORTAL_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
    } while (0)

void drop_graph(portal_batch *b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

// the whole pass on the batch stream: per-model line tables and zeroed
// outputs, one radiation-field launch, zeroed SE outputs, one SE launch
int enqueue_pass(portal_batch *b, const int2 *items, long long n_items) {
    int rc;
    for (size_t m = 0; m < b->models.size(); m++)
        if ((rc = rf_pass(b->models[m], b->rf[m], b->stream)))
            return bfail(b, rc, "model " + std::to_string(m) + ": " + b->models[m]->err);
    BCHECK(b, cudaMemsetAsync(b->queue.p, 0, 2 * sizeof(unsigned long long), b->stream));
    RFBatch rb{b->d_rf.p, items, n_items, b->queue.p, b->walk.p, b->n_depth};
    if ((rc = rf_batch_launch(b->stream, b->rf_bps * b->sm_count, b->nch, b->dust, b->nlg, b->max_lines, rb)))
        return bfail(b, rc, "radiation-field launch failed");
    for (size_t m = 0; m < b->models.size(); m++)
        if ((rc = se_pass(b->models[m], b->stream)))
            return bfail(b, rc, "model " + std::to_string(m) + ": " + b->models[m]->err);
    SEBatch sb{b->d_se.p, items, n_items, b->se_wb, b->se_a64.p, b->se_a64_stride};
    if ((rc = se_batch_launch(b->stream, b->se_bps * b->sm_count, b->se_warps, sb)))
        return bfail(b, rc, "SE launch failed");
    return PORTAL_OK;
}

// time one candidate launch on the sample (after one untimed launch)
template <typename F>
int time_launch(portal_batch *b, F launch, double *ms) {
    for (int rep = 0; rep < 2; rep++) {
        BCHECK(b, cudaMemsetAsync(b->queue.p, 0, 2 * sizeof(unsigned long long), b->stream));
        BCHECK(b, cudaEventRecord(b->ev0, b->stream));
        int rc = launch();
        if (rc) return bfail(b, rc, "candidate launch failed");
        BCHECK(b, cudaEventRecord(b->ev1, b->stream));
        BCHECK(b, cudaStreamSynchronize(b->stream));
    }
    float t = 0.f;
    BCHECK(b, cudaEventElapsedTime(&t, b->ev0, b->ev1));
    *ms = t;
    return PORTAL_OK;
}

}  // namespace

extern "C" int portal_batch_create(portal_batch **out, int device) {
    if (!out) return PORTAL_ERR_ARG;
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess) return PORTAL_ERR_NODEVICE;
    portal_batch *b = new portal_batch();
    b->device = device;
    if (cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess ||
        b->queue.reserve(2) != cudaSuccess) {
        delete b;
        return PORTAL_ERR_CUDA;
    }
    *out = b;
    return PORTAL_OK;
}

extern "C" int portal_batch_destroy(portal_batch *b) {
    if (!b) return PORTAL_OK;
    cudaSetDevice(b->device);
    cudaStreamSynchronize(b->stream);
    drop_graph(b);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    cudaStreamDestroy(b->stream);
    delete b;
    return PORTAL_OK;
}

extern "C" const char *portal_batch_last_error(const portal_batch *b) { return b ? b->err.c_str() : ""; }

extern "C" int portal_batch_add(portal_batch *b, portal_ctx *c) {
    if (!b || !c) return PORTAL_ERR_ARG;
    if (c->device != b->device) return bfail(b, PORTAL_ERR_ARG, "model context on another device");
    if (!c->have_cloud || !c->have_mol) return bfail(b, PORTAL_ERR_STATE, "model context has no cloud or molecule");
    for (auto *m : b->models)
        if (m == c) return bfail(b, PORTAL_ERR_ARG, "model context added twice");
    b->models.push_back(c);
    b->prepared = false;
    drop_graph(b);
    return (int)b->models.size() - 1;
}

extern "C" int portal_batch_prepare(portal_batch *b, int nth, int nph, int nvel, const double *gvec, double dx,
                                    int n_depth, int kmax, int autotune) {
    if (!b || !gvec) return PORTAL_ERR_ARG;
    if (b->models.empty()) return bfail(b, PORTAL_ERR_STATE, "empty batch");
    cudaSetDevice(b->device);
    drop_graph(b);
    b->prepared = false;
    const int M = (int)b->models.size();
    b->rf.assign(M, RFArgs{});
    b->se.assign(M, SEArgs{});
    b->dust = false;
    b->max_lines = 0;
    size_t wb = 0;
    b->se_a64_stride = 0;
    std::vector<double> cost(M);
    for (int m = 0; m < M; m++) {
        portal_ctx *c = b->models[m];
        int rc = rf_prepare(c, nth, nph, nvel, gvec, dx, n_depth, false, &b->rf[m]);
        if (rc) return bfail(b, rc, "model " + std::to_string(m) + ": " + c->err);
        c->ali_valid = false;
        size_t w = 0;
        if ((rc = se_prepare(c, kmax, &b->se[m], &w)))
            return bfail(b, rc, "model " + std::to_string(m) + ": " + c->err);
        wb = std::max(wb, w);
        b->se_a64_stride = std::max(b->se_a64_stride, se_matrix_doubles(c));
        b->dust = b->dust || c->has_dust;
        b->max_lines = std::max(b->max_lines, c->r_num);
        // per-node cost ~ lines x cells per ray ~ L N^(1/3)
        cost[m] = (double)c->r_num * std::cbrt((double)c->N);
    }
    b->nch = 2 * nvel + 1;
    b->n_depth = n_depth;
    b->kmax = kmax;
    b->se_wb = wb;
    // work items, models by descending cost per node
    std::vector<int> ord(M);
    for (int m = 0; m < M; m++) ord[m] = m;
    std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return cost[x] > cost[y]; });
    std::vector<int2> it, sm;
    for (int m : ord)
        for (int n = 0; n < b->models[m]->bulk; n++) it.push_back(make_int2(m, n));
    for (size_t i = 0; i < it.size(); i += 16) sm.push_back(it[i]);
    b->n_items = (long long)it.size();
    b->n_sample = (long long)sm.size();
    if (b->d_rf.reserve(M) || b->d_se.reserve(M) || b->items.reserve(it.size()) || b->sample.reserve(sm.size()))
        return bfail(b, PORTAL_ERR_NOMEM, "batch tables");
    BCHECK(b, cudaMemcpyAsync(b->d_rf.p, b->rf.data(), sizeof(RFArgs) * M, cudaMemcpyHostToDevice, b->stream));
    BCHECK(b, cudaMemcpyAsync(b->d_se.p, b->se.data(), sizeof(SEArgs) * M, cudaMemcpyHostToDevice, b->stream));
    BCHECK(b, cudaMemcpyAsync(b->items.p, it.data(), sizeof(int2) * it.size(), cudaMemcpyHostToDevice, b->stream));
    BCHECK(b, cudaMemcpyAsync(b->sample.p, sm.data(), sizeof(int2) * sm.size(), cudaMemcpyHostToDevice, b->stream));
    BCHECK(b, cudaStreamSynchronize(b->stream));

    // candidate launch shapes: radiation field (line group, blocks per SM),
    // SE (warps per block; blocks per SM from the occupancy)
    struct RFC { int nlg, bps; };
    std::vector<RFC> rfc;
    const void *seen = nullptr;
    for (int nlg : {5, 10}) {
        // layouts with the lanes-over-lines remainder channel have one line
        // group; do not time the same kernel twice
        const void *k = rf_batch_kernel_ptr(b->nch, b->dust, nlg, b->max_lines);
        if (k == seen) continue;
        seen = k;
        int mx = 0;
        if (rf_batch_blocks_per_sm(b->nch, b->dust, nlg, b->max_lines, &mx))
            return bfail(b, PORTAL_ERR_CUDA, "occupancy query");
        for (int bps = 1; bps <= std::min(mx, 2); bps++) rfc.push_back({nlg, bps});
    }
    if (rfc.empty()) return bfail(b, PORTAL_ERR_CUDA, "radiation-field kernel does not fit on an SM");
    std::vector<int> sec;
    for (int w : {2, 4, 8})
        if (wb * w <= 200 * 1024) sec.push_back(w);
    if (sec.empty()) return bfail(b, PORTAL_ERR_ARG, "SE system too large for shared memory");
    int dummy = 0;
    if (se_batch_blocks_per_sm(sec.back(), wb, b->se_a64_stride, &dummy))  // raises the smem limit to the largest candidate
        return bfail(b, PORTAL_ERR_CUDA, "SE occupancy query");
    // FP64 matrix slots for the largest SE grid among the candidates
    {
        size_t most = 0;
        for (int w : sec) {
            int bps = 0;
            if (se_batch_blocks_per_sm(w, wb, b->se_a64_stride, &bps)) return bfail(b, PORTAL_ERR_CUDA, "SE occupancy query");
            most = std::max(most, (size_t)std::max(1, bps) * b->sm_count * w);
        }
        se_batch_blocks_per_sm(sec.back(), wb, b->se_a64_stride, &dummy);
        if (b->se_a64.reserve(most * b->se_a64_stride)) return bfail(b, PORTAL_ERR_NOMEM, "SE matrix scratch");
    }
    // walk scratch for the largest grid
    const size_t warps = (size_t)2 * b->sm_count * 8;
    if (b->walk.reserve(warps * 32 * (size_t)n_depth)) return bfail(b, PORTAL_ERR_NOMEM, "walk scratch");

    b->tune.clear();
    if (autotune) {
        // line tables for the trials (the trials' results are overwritten by
        // every later pass)
        for (int m = 0; m < M; m++)
            if (int rc = rf_pass(b->models[m], b->rf[m], b->stream)) return bfail(b, rc, b->models[m]->err);
        double best = 1e300;
        for (const RFC &c : rfc) {
            RFBatch rb{b->d_rf.p, b->sample.p, b->n_sample, b->queue.p, b->walk.p, n_depth};
            double ms = 0.0;
            int rc = time_launch(b, [&]() { return rf_batch_launch(b->stream, c.bps * b->sm_count, b->nch, b->dust,
                                                                  c.nlg, b->max_lines, rb); }, &ms);
            if (rc) return rc;
            b->tune.insert(b->tune.end(), {(double)c.nlg, (double)c.bps, ms});
            if (ms < best) { best = ms; b->nlg = c.nlg; b->rf_bps = c.bps; }
        }
        best = 1e300;
        for (int w : sec) {
            int bps = 0;
            if (se_batch_blocks_per_sm(w, wb, b->se_a64_stride, &bps)) return bfail(b, PORTAL_ERR_CUDA, "SE occupancy query");
            bps = std::max(1, bps);
            SEBatch sb{b->d_se.p, b->sample.p, b->n_sample, wb, b->se_a64.p, b->se_a64_stride};
            double ms = 0.0;
            int rc = time_launch(b, [&]() { return se_batch_launch(b->stream, bps * b->sm_count, w, sb); }, &ms);
            if (rc) return rc;
            b->tune.insert(b->tune.end(), {(double)w, (double)bps, ms});
            if (ms < best) { best = ms; b->se_warps = w; b->se_bps = bps; }
        }
        se_batch_blocks_per_sm(sec.back(), wb, b->se_a64_stride, &dummy);
    } else {
        b->nlg = 5;
        b->rf_bps = 1;
        for (const RFC &c : rfc)
            if (c.nlg == 5) b->rf_bps = std::max(b->rf_bps, c.bps);
        b->se_warps = sec.back();
        int bps = 0;
        se_batch_blocks_per_sm(b->se_warps, wb, b->se_a64_stride, &bps);
        b->se_bps = std::max(1, bps);
    }

    // capture the pass once
    BCHECK(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue_pass(b, b->items.p, b->n_items);
    cudaGraph_t g = nullptr;
    cudaError_t ee = cudaStreamEndCapture(b->stream, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (ee != cudaSuccess) return bfail(b, PORTAL_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ee));
    b->graph = g;
    BCHECK(b, cudaGraphInstantiate(&b->exec, b->graph, 0));
    b->prepared = true;
    return PORTAL_OK;
}

// One node-loop pass of every model (radiation field + SE); the results
// stay on the device in each model's context.  use_graph 0 enqueues the
// same launches directly instead of replaying the graph.
extern "C" int portal_batch_run(portal_batch *b, int use_graph, long long *n_segments, double *ms) {
    if (!b) return PORTAL_ERR_ARG;
    if (!b->prepared) return bfail(b, PORTAL_ERR_STATE, "portal_batch_prepare first");
    cudaSetDevice(b->device);
    BCHECK(b, cudaEventRecord(b->ev0, b->stream));
    if (use_graph) {
        BCHECK(b, cudaGraphLaunch(b->exec, b->stream));
    } else {
        int rc = enqueue_pass(b, b->items.p, b->n_items);
        if (rc) return rc;
    }
    BCHECK(b, cudaEventRecord(b->ev1, b->stream));
    unsigned long long q[2] = {0, 0};
    BCHECK(b, cudaMemcpyAsync(q, b->queue.p, sizeof q, cudaMemcpyDeviceToHost, b->stream));
    BCHECK(b, cudaStreamSynchronize(b->stream));
    float t = 0.f;
    BCHECK(b, cudaEventElapsedTime(&t, b->ev0, b->ev1));
    if (ms) *ms = t;
    if (n_segments) *n_segments = (long long)q[1];
    for (auto *c : b->models) {
        c->j_valid = true;
        c->ali_valid = false;
    }
    return PORTAL_OK;
}

// The launch shapes in use and the tuner's timings: config = (line group,
// radiation-field blocks per SM, SE warps per block, SE blocks per SM);
// tune receives up to max_tune values, triples (shape, shape, ms) per
// candidate; returns the number of values available.
extern "C" int portal_batch_config(const portal_batch *b, int *config, double *tune, int max_tune) {
    if (!b) return PORTAL_ERR_ARG;
    if (config) {
        config[0] = b->nlg;
        config[1] = b->rf_bps;
        config[2] = b->se_warps;
        config[3] = b->se_bps;
    }
    if (tune)
        for (int i = 0; i < max_tune && i < (int)b->tune.size(); i++) tune[i] = b->tune[i];
    return (int)b->tune.size();
}
