// depix_queue.cu -- host side of the uneven-batch path: per-call tile
// descriptors, the launch-shape tuner and the CUDA graphs that replay the
// persistent stage kernels.
//
// The reference processes one frame per launch_kernel call (kernel.cu:286-526)
// with a grid sized to that frame. Batching frames of different sizes into one
// grid per stage needs a map from a block to its frame; here every stage is a
// persistent kernel that pulls tile indices from a counter and finds the
// frame by binary search over a per-stage prefix of the frames' tile counts.
// Descriptors (frame sizes, offsets, prefixes) travel to the device in one
// copy per call from a ring of pinned slots; the kernels' parameters do not
// change between calls, so each launch shape is captured once as a graph.
#include <algorithm>
#include <cstring>
#include <map>
#include <string>

#include "depix_internal.h"

namespace depix {

namespace {

constexpr int kSlots = 4;             // pinned descriptor slots in flight
constexpr size_t kHeaderBytes = 128;  // QueueHeader, rounded up
static_assert(sizeof(QueueHeader) <= kHeaderBytes, "descriptor header");
static_assert(sizeof(QueueFrame) % 16 == 0, "descriptor frames");
constexpr uint32_t kMaxTiles = 1u << 30; // keeps the int tile counters far from overflow

size_t prefix_bytes(int n) { return ((size_t)kQPrefixes * (n + 1) * sizeof(uint32_t) + 15) & ~(size_t)15; }
size_t desc_bytes(int n) { return kHeaderBytes + prefix_bytes(n) + (size_t)n * sizeof(QueueFrame); }

uint32_t tiles(int w, int h, int tw, int th) { return (uint32_t)((w + tw - 1) / tw) * (uint32_t)((h + th - 1) / th); }

int log2_floor(uint64_t x)
{
    int k = 0;
    while (x > 1) {
        x >>= 1;
        k++;
    }
    return k;
}

// Graph cache key: everything a captured graph bakes in besides the context.
uint64_t graph_key(int scale, bool labels, int vote, const QueueShape& sh)
{
    const int shape = sh.rtw == 0 ? 3 : raster_shape_index(sh.rtw, sh.rth);
    uint64_t k = (uint64_t)scale | (uint64_t)labels << 8 | (uint64_t)shape << 9 | (uint64_t)vote << 28;
    for (int st = 0; st < QS_COUNT; st++) k |= (uint64_t)log2_floor((uint64_t)sh.gran[st]) << (12 + 4 * st);
    return k;
}

#define DEPIX_TRY_STATUS(call)                                          \
    do {                                                                \
        depix_status st_ = (call);                                      \
        if (st_ != DEPIX_OK) return st_;                                \
    } while (0)

depix_status fail(cudaError_t e, const char* where)
{
    set_last_error(std::string(where) + ": " + cudaGetErrorString(e));
    return DEPIX_ERR_CUDA;
}

}  // namespace

class QueueRunner {
public:
    int cap = 0, sms = 0;
    uint8_t* d_desc = nullptr;
    int* d_counters = nullptr;
    uint8_t* h_slot[kSlots] = {};
    cudaEvent_t slot_copied[kSlots] = {};
    int next_slot = 0;
    cudaStream_t capture_stream = nullptr;
    cudaEvent_t tev[QS_COUNT + 1] = {};
    std::map<uint64_t, QueueShape> tuned;     // per size bucket
    std::map<uint64_t, cudaGraphExec_t> graphs; // per graph_key
    std::map<uint64_t, int> occ;              // blocks per SM per stage variant
    bool forced = false;
    QueueShape force{};
    // the prepared call
    QueueBatch q{};
    QueueShape shape{};
    uint32_t total[kQPrefixes] = {};
    bool labels = false;

    ~QueueRunner()
    {
        for (auto& g : graphs) cudaGraphExecDestroy(g.second);
        for (int k = 0; k < kSlots; k++) {
            if (slot_copied[k]) {
                cudaEventSynchronize(slot_copied[k]);
                cudaEventDestroy(slot_copied[k]);
            }
            cudaFreeHost(h_slot[k]);
        }
        for (auto e : tev)
            if (e) cudaEventDestroy(e);
        if (capture_stream) cudaStreamDestroy(capture_stream);
        dev_free(d_desc);
        dev_free(d_counters);
    }

    // blocks per SM of a stage's kernel (the raster's depends on the scale
    // and tile); 0 when the variant cannot launch
    int blocks_per_sm(int stage, const QueueBatch& b)
    {
        const uint64_t key = stage == QS_RASTER
                                 ? (uint64_t)(4 + raster_shape_index(b.rtw, b.rth)) | (uint64_t)b.scale << 8
                                 : (uint64_t)stage | (uint64_t)b.vote << 16;
        auto it = occ.find(key);
        if (it != occ.end()) return it->second;
        const int v = queue_blocks_per_sm(stage, b);
        occ[key] = v;
        return v;
    }

    // one raster launch per tile shape when each frame has its own shape
    cudaError_t launch_mixed_raster(const QueueBatch& b, cudaStream_t s, bool trim)
    {
        for (int k = 0; k < kQRasterShapes; k++) {
            QueueBatch bb = b;
            bb.rtw = kQRasterTW[k];
            bb.rth = kQRasterTH[k];
            bb.rbase = kQMixedBase;
            const int bps = blocks_per_sm(QS_RASTER, bb);
            if (bps <= 0) return cudaErrorInvalidConfiguration;
            int blocks = sms * bps;
            if (trim) {
                const uint32_t t = total[kQMixedBase + k];
                if (t == 0) continue;
                blocks = (int)std::min<uint32_t>((uint32_t)blocks, (t + bb.gran[QS_RASTER] - 1) / bb.gran[QS_RASTER]);
            }
            const cudaError_t e = queue_raster(bb, blocks, s);
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    }

    cudaError_t launch(int stage, const QueueBatch& b, cudaStream_t s, bool trim)
    {
        if (stage == QS_RASTER && b.rtw == 0) return launch_mixed_raster(b, s, trim);
        const int bps = blocks_per_sm(stage, b);
        if (bps <= 0) return cudaErrorInvalidConfiguration;
        int blocks = sms * bps;
        if (trim) {
            const uint32_t t = stage == QS_RASTER ? total[QS_RASTER + raster_shape_index(b.rtw, b.rth)] : total[stage];
            const uint32_t need = (t + b.gran[stage] - 1) / b.gran[stage];
            blocks = (int)std::max<uint32_t>(1, std::min<uint32_t>((uint32_t)blocks, need));
        }
        switch (stage) {
        case QS_GRAPH: return queue_graph(b, blocks, s);
        case QS_HEUR: return queue_heuristics(b, blocks, s);
        case QS_LABEL: return queue_labels(b, blocks, s);
        default: return queue_raster(b, blocks, s);
        }
    }

    QueueBatch batch_for(const QueueShape& sh) const
    {
        QueueBatch b = q;
        for (int st = 0; st < QS_COUNT; st++) b.gran[st] = sh.gran[st];
        b.rtw = sh.rtw;
        b.rth = sh.rth;
        b.rbase = sh.rtw == 0 ? kQMixedBase : QS_RASTER;
        return b;
    }

    depix_status tune(cudaStream_t s, QueueShape* out);
    depix_status graph_for(cudaGraphExec_t* out);
};

depix_status queue_runner_create(int cap, QueueRunner** out)
{
    *out = nullptr;
    QueueRunner* r = new (std::nothrow) QueueRunner();
    if (!r) return DEPIX_ERR_ALLOC;
    r->cap = cap;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&r->sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = dev_alloc(&r->d_desc, desc_bytes(cap));
    if (e == cudaSuccess) e = dev_alloc(&r->d_counters, QC_COUNT * sizeof(int));
    for (int k = 0; k < kSlots && e == cudaSuccess; k++) {
        e = cudaHostAlloc(&r->h_slot[k], desc_bytes(cap), cudaHostAllocDefault);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&r->slot_copied[k], cudaEventDisableTiming);
    }
    for (int k = 0; k <= QS_COUNT && e == cudaSuccess; k++) e = cudaEventCreate(&r->tev[k]);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&r->capture_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        cudaGetLastError();
        delete r;
        set_last_error(std::string("queue set-up: ") + cudaGetErrorString(e));
        return DEPIX_ERR_ALLOC;
    }
    *out = r;
    return DEPIX_OK;
}

void queue_runner_destroy(QueueRunner* r) { delete r; }

bool queue_has_labels(const QueueRunner* r) { return r->labels; }

void queue_force_shape(QueueRunner* r, const QueueShape* shape)
{
    r->forced = shape != nullptr;
    if (shape) r->force = *shape;
}

QueueShape queue_last_shape(const QueueRunner* r) { return r->shape; }

// Times every candidate shape on the prepared batch (all candidates compute
// the same result, so the batch's outputs stay valid whichever ran last):
// each stage but the raster gets the granularity that ran it fastest, the
// raster the fastest pair of granularity and tile shape.
depix_status QueueRunner::tune(cudaStream_t s, QueueShape* out)
{
    static const int grans[] = {1, 2, 4, 8};
    float best[QS_COUNT] = {1e30f, 1e30f, 1e30f, 1e30f};
    QueueShape pick{{1, 1, 1, 1}, 32, 32};
    auto elapsed = [&](int a, int b, float* ms) -> cudaError_t { return cudaEventElapsedTime(ms, tev[a], tev[b]); };
    // every stage at one granularity, raster in the first shape that launches
    int first_shape = -1;
    for (int k = 0; k < kQRasterShapes && first_shape < 0; k++) {
        QueueShape sh{{1, 1, 1, 1}, kQRasterTW[k], kQRasterTH[k]};
        if (blocks_per_sm(QS_RASTER, batch_for(sh)) > 0) first_shape = k;
    }
    if (first_shape < 0) {
        set_last_error("no raster tile shape fits this scale");
        return DEPIX_ERR_CUDA;
    }
    for (int g : grans) {
        QueueShape sh{{g, g, g, g}, kQRasterTW[first_shape], kQRasterTH[first_shape]};
        const QueueBatch b = batch_for(sh);
        for (int rep = 0; rep < 3; rep++) { // the first repetition warms up
            cudaError_t e = cudaMemsetAsync(d_counters, 0, QC_COUNT * sizeof(int), s);
            for (int st = 0; st < QS_COUNT && e == cudaSuccess; st++) {
                e = cudaEventRecord(tev[st], s);
                if (e == cudaSuccess && (st != QS_LABEL || labels)) e = launch(st, b, s, true);
            }
            if (e == cudaSuccess) e = cudaEventRecord(tev[QS_COUNT], s);
            if (e == cudaSuccess) e = cudaEventSynchronize(tev[QS_COUNT]);
            if (e != cudaSuccess) return fail(e, "tuning run");
            if (rep == 0) continue;
            for (int st = 0; st < QS_COUNT; st++) {
                float ms = 0;
                if ((e = elapsed(st, st + 1, &ms)) != cudaSuccess) return fail(e, "tuning events");
                if (ms < best[st]) {
                    best[st] = ms;
                    pick.gran[st] = g;
                    if (st == QS_RASTER) {
                        pick.rtw = sh.rtw;
                        pick.rth = sh.rth;
                    }
                }
            }
        }
    }
    // the raster alone in the other tile shapes (the graph it reads is done),
    // then with each frame in its own shape (k == kQRasterShapes)
    for (int k = first_shape + 1; k <= kQRasterShapes; k++) {
        for (int g : grans) {
            QueueShape sh{{g, g, g, g}, k < kQRasterShapes ? kQRasterTW[k] : 0,
                          k < kQRasterShapes ? kQRasterTH[k] : 0};
            const QueueBatch b = batch_for(sh);
            if (sh.rtw != 0 && blocks_per_sm(QS_RASTER, b) <= 0) break;
            for (int rep = 0; rep < 3; rep++) {
                cudaError_t e = cudaMemsetAsync(d_counters + QC_RASTER, 0, kQRasterShapes * sizeof(int), s);
                if (e == cudaSuccess) e = cudaEventRecord(tev[0], s);
                if (e == cudaSuccess) e = launch(QS_RASTER, b, s, true);
                if (e == cudaSuccess) e = cudaEventRecord(tev[1], s);
                if (e == cudaSuccess) e = cudaEventSynchronize(tev[1]);
                if (e != cudaSuccess) return fail(e, "tuning run");
                if (rep == 0) continue;
                float ms = 0;
                if ((e = elapsed(0, 1, &ms)) != cudaSuccess) return fail(e, "tuning events");
                if (ms < best[QS_RASTER]) {
                    best[QS_RASTER] = ms;
                    pick.gran[QS_RASTER] = g;
                    pick.rtw = sh.rtw;
                    pick.rth = sh.rth;
                }
            }
        }
    }
    *out = pick;
    return DEPIX_OK;
}

// The graph of the prepared call's scale, label choice and shape: a counter
// reset and the stage kernels, captured once on a private stream.
depix_status QueueRunner::graph_for(cudaGraphExec_t* out)
{
    const uint64_t key = graph_key(q.scale, labels, q.vote, shape);
    auto it = graphs.find(key);
    if (it != graphs.end()) {
        *out = it->second;
        return DEPIX_OK;
    }
    const QueueBatch b = batch_for(shape);
    // occupancy queries (and the raster's shared-memory opt-in) before capture
    for (int st = 0; st < QS_COUNT; st++) {
        if (st == QS_LABEL && !labels) continue;
        bool ok = true;
        if (st == QS_RASTER && b.rtw == 0) {
            for (int k = 0; k < kQRasterShapes; k++) {
                QueueBatch bb = b;
                bb.rtw = kQRasterTW[k];
                bb.rth = kQRasterTH[k];
                ok &= blocks_per_sm(QS_RASTER, bb) > 0;
            }
        } else {
            ok = blocks_per_sm(st, b) > 0;
        }
        if (!ok) {
            set_last_error("a stage kernel cannot launch in this shape");
            return DEPIX_ERR_CUDA;
        }
    }
    cudaError_t e = cudaStreamBeginCapture(capture_stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return fail(e, "cudaStreamBeginCapture");
    e = cudaMemsetAsync(d_counters, 0, QC_COUNT * sizeof(int), capture_stream);
    for (int st = 0; st < QS_COUNT && e == cudaSuccess; st++)
        if (st != QS_LABEL || labels) e = launch(st, b, capture_stream, false);
    cudaGraph_t g = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(capture_stream, &g);
    if (e == cudaSuccess) e = e2;
    cudaGraphExec_t exec = nullptr;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(e, "graph capture");
    }
    graphs[key] = exec;
    *out = exec;
    return DEPIX_OK;
}

depix_status queue_prepare(QueueRunner* r, const QueueCall& c, cudaStream_t s)
{
    if (c.n < 1 || c.n > r->cap) {
        set_last_error("queue batch size out of range");
        return DEPIX_ERR_INVALID_ARG;
    }
    const int n = c.n, slot = r->next_slot;
    // the slot's previous copy must have left host memory before refilling it
    cudaError_t e = cudaEventSynchronize(r->slot_copied[slot]);
    if (e != cudaSuccess) return fail(e, "descriptor slot");
    uint8_t* h = r->h_slot[slot];
    QueueHeader* H = reinterpret_cast<QueueHeader*>(h);
    uint32_t* base = reinterpret_cast<uint32_t*>(h + kHeaderBytes);
    QueueFrame* F = reinterpret_cast<QueueFrame*>(h + kHeaderBytes + prefix_bytes(n));
    uint64_t tot[kQPrefixes] = {};
    uint64_t px = 0;
    for (int f = 0; f < n; f++) {
        const int w = c.w[f], hh = c.h[f];
        F[f] = QueueFrame{c.in_off[f], c.out_off[f], px, w, hh};
        uint32_t t[kQPrefixes] = {tiles(w, hh, kQGraphTW, kQGraphTH), tiles(w, hh, kQHeurTW, kQHeurTH),
                                  tiles(w, hh, kQLabelT, kQLabelT),   tiles(w, hh, kQRasterTW[0], kQRasterTH[0]),
                                  tiles(w, hh, kQRasterTW[1], kQRasterTH[1]),
                                  tiles(w, hh, kQRasterTW[2], kQRasterTH[2]), 0, 0, 0};
        // the frame's own shape: fewest cells processed, each tile's ring included
        int best = 0;
        uint64_t best_cost = ~0ull;
        for (int k = 0; k < kQRasterShapes; k++) {
            const uint64_t cost = (uint64_t)t[QS_RASTER + k] * (kQRasterTW[k] + 2) * (kQRasterTH[k] + 2);
            if (cost < best_cost) {
                best_cost = cost;
                best = k;
            }
        }
        t[kQMixedBase + best] = t[QS_RASTER + best];
        for (int p = 0; p < kQPrefixes; p++) {
            base[p * (n + 1) + f] = (uint32_t)tot[p];
            tot[p] += t[p];
        }
        px += (uint64_t)w * hh;
    }
    for (int p = 0; p < kQPrefixes; p++) {
        if (tot[p] >= kMaxTiles) {
            set_last_error("too many tiles in one batch");
            return DEPIX_ERR_TOO_LARGE;
        }
        base[p * (n + 1) + n] = (uint32_t)tot[p];
        r->total[p] = (uint32_t)tot[p];
    }
    std::memset(H, 0, kHeaderBytes);
    H->n = n;
    H->thr = c.thr;
    H->subdivide = c.subdivide;
    H->img = c.img;
    H->out = c.out;
    H->labels = c.labels;
    H->frames = reinterpret_cast<const QueueFrame*>(r->d_desc + kHeaderBytes + prefix_bytes(n));
    H->base = reinterpret_cast<const uint32_t*>(r->d_desc + kHeaderBytes);
    for (int p = 0; p < kQPrefixes; p++) H->total[p] = r->total[p];
    e = cudaMemcpyAsync(r->d_desc, h, desc_bytes(n), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaEventRecord(r->slot_copied[slot], s);
    if (e != cudaSuccess) return fail(e, "descriptor copy");
    r->next_slot = (slot + 1) % kSlots;

    r->labels = c.labels != nullptr;
    r->q = QueueBatch{reinterpret_cast<const QueueHeader*>(r->d_desc), r->d_counters, c.graph_a, c.graph_b, c.lut,
                      c.scale, {1, 1, 1, 1}, 32, 32, QS_RASTER, c.vote};
    if (r->forced) {
        r->shape = r->force;
        return DEPIX_OK;
    }
    // size bucket: frame count and mean frame size (powers of two), scale, labels
    const uint64_t bucket = (uint64_t)log2_floor((uint64_t)n) | (uint64_t)log2_floor(px / (uint64_t)n) << 8 |
                            (uint64_t)c.scale << 16 | (uint64_t)r->labels << 24 | (uint64_t)c.vote << 25;
    auto it = r->tuned.find(bucket);
    if (it != r->tuned.end()) {
        r->shape = it->second;
        return DEPIX_OK;
    }
    QueueShape sh{};
    DEPIX_TRY_STATUS(r->tune(s, &sh));
    r->tuned[bucket] = sh;
    r->shape = sh;
    return DEPIX_OK;
}

depix_status queue_launch_graph(QueueRunner* r, cudaStream_t s)
{
    cudaGraphExec_t exec = nullptr;
    DEPIX_TRY_STATUS(r->graph_for(&exec));
    cudaError_t e = cudaGraphLaunch(exec, s);
    return e == cudaSuccess ? DEPIX_OK : fail(e, "cudaGraphLaunch");
}

depix_status queue_reset(QueueRunner* r, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(r->d_counters, 0, QC_COUNT * sizeof(int), s);
    return e == cudaSuccess ? DEPIX_OK : fail(e, "counter reset");
}

depix_status queue_launch_stage(QueueRunner* r, int stage, cudaStream_t s)
{
    cudaError_t e = r->launch(stage, r->batch_for(r->shape), s, true);
    return e == cudaSuccess ? DEPIX_OK : fail(e, "queue stage launch");
}

}  // namespace depix
