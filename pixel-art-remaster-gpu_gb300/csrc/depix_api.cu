// depix_api.cu -- host side of the C ABI: argument checks, per-device
// set-up, the frame/batch drivers and the drop-in launch_kernel.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h> // header-only: ranges cost a pointer test unless a profiler is attached

#include "depix_internal.h"

using namespace depix;

namespace {

thread_local std::string t_last_error;

}  // namespace

void depix::set_last_error(const std::string& msg) { t_last_error = msg; }

namespace {
std::atomic<long long> g_live_allocs{0};
std::atomic<int> g_fail_after{-1}; // < 0: never; n: n more allocations succeed, then all fail
}  // namespace

cudaError_t depix::dev_alloc(void** p, size_t bytes)
{
    *p = nullptr;
    int f = g_fail_after.load();
    while (f >= 0) {
        if (f == 0) return cudaErrorMemoryAllocation;
        if (g_fail_after.compare_exchange_weak(f, f - 1)) break;
    }
    cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaSuccess) g_live_allocs++;
    else cudaGetLastError();
    return e;
}

void depix::dev_free(void* p)
{
    if (!p) return;
    if (cudaFree(p) == cudaSuccess) g_live_allocs--;
}

namespace {

depix_status cuda_fail(cudaError_t e, const char* where)
{
    t_last_error = std::string(where) + ": " + cudaGetErrorString(e);
    return DEPIX_ERR_CUDA;
}

depix_status arg_fail(const char* what)
{
    t_last_error = what;
    return DEPIX_ERR_INVALID_ARG;
}

#define DEPIX_CK(call)                                                  \
    do {                                                                \
        cudaError_t e_ = (call);                                        \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);             \
    } while (0)

#define DEPIX_TRY(call)                                                 \
    do {                                                                \
        depix_status st_ = (call);                                      \
        if (st_ != DEPIX_OK) return st_;                                \
    } while (0)

std::mutex g_init_mu;
std::vector<char> g_init_done;

// Builds the cell-pattern tables on the current device once. Uses a private
// stream that it synchronises, so the tables are complete before any later
// work on any stream.
depix_status ensure_tables(cudaStream_t user)
{
    int dev = 0;
    DEPIX_CK(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_init_mu);
    if (dev < (int)g_init_done.size() && g_init_done[dev]) return DEPIX_OK;
    if (user) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        DEPIX_CK(cudaStreamIsCapturing(user, &cs));
        if (cs != cudaStreamCaptureStatusNone) {
            t_last_error = "first use on this device inside a stream capture: call depix_init_device() first";
            return DEPIX_ERR_CAPTURING;
        }
    }
    cudaStream_t s;
    DEPIX_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    cudaError_t e = init_tables(s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    if (e != cudaSuccess) return cuda_fail(e, "init_tables");
    if (dev >= (int)g_init_done.size()) g_init_done.resize(dev + 1, 0);
    g_init_done[dev] = 1;
    return DEPIX_OK;
}

// Per-device, per-scale coverage tables of the hull patterns, built once.
std::mutex g_scale_mu;
std::vector<std::vector<uint32_t*>> g_scale_lut; // [device][scale]

depix_status scale_table(int scale, cudaStream_t user, const uint32_t** out)
{
    int dev = 0;
    DEPIX_CK(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_scale_mu);
    if (dev >= (int)g_scale_lut.size()) g_scale_lut.resize(dev + 1);
    auto& v = g_scale_lut[dev];
    if (v.size() <= (size_t)scale) v.resize(scale + 1, nullptr);
    if (v[scale]) {
        *out = v[scale];
        return DEPIX_OK;
    }
    if (user) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        DEPIX_CK(cudaStreamIsCapturing(user, &cs));
        if (cs != cudaStreamCaptureStatusNone) {
            t_last_error = "first raster at this scale inside a stream capture: run one frame at this scale first";
            return DEPIX_ERR_CAPTURING;
        }
    }
    uint32_t* lut = nullptr;
    if (dev_alloc(&lut, scale_mask_words(scale) * sizeof(uint32_t)) != cudaSuccess) {
        t_last_error = "cudaMalloc of the scale table failed";
        return DEPIX_ERR_ALLOC;
    }
    cudaStream_t s;
    DEPIX_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    cudaError_t e = build_scale_masks(scale, lut, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    if (e != cudaSuccess) {
        dev_free(lut);
        return cuda_fail(e, "build_scale_masks");
    }
    v[scale] = lut;
    *out = lut;
    return DEPIX_OK;
}

depix_status check_size(int w, int h)
{
    if (w < 1 || h < 1) return arg_fail("width and height must be >= 1");
    if ((long long)w * h > (1LL << 30)) return arg_fail("frame larger than 2^30 pixels");
    return DEPIX_OK;
}

depix_status check_image(const uint8_t* img, int w, int h, int ws, int layout)
{
    DEPIX_TRY(check_size(w, h));
    if (!img) return arg_fail("image pointer is NULL");
    if (layout == DEPIX_LAYOUT_BGR) {
        if (ws < 3 * w) return arg_fail("BGR widthstep must be >= 3*width");
    } else if (layout == DEPIX_LAYOUT_RGBA) {
        if (ws < 4 * w || (ws & 3) || (reinterpret_cast<uintptr_t>(img) & 3))
            return arg_fail("RGBA widthstep must be >= 4*width, rows and base 4-byte aligned");
    } else {
        return arg_fail("unknown layout");
    }
    return DEPIX_OK;
}

depix_status check_params(const depix_params* p)
{
    if (!p) return arg_fail("params pointer is NULL");
    if (p->scale < 1 || p->scale > 64) return arg_fail("scale must be in 1..64");
    if (p->tr_y < 0 || p->tr_u < 0 || p->tr_v < 0) return arg_fail("thresholds must be >= 0");
    if (p->vote != 0 && p->vote != 1) return arg_fail("vote must be 0 or 1");
    if (p->yuv != DEPIX_YUV_CUDA && p->yuv != DEPIX_YUV_HOST) return arg_fail("yuv must be DEPIX_YUV_CUDA or DEPIX_YUV_HOST");
    return DEPIX_OK;
}

// the raster addresses samples in 1/256 output pixel with 32-bit integers
constexpr long long kMaxOutSide = 1LL << 22;

depix_status check_out_size(int w, int h, const depix_params* p)
{
    if ((long long)w * p->scale > kMaxOutSide || (long long)h * p->scale > kMaxOutSide)
        return arg_fail("output side beyond 2^22 pixels");
    return DEPIX_OK;
}

inline cudaStream_t S(depix_stream s) { return reinterpret_cast<cudaStream_t>(s); }

// Coverage-mask raster up to scale 12, per-pixel gather beyond.
depix_status raster_launch(const RasterBatch& b, int nframes, cudaStream_t s)
{
    DEPIX_TRY(ensure_tables(s));
    if (b.scale <= kMaxMaskScale) {
        const uint32_t* lut = nullptr;
        DEPIX_TRY(scale_table(b.scale, s, &lut));
        DEPIX_CK(launch_mask_raster(b, nframes, lut, s));
    } else {
        DEPIX_CK(launch_raster(b, nframes, s));
    }
    return DEPIX_OK;
}

}  // namespace

extern "C" {

void depix_default_params(depix_params* p)
{
    if (!p) return;
    p->tr_y = 48;
    p->tr_u = 7;
    p->tr_v = 6;
    p->subdivide = 1;
    p->scale = 4;
    p->vote = 0;
    p->yuv = DEPIX_YUV_CUDA;
}

const char* depix_status_string(depix_status s)
{
    switch (s) {
    case DEPIX_OK: return "ok";
    case DEPIX_ERR_INVALID_ARG: return "invalid argument";
    case DEPIX_ERR_CUDA: return "CUDA error";
    case DEPIX_ERR_ALLOC: return "allocation failed";
    case DEPIX_ERR_TOO_LARGE: return "request exceeds capacity";
    case DEPIX_ERR_TIMEOUT: return "device wait timed out";
    case DEPIX_ERR_CAPTURING: return "set-up needed during stream capture";
    case DEPIX_ERR_STATE: return "device consistency check failed";
    }
    return "unknown status";
}

const char* depix_last_error(void) { return t_last_error.c_str(); }

depix_status depix_init_device(void) { return ensure_tables(nullptr); }

depix_status depix_take_device_faults(int* flags)
{
    if (!flags) return arg_fail("NULL flags");
    *flags = 0;
    int raster = 0, graph = 0, heur = 0;
    DEPIX_CK(take_raster_fault(&raster));
    DEPIX_CK(take_graph_fault(&graph));
    DEPIX_CK(take_heuristics_fault(&heur));
    *flags = (raster ? 1 : 0) | (graph ? 2 : 0) | (heur ? 4 : 0);
    if (*flags) {
        t_last_error = "a bounded device-side wait for a TMA tile load gave up; the tiles of those blocks were "
                       "left unwritten";
        return DEPIX_ERR_TIMEOUT;
    }
    return DEPIX_OK;
}

depix_status depix_debug_fail_allocations(int after)
{
    g_fail_after.store(after < 0 ? -1 : after);
    return DEPIX_OK;
}

depix_status depix_debug_live_allocations(long long* count)
{
    if (!count) return arg_fail("NULL count");
    *count = g_live_allocs.load();
    return DEPIX_OK;
}

depix_status depix_debug_tma_timeout(int enable)
{
    DEPIX_TRY(ensure_tables(nullptr));
    DEPIX_CK(set_graph_tma_timeout_test(enable));
    return DEPIX_OK;
}

depix_status depix_graph(const uint8_t* d_img, int w, int h, int widthstep, depix_layout layout,
                         const depix_params* p, int fuse_trivial, uint8_t* d_graph, depix_stream s)
{
    DEPIX_TRY(check_image(d_img, w, h, widthstep, layout));
    DEPIX_TRY(check_params(p));
    if (!d_graph) return arg_fail("graph pointer is NULL");
    FrameBatch b{d_img, 0, d_graph, 0, w, h, widthstep, (int)layout};
    DEPIX_CK(launch_graph(b, 1, pack_thresholds(p->tr_y, p->tr_u, p->tr_v, p->yuv), fuse_trivial != 0, S(s)));
    return DEPIX_OK;
}

depix_status depix_resolve_trivial(uint8_t* d_graph, int w, int h, depix_stream s)
{
    DEPIX_TRY(check_size(w, h));
    if (!d_graph) return arg_fail("graph pointer is NULL");
    DEPIX_CK(launch_trivial(d_graph, w, h, S(s)));
    return DEPIX_OK;
}

depix_status depix_resolve_heuristics(const uint8_t* d_snapshot, int w, int h, uint8_t* d_out, depix_stream s)
{
    DEPIX_TRY(check_size(w, h));
    if (!d_snapshot || !d_out) return arg_fail("graph pointer is NULL");
    if (d_snapshot == d_out) return arg_fail("snapshot and output must be distinct buffers");
    GraphBatch b{d_snapshot, d_out, 0, w, h};
    DEPIX_CK(launch_heuristics(b, 1, S(s)));
    return DEPIX_OK;
}

depix_status depix_resolve_heuristics_vote(const uint8_t* d_snapshot, int w, int h, uint8_t* d_out, depix_stream s)
{
    DEPIX_TRY(check_size(w, h));
    if (!d_snapshot || !d_out) return arg_fail("graph pointer is NULL");
    if (d_snapshot == d_out) return arg_fail("snapshot and output must be distinct buffers");
    GraphBatch b{d_snapshot, d_out, 0, w, h, 1};
    DEPIX_CK(launch_heuristics(b, 1, S(s)));
    return DEPIX_OK;
}

depix_status depix_cells(const uint8_t* d_graph, int w, int h, float* d_diagram, int* d_edge_count, depix_stream s)
{
    DEPIX_TRY(check_size(w, h));
    if (!d_graph || !d_diagram || !d_edge_count) return arg_fail("NULL pointer");
    DEPIX_TRY(ensure_tables(S(s)));
    DEPIX_CK(launch_cells(d_graph, w, h, d_diagram, d_edge_count, S(s)));
    return DEPIX_OK;
}

depix_status depix_subdivide(const uint8_t* d_img, int w, int h, int widthstep, depix_layout layout,
                             const uint8_t* d_graph, const float* d_diagram_snap, const int* d_edge_count_snap,
                             float* d_diagram, int* d_edge_count, depix_stream s)
{
    DEPIX_TRY(check_image(d_img, w, h, widthstep, layout));
    if (!d_graph || !d_diagram_snap || !d_edge_count_snap || !d_diagram || !d_edge_count)
        return arg_fail("NULL pointer");
    DEPIX_CK(launch_subdivide(d_img, w, h, widthstep, layout, d_graph, d_diagram_snap, d_edge_count_snap, d_diagram,
                              d_edge_count, S(s)));
    return DEPIX_OK;
}

depix_status depix_triangulate(float* d_diagram, const int* d_edge_count, int w, int h, depix_stream s)
{
    DEPIX_TRY(check_size(w, h));
    if (!d_diagram || !d_edge_count) return arg_fail("NULL pointer");
    DEPIX_CK(launch_triangulate(d_diagram, d_edge_count, w, h, S(s)));
    return DEPIX_OK;
}

depix_status depix_emit_vbo(const uint8_t* d_img, int w, int h, int widthstep, depix_layout layout,
                            const float* d_diagram, const int* d_edge_count, float* d_pos, uint8_t* d_col,
                            depix_stream s)
{
    DEPIX_TRY(check_image(d_img, w, h, widthstep, layout));
    if (!d_diagram || !d_edge_count) return arg_fail("NULL pointer");
    DEPIX_CK(launch_emit(d_img, w, h, widthstep, layout, d_diagram, d_edge_count, d_pos, d_col, S(s)));
    return DEPIX_OK;
}

depix_status depix_label_components(const uint8_t* d_graph, int w, int h, int32_t* d_labels, depix_stream s)
{
    DEPIX_TRY(check_size(w, h));
    if (!d_graph || !d_labels) return arg_fail("NULL pointer");
    DEPIX_CK(launch_labels(d_graph, d_labels, w, h, 1, 0, S(s)));
    return DEPIX_OK;
}

depix_status depix_border_walks(const uint8_t* d_graph, int w, int h, int nframes, uint8_t* d_scratch, int32_t* d_nodes,
                                int8_t* d_edges, int32_t* d_offsets, int max_nodes, int max_walks, int32_t* d_counts,
                                depix_stream s)
{
    DEPIX_TRY(check_size(w, h));
    if (nframes < 1) return arg_fail("nframes must be >= 1");
    if (max_nodes < 1 || max_walks < 1) return arg_fail("capacities must be >= 1");
    if (!d_graph || !d_scratch || !d_nodes || !d_edges || !d_offsets || !d_counts) return arg_fail("NULL pointer");
    DEPIX_CK(launch_border_walks(d_graph, w, h, nframes, d_scratch, d_nodes, d_edges, d_offsets, max_nodes, max_walks,
                                 d_counts, S(s)));
    return DEPIX_OK;
}

depix_status depix_yuv_words(const uint8_t* d_px3, size_t n, int yuv, uint32_t* d_words, depix_stream s)
{
    if (n && (!d_px3 || !d_words)) return arg_fail("NULL pointer");
    if (yuv != DEPIX_YUV_CUDA && yuv != DEPIX_YUV_HOST) return arg_fail("yuv must be DEPIX_YUV_CUDA or DEPIX_YUV_HOST");
    DEPIX_CK(launch_yuv_words(d_px3, n, yuv, d_words, S(s)));
    return DEPIX_OK;
}

depix_status depix_pattern_tables(uint64_t* h_hull, uint64_t* h_tri)
{
    if (!h_hull || !h_tri) return arg_fail("NULL pointer");
    DEPIX_TRY(ensure_tables(nullptr));
    DEPIX_CK(copy_tables(h_hull, h_tri));
    return DEPIX_OK;
}

depix_status depix_raster(const uint8_t* d_img, int w, int h, int widthstep, depix_layout layout,
                          const uint8_t* d_graph, const depix_params* p, uint8_t* d_out, depix_stream s)
{
    DEPIX_TRY(check_image(d_img, w, h, widthstep, layout));
    DEPIX_TRY(check_params(p));
    if (!d_graph || !d_out) return arg_fail("NULL pointer");
    DEPIX_TRY(check_out_size(w, h, p));
    DEPIX_TRY(ensure_tables(S(s)));
    RasterBatch b{d_img, 0, d_graph, 0, d_out, 0, w, h, widthstep, (int)layout, p->scale, p->subdivide};
    DEPIX_TRY(raster_launch(b, 1, S(s)));
    return DEPIX_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ context

struct depix_context {
    int device = 0;
    size_t max_pixels = 0;
    int max_frames = 0;
    uint8_t* graph_a = nullptr; // after graph + trivial, max_frames slots of max_pixels
    uint8_t* graph_b = nullptr; // resolved
    // device staging of the host-buffer batch call
    uint8_t* stage_in = nullptr;
    size_t stage_in_bytes = 0;
    uint8_t* stage_out = nullptr;
    size_t stage_out_bytes = 0;
    int32_t* stage_labels = nullptr;
    size_t stage_label_count = 0;
    // per-stage event timing
    bool timing = false;
    struct Mark {
        int stage;
        int launches;
        cudaEvent_t a, b;
    };
    std::vector<Mark> marks;
    std::vector<cudaEvent_t> spare;
    double ms[DEPIX_STAGE_COUNT] = {};
    long long launches[DEPIX_STAGE_COUNT] = {};
    long long calls[DEPIX_STAGE_COUNT] = {};
    // host-buffer batches: copy-back stream and per-chunk events
    cudaStream_t copy_stream = nullptr;
    std::vector<cudaEvent_t> chunk_done;
    // uneven batches (created on the first one)
    QueueRunner* queue = nullptr;
    bool shape_forced = false;
    QueueShape shape{};

    cudaEvent_t take_event()
    {
        if (!spare.empty()) {
            cudaEvent_t e = spare.back();
            spare.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        cudaEventCreate(&e);
        return e;
    }
};

namespace {

const char* const kStageName[DEPIX_STAGE_COUNT] = {"depix graph", "depix heuristics", "depix labels",
                                                   "depix raster"};

// Brackets one stage's launches with an NVTX range (host side, seen by
// profilers) and, when the context is timing, with CUDA events.
struct StageTimer {
    depix_context* c;
    int stage, launches;
    cudaStream_t s;
    cudaEvent_t a = nullptr;
    StageTimer(depix_context* c_, int stage_, int launches_, cudaStream_t s_)
        : c(c_), stage(stage_), launches(launches_), s(s_)
    {
        nvtxRangePushA(kStageName[stage]);
        if (c->timing) {
            a = c->take_event();
            cudaEventRecord(a, s);
        }
    }
    ~StageTimer()
    {
        nvtxRangePop();
        if (!c->timing || !a) return;
        cudaEvent_t b = c->take_event();
        cudaEventRecord(b, s);
        c->marks.push_back({stage, launches, a, b});
    }
};

// Raster of a context call.
depix_status ctx_raster(depix_context* c, const RasterBatch& rb, int nframes, cudaStream_t s)
{
    StageTimer t(c, DEPIX_STAGE_RASTER, 1, s);
    DEPIX_TRY(raster_launch(rb, nframes, s));
    return DEPIX_OK;
}

depix_status ensure_staging(depix_context* c, size_t in_bytes, size_t out_bytes, size_t labels)
{
    if (in_bytes > c->stage_in_bytes) {
        dev_free(c->stage_in);
        c->stage_in = nullptr;
        c->stage_in_bytes = 0;
        if (dev_alloc(&c->stage_in, in_bytes) != cudaSuccess) {
            t_last_error = "cudaMalloc of input staging failed";
            return DEPIX_ERR_ALLOC;
        }
        c->stage_in_bytes = in_bytes;
    }
    if (out_bytes > c->stage_out_bytes) {
        dev_free(c->stage_out);
        c->stage_out = nullptr;
        c->stage_out_bytes = 0;
        if (dev_alloc(&c->stage_out, out_bytes) != cudaSuccess) {
            t_last_error = "cudaMalloc of output staging failed";
            return DEPIX_ERR_ALLOC;
        }
        c->stage_out_bytes = out_bytes;
    }
    if (labels > c->stage_label_count) {
        dev_free(c->stage_labels);
        c->stage_labels = nullptr;
        c->stage_label_count = 0;
        if (dev_alloc(&c->stage_labels, labels * sizeof(int32_t)) != cudaSuccess) {
            t_last_error = "cudaMalloc of label staging failed";
            return DEPIX_ERR_ALLOC;
        }
        c->stage_label_count = labels;
    }
    return DEPIX_OK;
}

struct BatchShape {
    bool uniform = true, strided = true;
    size_t total_pixels = 0;
};

depix_status check_batch(depix_context* ctx, int n, const int* w, const int* h, const uint64_t* in_offset,
                         const uint64_t* out_offset, BatchShape& shape)
{
    if (n > ctx->max_frames) {
        t_last_error = "more frames than the context capacity";
        return DEPIX_ERR_TOO_LARGE;
    }
    for (int k = 0; k < n; k++) {
        DEPIX_TRY(check_size(w[k], h[k]));
        if ((size_t)w[k] * h[k] > ctx->max_pixels) {
            t_last_error = "frame larger than the context capacity";
            return DEPIX_ERR_TOO_LARGE;
        }
        if ((in_offset[k] & 15) || (out_offset[k] & 15)) return arg_fail("offsets must be multiples of 16");
        if (w[k] != w[0] || h[k] != h[0]) shape.uniform = false;
        shape.total_pixels += (size_t)w[k] * h[k];
    }
    if (n > 1) {
        uint64_t is = in_offset[1] - in_offset[0], os = out_offset[1] - out_offset[0];
        for (int k = 1; k < n; k++)
            if (in_offset[k] - in_offset[k - 1] != is || out_offset[k] - out_offset[k - 1] != os) shape.strided = false;
    }
    return DEPIX_OK;
}

depix_status run_batch(depix_context* ctx, int n, const int* w, const int* h, const uint64_t* in_offset,
                       const uint64_t* out_offset, const uint8_t* d_img, const depix_params* p, uint8_t* d_out,
                       int32_t* d_labels, const BatchShape& shape, cudaStream_t s)
{
    const uint32_t thr = pack_thresholds(p->tr_y, p->tr_u, p->tr_v, p->yuv);
    if (shape.uniform && shape.strided) {
        // equal sizes at equal strides: one launch per stage for the batch
        size_t px = (size_t)w[0] * h[0];
        uint64_t is = n > 1 ? in_offset[1] - in_offset[0] : 0, os = n > 1 ? out_offset[1] - out_offset[0] : 0;
        const uint8_t* img0 = d_img + in_offset[0];
        {
            StageTimer t(ctx, DEPIX_STAGE_GRAPH, 1, s);
            FrameBatch gb{img0, (size_t)is, ctx->graph_a, px, w[0], h[0], 4 * w[0], DEPIX_LAYOUT_RGBA};
            DEPIX_CK(launch_graph(gb, n, thr, true, s));
        }
        {
            // with labels, each heuristics tile also makes its local labels
            StageTimer t(ctx, DEPIX_STAGE_HEURISTICS, 1, s);
            GraphBatch hb{ctx->graph_a, ctx->graph_b, px, w[0], h[0], p->vote};
            if (d_labels) DEPIX_CK(launch_heuristics_labels(hb, n, d_labels, s));
            else DEPIX_CK(launch_heuristics(hb, n, s));
        }
        if (d_labels) {
            StageTimer t(ctx, DEPIX_STAGE_LABELS, 2, s);
            DEPIX_CK(launch_labels_after_heuristics(ctx->graph_b, d_labels, w[0], h[0], n, px, s));
        }
        {
            RasterBatch rb{img0, (size_t)is, ctx->graph_b, px, d_out + out_offset[0], (size_t)os, w[0], h[0],
                           4 * w[0], DEPIX_LAYOUT_RGBA, p->scale, p->subdivide};
            DEPIX_TRY(ctx_raster(ctx, rb, n, s));
        }
        return DEPIX_OK;
    }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    DEPIX_CK(cudaStreamIsCapturing(s, &cs));
    if (p->scale <= kMaxMaskScale && cs == cudaStreamCaptureStatusNone) {
        // uneven frames: persistent kernels over one tile queue per stage
        if (!ctx->queue) DEPIX_TRY(queue_runner_create(ctx->max_frames, &ctx->queue));
        queue_force_shape(ctx->queue, ctx->shape_forced ? &ctx->shape : nullptr);
        const uint32_t* lut = nullptr;
        DEPIX_TRY(ensure_tables(s));
        DEPIX_TRY(scale_table(p->scale, s, &lut));
        const QueueCall c{n, w, h, in_offset, out_offset, d_img, d_out, d_labels, thr, p->subdivide, p->scale,
                          p->vote, lut, ctx->graph_a, ctx->graph_b};
        DEPIX_TRY(queue_prepare(ctx->queue, c, s));
        if (!ctx->timing) return queue_launch_graph(ctx->queue, s);
        DEPIX_TRY(queue_reset(ctx->queue, s));
        static const int kStage[QS_COUNT] = {DEPIX_STAGE_GRAPH, DEPIX_STAGE_HEURISTICS, DEPIX_STAGE_LABELS,
                                             DEPIX_STAGE_RASTER};
        for (int st = 0; st < QS_COUNT; st++) {
            if (st == QS_LABEL && !d_labels) continue;
            StageTimer t(ctx, kStage[st], st == QS_LABEL ? 2 : 1, s);
            DEPIX_TRY(queue_launch_stage(ctx->queue, st, s));
        }
        return DEPIX_OK;
    }
    // uneven frames while capturing, or beyond the mask raster's scales: one
    // launch per stage and frame
    size_t goff = 0, loff = 0;
    for (int k = 0; k < n; k++) {
        const uint8_t* img = d_img + in_offset[k];
        {
            StageTimer t(ctx, DEPIX_STAGE_GRAPH, 1, s);
            FrameBatch gb{img, 0, ctx->graph_a + goff, 0, w[k], h[k], 4 * w[k], DEPIX_LAYOUT_RGBA};
            DEPIX_CK(launch_graph(gb, 1, thr, true, s));
        }
        {
            StageTimer t(ctx, DEPIX_STAGE_HEURISTICS, 1, s);
            GraphBatch hb{ctx->graph_a + goff, ctx->graph_b + goff, 0, w[k], h[k], p->vote};
            if (d_labels) DEPIX_CK(launch_heuristics_labels(hb, 1, d_labels + loff, s));
            else DEPIX_CK(launch_heuristics(hb, 1, s));
        }
        if (d_labels) {
            StageTimer t(ctx, DEPIX_STAGE_LABELS, 2, s);
            DEPIX_CK(launch_labels_after_heuristics(ctx->graph_b + goff, d_labels + loff, w[k], h[k], 1, 0, s));
        }
        {
            RasterBatch rb{img, 0, ctx->graph_b + goff, 0, d_out + out_offset[k], 0, w[k], h[k], 4 * w[k],
                           DEPIX_LAYOUT_RGBA, p->scale, p->subdivide};
            DEPIX_TRY(ctx_raster(ctx, rb, 1, s));
        }
        goff += ctx->max_pixels;
        loff += (size_t)w[k] * h[k];
    }
    return DEPIX_OK;
}

// ---- host-buffer batches in chunks: the copy back of one chunk overlaps the
// upload and the kernels of the next (the device-to-host link, not the
// kernels, bounds a host-buffer batch of x4 rasters)

constexpr int kMinChunkFrames = 16, kMaxChunks = 8;

// frames in order, each input and output range after the previous one's
bool frames_in_order(int n, const int* w, const int* h, const uint64_t* in_offset, const uint64_t* out_offset,
                     int scale)
{
    for (int k = 1; k < n; k++) {
        const uint64_t ib = (uint64_t)w[k - 1] * h[k - 1] * 4, ob = ib * (uint64_t)scale * scale;
        if (in_offset[k] < in_offset[k - 1] + ib || out_offset[k] < out_offset[k - 1] + ob) return false;
    }
    return true;
}

BatchShape chunk_shape(int n, const int* w, const int* h, const uint64_t* in_offset, const uint64_t* out_offset)
{
    BatchShape sh;
    for (int k = 0; k < n; k++) {
        if (w[k] != w[0] || h[k] != h[0]) sh.uniform = false;
        sh.total_pixels += (size_t)w[k] * h[k];
    }
    for (int k = 2; k < n; k++)
        if (in_offset[k] - in_offset[k - 1] != in_offset[1] - in_offset[0] ||
            out_offset[k] - out_offset[k - 1] != out_offset[1] - out_offset[0])
            sh.strided = false;
    return sh;
}

depix_status batch_host_pipelined(depix_context* ctx, int n, const int* w, const int* h, const uint64_t* in_offset,
                                  const uint64_t* out_offset, const uint8_t* h_img, const depix_params* p,
                                  uint8_t* h_out, int32_t* h_labels, cudaStream_t s)
{
    if (!ctx->copy_stream) DEPIX_CK(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
    while ((int)ctx->chunk_done.size() < kMaxChunks + 1) {
        cudaEvent_t e = nullptr;
        DEPIX_CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ctx->chunk_done.push_back(e);
    }
    const int chunks = std::min(kMaxChunks, n / kMinChunkFrames);
    const size_t s2 = (size_t)p->scale * p->scale;
    size_t lab = 0;
    for (int c = 0; c < chunks; c++) {
        const int a = (int)((long long)n * c / chunks), b = (int)((long long)n * (c + 1) / chunks);
        const size_t ib_last = (size_t)w[b - 1] * h[b - 1] * 4;
        const size_t in0 = in_offset[a], in1 = in_offset[b - 1] + ib_last;
        const size_t out0 = out_offset[a], out1 = out_offset[b - 1] + ib_last * s2;
        DEPIX_CK(cudaMemcpyAsync(ctx->stage_in + in0, h_img + in0, in1 - in0, cudaMemcpyHostToDevice, s));
        const BatchShape sh = chunk_shape(b - a, w + a, h + a, in_offset + a, out_offset + a);
        DEPIX_TRY(run_batch(ctx, b - a, w + a, h + a, in_offset + a, out_offset + a, ctx->stage_in, p,
                            ctx->stage_out, h_labels ? ctx->stage_labels + lab : nullptr, sh, s));
        DEPIX_CK(cudaEventRecord(ctx->chunk_done[c], s));
        DEPIX_CK(cudaStreamWaitEvent(ctx->copy_stream, ctx->chunk_done[c], 0));
        DEPIX_CK(cudaMemcpyAsync(h_out + out0, ctx->stage_out + out0, out1 - out0, cudaMemcpyDeviceToHost,
                                 ctx->copy_stream));
        if (h_labels)
            DEPIX_CK(cudaMemcpyAsync(h_labels + lab, ctx->stage_labels + lab, sh.total_pixels * sizeof(int32_t),
                                     cudaMemcpyDeviceToHost, ctx->copy_stream));
        lab += sh.total_pixels;
    }
    // the caller's stream resumes after the last copy
    DEPIX_CK(cudaEventRecord(ctx->chunk_done[kMaxChunks], ctx->copy_stream));
    DEPIX_CK(cudaStreamWaitEvent(s, ctx->chunk_done[kMaxChunks], 0));
    DEPIX_CK(cudaStreamSynchronize(s));
    return DEPIX_OK;
}

}  // namespace

extern "C" {

depix_status depix_context_create(depix_context** out, size_t max_pixels, int max_frames)
{
    if (!out) return arg_fail("NULL context pointer");
    *out = nullptr;
    if (max_pixels < 1 || max_frames < 1) return arg_fail("capacity must be >= 1");
    DEPIX_TRY(ensure_tables(nullptr));
    depix_context* c = new (std::nothrow) depix_context();
    if (!c) return DEPIX_ERR_ALLOC;
    DEPIX_CK(cudaGetDevice(&c->device));
    c->max_pixels = max_pixels;
    c->max_frames = max_frames;
    size_t bytes = max_pixels * (size_t)max_frames;
    if (dev_alloc(&c->graph_a, bytes) != cudaSuccess || dev_alloc(&c->graph_b, bytes) != cudaSuccess) {
        dev_free(c->graph_a);
        delete c;
        t_last_error = "cudaMalloc of context scratch failed";
        return DEPIX_ERR_ALLOC;
    }
    *out = c;
    return DEPIX_OK;
}

depix_status depix_context_destroy(depix_context* c)
{
    if (!c) return DEPIX_OK;
    dev_free(c->graph_a);
    dev_free(c->graph_b);
    dev_free(c->stage_in);
    dev_free(c->stage_out);
    dev_free(c->stage_labels);
    if (c->queue) queue_runner_destroy(c->queue);
    if (c->copy_stream) {
        cudaStreamSynchronize(c->copy_stream);
        cudaStreamDestroy(c->copy_stream);
    }
    for (auto e : c->chunk_done) cudaEventDestroy(e);
    for (auto& m : c->marks) {
        cudaEventDestroy(m.a);
        cudaEventDestroy(m.b);
    }
    for (auto e : c->spare) cudaEventDestroy(e);
    delete c;
    return DEPIX_OK;
}

depix_status depix_context_set_launch_shape(depix_context* c, int gran, int tile_w, int tile_h)
{
    if (!c) return arg_fail("NULL context");
    if (gran == 0) {
        c->shape_forced = false;
        return DEPIX_OK;
    }
    if (gran != 1 && gran != 2 && gran != 4 && gran != 8) return arg_fail("granularity must be 0, 1, 2, 4 or 8");
    if (!((tile_w == 32 && tile_h == 32) || (tile_w == 32 && tile_h == 16) || (tile_w == 16 && tile_h == 16) ||
          (tile_w == 0 && tile_h == 0)))
        return arg_fail("raster tile must be 32x32, 32x16, 16x16 or 0x0 (each frame its own)");
    c->shape = QueueShape{{gran, gran, gran, gran}, tile_w, tile_h};
    c->shape_forced = true;
    return DEPIX_OK;
}

depix_status depix_context_launch_shape(depix_context* c, int* gran, int* tile_w, int* tile_h)
{
    if (!c) return arg_fail("NULL context");
    QueueShape sh = c->queue ? queue_last_shape(c->queue) : QueueShape{{0, 0, 0, 0}, 0, 0};
    if (gran)
        for (int k = 0; k < QS_COUNT; k++) gran[k] = sh.gran[k];
    if (tile_w) *tile_w = sh.rtw;
    if (tile_h) *tile_h = sh.rth;
    return DEPIX_OK;
}

depix_status depix_context_set_timing(depix_context* c, int enable)
{
    if (!c) return arg_fail("NULL context");
    c->timing = enable != 0;
    return DEPIX_OK;
}

depix_status depix_context_stage_times(depix_context* c, double* ms, long long* launches, long long* calls)
{
    if (!c) return arg_fail("NULL context");
    for (auto& m : c->marks) {
        DEPIX_CK(cudaEventSynchronize(m.b));
        float t = 0;
        DEPIX_CK(cudaEventElapsedTime(&t, m.a, m.b));
        c->ms[m.stage] += t;
        c->launches[m.stage] += m.launches;
        c->calls[m.stage] += 1;
        c->spare.push_back(m.a);
        c->spare.push_back(m.b);
    }
    c->marks.clear();
    for (int k = 0; k < DEPIX_STAGE_COUNT; k++) {
        if (ms) ms[k] = c->ms[k];
        if (launches) launches[k] = c->launches[k];
        if (calls) calls[k] = c->calls[k];
        c->ms[k] = 0;
        c->launches[k] = 0;
        c->calls[k] = 0;
    }
    return DEPIX_OK;
}

depix_status depix_frame(depix_context* ctx, const uint8_t* d_img, int w, int h, int widthstep, depix_layout layout,
                         const depix_params* p, uint8_t* d_out, uint8_t* d_graph_out, int32_t* d_labels,
                         depix_stream s_)
{
    if (!ctx) return arg_fail("NULL context");
    DEPIX_TRY(check_image(d_img, w, h, widthstep, layout));
    DEPIX_TRY(check_params(p));
    if ((size_t)w * h > ctx->max_pixels) {
        t_last_error = "frame larger than the context capacity";
        return DEPIX_ERR_TOO_LARGE;
    }
    if (d_out) DEPIX_TRY(check_out_size(w, h, p));
    cudaStream_t s = S(s_);
    uint8_t* resolved = d_graph_out ? d_graph_out : ctx->graph_b;
    {
        StageTimer t(ctx, DEPIX_STAGE_GRAPH, 1, s);
        FrameBatch gb{d_img, 0, ctx->graph_a, 0, w, h, widthstep, (int)layout};
        DEPIX_CK(launch_graph(gb, 1, pack_thresholds(p->tr_y, p->tr_u, p->tr_v, p->yuv), true, s));
    }
    {
        StageTimer t(ctx, DEPIX_STAGE_HEURISTICS, 1, s);
        GraphBatch hb{ctx->graph_a, resolved, 0, w, h, p->vote};
        if (d_labels) DEPIX_CK(launch_heuristics_labels(hb, 1, d_labels, s));
        else DEPIX_CK(launch_heuristics(hb, 1, s));
    }
    if (d_labels) {
        StageTimer t(ctx, DEPIX_STAGE_LABELS, 2, s);
        DEPIX_CK(launch_labels_after_heuristics(resolved, d_labels, w, h, 1, 0, s));
    }
    if (d_out) {
        RasterBatch rb{d_img, 0, resolved, 0, d_out, 0, w, h, widthstep, (int)layout, p->scale, p->subdivide};
        DEPIX_TRY(ctx_raster(ctx, rb, 1, s));
    }
    return DEPIX_OK;
}

depix_status depix_batch(depix_context* ctx, int n, const int* w, const int* h, const uint64_t* in_offset,
                         const uint64_t* out_offset, const uint8_t* d_img, const depix_params* p, uint8_t* d_out,
                         int32_t* d_labels, depix_stream s)
{
    if (!ctx) return arg_fail("NULL context");
    if (n < 0 || (n > 0 && (!w || !h || !in_offset || !out_offset || !d_img || !d_out)))
        return arg_fail("bad batch arguments");
    DEPIX_TRY(check_params(p));
    if (n == 0) return DEPIX_OK;
    BatchShape shape;
    DEPIX_TRY(check_batch(ctx, n, w, h, in_offset, out_offset, shape));
    for (int k = 0; k < n; k++) DEPIX_TRY(check_out_size(w[k], h[k], p));
    return run_batch(ctx, n, w, h, in_offset, out_offset, d_img, p, d_out, d_labels, shape, S(s));
}

depix_status depix_batch_host(depix_context* ctx, int n, const int* w, const int* h, const uint64_t* in_offset,
                              const uint64_t* out_offset, const uint8_t* h_img, size_t in_bytes,
                              const depix_params* p, uint8_t* h_out, size_t out_bytes, int32_t* h_labels,
                              depix_stream s_)
{
    if (!ctx) return arg_fail("NULL context");
    if (n < 0 || (n > 0 && (!w || !h || !in_offset || !out_offset || !h_img || !h_out)))
        return arg_fail("bad batch arguments");
    DEPIX_TRY(check_params(p));
    if (n == 0) return DEPIX_OK;
    BatchShape shape;
    DEPIX_TRY(check_batch(ctx, n, w, h, in_offset, out_offset, shape));
    for (int k = 0; k < n; k++) DEPIX_TRY(check_out_size(w[k], h[k], p));
    for (int k = 0; k < n; k++) {
        // compared without forming offset + size, which a corrupt offset
        // near 2^64 would wrap around
        size_t ib = (size_t)w[k] * h[k] * 4, ob = ib * (size_t)p->scale * p->scale;
        if (in_offset[k] > in_bytes || ib > in_bytes - in_offset[k] || out_offset[k] > out_bytes ||
            ob > out_bytes - out_offset[k])
            return arg_fail("a frame lies outside the host buffers");
    }
    DEPIX_TRY(ensure_staging(ctx, in_bytes, out_bytes, h_labels ? shape.total_pixels : 0));
    cudaStream_t s = S(s_);
    if (n >= 2 * kMinChunkFrames && frames_in_order(n, w, h, in_offset, out_offset, p->scale)) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        DEPIX_CK(cudaStreamIsCapturing(s, &cs));
        if (cs == cudaStreamCaptureStatusNone)
            return batch_host_pipelined(ctx, n, w, h, in_offset, out_offset, h_img, p, h_out, h_labels, s);
    }
    DEPIX_CK(cudaMemcpyAsync(ctx->stage_in, h_img, in_bytes, cudaMemcpyHostToDevice, s));
    DEPIX_TRY(run_batch(ctx, n, w, h, in_offset, out_offset, ctx->stage_in, p, ctx->stage_out,
                        h_labels ? ctx->stage_labels : nullptr, shape, s));
    DEPIX_CK(cudaMemcpyAsync(h_out, ctx->stage_out, out_bytes, cudaMemcpyDeviceToHost, s));
    if (h_labels)
        DEPIX_CK(cudaMemcpyAsync(h_labels, ctx->stage_labels, shape.total_pixels * sizeof(int32_t),
                                 cudaMemcpyDeviceToHost, s));
    DEPIX_CK(cudaStreamSynchronize(s));
    return DEPIX_OK;
}

}  // extern "C"

// ------------------------------------------------------ drop-in frame driver

namespace {

struct CompatScratch {
    size_t img_bytes = 0, pixels = 0;
    uint8_t* img = nullptr;
    uint8_t* g0 = nullptr;
    uint8_t* g1 = nullptr;
    float* diag = nullptr;
    float* snap = nullptr;
    int* ec = nullptr;
    int* ec_snap = nullptr;
    void release()
    {
        dev_free(img); dev_free(g0); dev_free(g1); dev_free(diag); dev_free(snap); dev_free(ec); dev_free(ec_snap);
        *this = CompatScratch();
    }
    bool reserve(size_t ib, size_t px)
    {
        if (ib <= img_bytes && px <= pixels && img) return true;
        release();
        bool ok = dev_alloc(&img, ib) == cudaSuccess && dev_alloc(&g0, px) == cudaSuccess &&
                  dev_alloc(&g1, px) == cudaSuccess &&
                  dev_alloc(&diag, px * kCell * sizeof(float2)) == cudaSuccess &&
                  dev_alloc(&snap, px * kCell * sizeof(float2)) == cudaSuccess &&
                  dev_alloc(&ec, px * sizeof(int)) == cudaSuccess &&
                  dev_alloc(&ec_snap, px * sizeof(int)) == cudaSuccess;
        if (!ok) {
            cudaGetLastError();
            release();
            return false;
        }
        img_bytes = ib;
        pixels = px;
        return true;
    }
};

std::mutex g_compat_mu;
CompatScratch g_compat;

depix_status compat_run(void* pos, void* colorPos, char* img_data, int w, int h, int ws, int* edge_count_h,
                        char* graph_h, int subdivide, const depix_params* p, depix_point** result)
{
    DEPIX_TRY(check_size(w, h));
    if (!img_data || ws < 3 * w) return arg_fail("bad host image");
    depix_params ref{5, 7, 6, 0, 1, 0, DEPIX_YUV_CUDA};
    if (!p) p = &ref;
    DEPIX_TRY(check_params(p));
    DEPIX_TRY(ensure_tables(nullptr));
    std::lock_guard<std::mutex> lk(g_compat_mu);
    size_t px = (size_t)w * h, ib = (size_t)ws * h;
    if (!g_compat.reserve(ib, px)) {
        t_last_error = "cudaMalloc of compat scratch failed";
        return DEPIX_ERR_ALLOC;
    }
    CompatScratch& c = g_compat;
    cudaStream_t s = 0;
    DEPIX_CK(cudaMemcpyAsync(c.img, img_data, ib, cudaMemcpyHostToDevice, s));
    FrameBatch gb{c.img, 0, c.g0, 0, w, h, ws, DEPIX_LAYOUT_BGR};
    DEPIX_CK(launch_graph(gb, 1, pack_thresholds(p->tr_y, p->tr_u, p->tr_v, p->yuv), true, s));
    GraphBatch hb{c.g0, c.g1, 0, w, h, p->vote};
    DEPIX_CK(launch_heuristics(hb, 1, s));
    DEPIX_CK(launch_cells(c.g1, w, h, c.diag, c.ec, s));
    if (subdivide) {
        DEPIX_CK(cudaMemcpyAsync(c.snap, c.diag, px * kCell * sizeof(float2), cudaMemcpyDeviceToDevice, s));
        DEPIX_CK(cudaMemcpyAsync(c.ec_snap, c.ec, px * sizeof(int), cudaMemcpyDeviceToDevice, s));
        DEPIX_CK(launch_subdivide(c.img, w, h, ws, DEPIX_LAYOUT_BGR, c.g1, c.snap, c.ec_snap, c.diag, c.ec, s));
    }
    DEPIX_CK(launch_triangulate(c.diag, c.ec, w, h, s));
    if (pos || colorPos)
        DEPIX_CK(launch_emit(c.img, w, h, ws, DEPIX_LAYOUT_BGR, c.diag, c.ec, static_cast<float*>(pos),
                             static_cast<uint8_t*>(colorPos), s));
    if (edge_count_h) DEPIX_CK(cudaMemcpyAsync(edge_count_h, c.ec, px * sizeof(int), cudaMemcpyDeviceToHost, s));
    if (graph_h) DEPIX_CK(cudaMemcpyAsync(graph_h, c.g1, px, cudaMemcpyDeviceToHost, s));
    depix_point* out = static_cast<depix_point*>(malloc(px * kCell * sizeof(depix_point)));
    if (!out) {
        cudaStreamSynchronize(s);
        t_last_error = "host malloc failed";
        return DEPIX_ERR_ALLOC;
    }
    cudaError_t e = cudaMemcpyAsync(out, c.diag, px * kCell * sizeof(float2), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        free(out);
        return cuda_fail(e, "compat frame");
    }
    *result = out;
    return DEPIX_OK;
}

}  // namespace

extern "C" {

depix_point* depix_launch_kernel_compat(void* pos, void* colorPos, float, char* img_data, int img_width,
                                        int img_height, int img_widthstep, int* edge_count_h, char* graph_h,
                                        int subdivide, const depix_params* p)
{
    depix_point* r = nullptr;
    if (compat_run(pos, colorPos, img_data, img_width, img_height, img_widthstep, edge_count_h, graph_h, subdivide, p,
                   &r) != DEPIX_OK)
        return nullptr;
    return r;
}

depix_point* launch_kernel(void* pos, void* colorPos, float time, char* img_data, int img_width, int img_height,
                           int img_widthstep, int* edge_count_h, char* graph_h, bool subdivide)
{
    return depix_launch_kernel_compat(pos, colorPos, time, img_data, img_width, img_height, img_widthstep,
                                      edge_count_h, graph_h, subdivide ? 1 : 0, nullptr);
}

}  // extern "C"
