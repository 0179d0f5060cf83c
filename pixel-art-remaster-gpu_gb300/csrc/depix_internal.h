// depix_internal.h -- declarations shared by the library's translation units.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <cuda_runtime.h>

#include "depix_device.cuh"

namespace depix {

// One frame of a stage call.
struct FrameRef {
    const uint8_t* img;
    int w, h, ws;
    uint8_t* graph;
};

// Equal-size frames laid out at fixed strides (a single frame: strides unused).
struct FrameBatch {
    const uint8_t* img;
    size_t img_stride;   // bytes between frames' images
    uint8_t* graph;
    size_t graph_stride; // bytes between frames' graphs
    int w, h, ws, layout;
    __device__ __forceinline__ FrameRef frame(int z) const
    {
        return FrameRef{img + img_stride * z, w, h, ws, graph + graph_stride * z};
    }
};

struct GraphBatch {
    const uint8_t* snap;
    uint8_t* out;
    size_t frame_stride;
    int w, h;
    int vote = 0; // heuristics: 0 the reference's ordered tests, 1 the weighted vote
};

// Raster of equal-size frames.
struct RasterBatch {
    const uint8_t* img;
    size_t img_stride;
    const uint8_t* graph;
    size_t graph_stride;
    uint8_t* out;
    size_t out_stride;
    int w, h, ws, layout;
    int scale;
    int subdivide;
};

// ------------------------------------------------ uneven batches (queue)
//
// Frames of any sizes in one launch per stage: per-frame descriptors and,
// per stage, the prefix sums of the frames' tile counts live in device
// memory; persistent kernels pull tile indices from a counter and find a
// tile's frame by binary search over the prefix.
enum QueueStage { QS_GRAPH = 0, QS_HEUR = 1, QS_LABEL = 2, QS_RASTER = 3, QS_COUNT = 4 };
// the raster has one counter per tile shape (QC_RASTER + shape index)
enum QueueCounter { QC_GRAPH = 0, QC_HEUR, QC_MERGE, QC_FLATTEN, QC_RASTER, QC_COUNT = QC_RASTER + 3 };

struct QueueFrame {
    uint64_t in_off;  // bytes into the batch input (RGBA8, rows 4*w bytes)
    uint64_t out_off; // bytes into the batch raster output
    uint64_t px_off;  // pixels into the scratch graphs and the labels
    int w, h;
};

// Per-call descriptor block, copied to the device in one piece: this header,
// then the QS_COUNT prefix arrays (n + 1 entries each), then the frames.
struct QueueHeader {
    int n;            // frames in this batch
    uint32_t thr;     // packed similarity thresholds
    int subdivide;
    int pad_;
    const uint8_t* img;
    uint8_t* out;
    int32_t* labels;
    const QueueFrame* frames;
    const uint32_t* base;     // base[prefix * (n + 1) + f]: first tile of frame f
    uint32_t total[9];        // tiles per prefix (kQPrefixes)
};

// Kernel parameters: fixed for a context, a scale and a launch shape, so a
// captured graph replays them for every batch.
struct QueueBatch {
    const QueueHeader* hdr;
    int* counters;        // QC_COUNT tile counters, zeroed before each batch
    uint8_t* graph_a;     // after graph + trivial
    uint8_t* graph_b;     // resolved
    const uint32_t* lut;  // scale table
    int scale;
    int gran[QS_COUNT];   // tiles pulled per counter step, per stage
    int rtw, rth;         // raster tile (cells); 0, 0: each frame in its own shape
    int rbase;            // first raster prefix: QS_RASTER (one shape for all) or kQMixedBase
    int vote;             // heuristics by the weighted vote (GraphBatch::vote)
};

// tiles of a frame per stage; the raster has three tile shapes, each with its
// own prefix (QS_RASTER + shape index), so a batch can be raster-timed in
// every shape without new descriptors, and three more prefixes in which each
// frame counts only in the shape assigned to it (kQMixedBase + shape index:
// the shape with the fewest cells to process, ring included)
constexpr int kQGraphTW = 64, kQGraphTH = 16, kQHeurTW = 64, kQHeurTH = 16, kQLabelT = 32;
constexpr int kQRasterShapes = 3;
constexpr int kQMixedBase = QS_RASTER + kQRasterShapes;
constexpr int kQPrefixes = kQMixedBase + kQRasterShapes;
static_assert(kQPrefixes == 9, "QueueHeader::total");
constexpr int kQRasterTW[kQRasterShapes] = {32, 32, 16}, kQRasterTH[kQRasterShapes] = {32, 16, 16};
__host__ __device__ constexpr int raster_shape_index(int tw, int th)
{
    return (tw == 32 && th == 32) ? 0 : (tw == 32 ? 1 : 2);
}

class QueueRunner;
struct QueueCall {
    int n;
    const int* w;
    const int* h;
    const uint64_t* in_off;
    const uint64_t* out_off;
    const uint8_t* img;
    uint8_t* out;
    int32_t* labels;      // NULL: no label stage
    uint32_t thr;
    int subdivide, scale;
    int vote;
    const uint32_t* lut;
    uint8_t* graph_a;
    uint8_t* graph_b;
};
// Launch shape of the queue path: granularity per stage and raster tile
// (0 x 0: each frame in the tile shape assigned to it).
struct QueueShape {
    int gran[QS_COUNT];
    int rtw, rth;
};
depix_status queue_runner_create(int cap, QueueRunner** out);
void queue_runner_destroy(QueueRunner* r);
// fills a pinned descriptor slot for the call, copies it to the device on s
// and picks the launch shape (forced, tuned for the batch's size bucket, or
// tuned now by timing the candidates on s)
depix_status queue_prepare(QueueRunner* r, const QueueCall& c, cudaStream_t s);
// the prepared batch as one graph replay, or stage by stage
depix_status queue_launch_graph(QueueRunner* r, cudaStream_t s);
depix_status queue_reset(QueueRunner* r, cudaStream_t s);
depix_status queue_launch_stage(QueueRunner* r, int stage, cudaStream_t s);
bool queue_has_labels(const QueueRunner* r);
void queue_force_shape(QueueRunner* r, const QueueShape* shape); // NULL: tune
QueueShape queue_last_shape(const QueueRunner* r);

cudaError_t queue_graph(const QueueBatch& q, int blocks, cudaStream_t s);
cudaError_t queue_heuristics(const QueueBatch& q, int blocks, cudaStream_t s);
cudaError_t queue_labels(const QueueBatch& q, int blocks, cudaStream_t s);
cudaError_t queue_raster(const QueueBatch& q, int blocks, cudaStream_t s);
int queue_blocks_per_sm(int stage, const QueueBatch& q);
int queue_raster_blocks_per_sm(const QueueBatch& q);

// text returned by depix_last_error() on this thread
void set_last_error(const std::string& msg);

// graph stage
cudaError_t launch_graph(const FrameBatch& b, int nframes, uint32_t thr, bool fuse_trivial, cudaStream_t s);
cudaError_t launch_trivial(uint8_t* g, int w, int h, cudaStream_t s);
cudaError_t launch_border_walks(const uint8_t* graph, int w, int h, int nframes, uint8_t* flags, int32_t* nodes,
                                int8_t* edges, int32_t* offsets, int max_nodes, int max_walks, int32_t* counts,
                                cudaStream_t s);
cudaError_t launch_heuristics(const GraphBatch& b, int nframes, cudaStream_t s);
// heuristics with each tile's local component labels fused in, then the
// label stage's remainder (merge across the 64x16 tile borders, flatten)
cudaError_t launch_heuristics_labels(const GraphBatch& b, int nframes, int32_t* labels, cudaStream_t s);
cudaError_t launch_labels_after_heuristics(const uint8_t* g, int32_t* labels, int w, int h, int nframes,
                                          size_t frame_stride, cudaStream_t s);
cudaError_t launch_labels(const uint8_t* g, int32_t* labels, int w, int h, int nframes, size_t frame_stride,
                          cudaStream_t s);

// Device allocations of the library's own scratch go through these two: a
// count of live allocations, and fault injection for tests
// (depix_debug_fail_allocations): an injected failure returns
// cudaErrorMemoryAllocation without calling cudaMalloc.
cudaError_t dev_alloc(void** p, size_t bytes);
template <typename T>
inline cudaError_t dev_alloc(T** p, size_t bytes)
{
    return dev_alloc(reinterpret_cast<void**>(p), bytes);
}
void dev_free(void* p);
// Test switch (depix_debug_tma_timeout): the TMA graph kernel issues no tile
// load and gives up after a few polls, so its bounded wait's error path runs
// with nothing in flight.
cudaError_t set_graph_tma_timeout_test(int on);

cudaError_t launch_yuv_words(const uint8_t* px3, size_t n, int mode, uint32_t* out, cudaStream_t s);

// geometry stage
cudaError_t init_tables(cudaStream_t s);
cudaError_t copy_tables(uint64_t* hull, uint64_t* tri);
// device address of the per-pattern hull table (this device)
cudaError_t hull_table_address(const uint64_t** out);
cudaError_t launch_cells(const uint8_t* g, int w, int h, float* diagram, int* ec, cudaStream_t s);
cudaError_t launch_subdivide(const uint8_t* img, int w, int h, int ws, int layout, const uint8_t* g,
                             const float* snap, const int* ec_snap, float* diagram, int* ec, cudaStream_t s);
cudaError_t launch_triangulate(float* diagram, const int* ec, int w, int h, cudaStream_t s);
cudaError_t launch_emit(const uint8_t* img, int w, int h, int ws, int layout, const float* diagram, const int* ec,
                        float* pos, uint8_t* col, cudaStream_t s);
cudaError_t launch_raster(const RasterBatch& b, int nframes, cudaStream_t s);
// coverage-mask raster (scale <= kMaxMaskScale) and its per-scale pattern table
constexpr int kMaxMaskScale = 12;
size_t scale_mask_words(int scale);
// reads and clears the raster's and the graph stage's sticky fault flags (a
// TMA wait that gave up)
cudaError_t take_raster_fault(int* out);
cudaError_t take_graph_fault(int* out);
cudaError_t take_heuristics_fault(int* out);
bool u8_tensor_map(const uint8_t* base, int w, int h, size_t frame_stride, int nframes, int box_w, int box_h,
                   CUtensorMap* map);
// tensor map of RGBA frames as words, (w, h, frames), box (box_w, box_h, 1);
// false when the buffers do not meet TMA's alignment rules
bool rgba_tensor_map(const uint8_t* img, int w, int h, int ws, size_t frame_stride, int nframes, int box_w, int box_h,
                     CUtensorMap* map);
cudaError_t build_scale_masks(int scale, uint32_t* lut, cudaStream_t s);
cudaError_t launch_mask_raster(const RasterBatch& b, int nframes, const uint32_t* lut, cudaStream_t s);


}  // namespace depix
