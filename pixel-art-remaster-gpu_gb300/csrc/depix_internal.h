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

// One frame of a variable-size batch (device array entry).
struct BatchFrame {
    uint64_t in_off;  // image offset (bytes) in the batch input
    uint64_t out_off; // raster offset (bytes) in the batch output
    uint64_t px_off;  // offset (pixels) of the frame's graph in the scratch graphs
    int w, h;
    int tile_base_graph; // first graph-stage tile index of this frame
    int tile_base_heur;  // first heuristics-stage tile index
    int tile_base_rast;  // first raster-stage tile index
    int pad;
};

// text returned by depix_last_error() on this thread
void set_last_error(const std::string& msg);

// graph stage
cudaError_t launch_graph(const FrameBatch& b, int nframes, uint32_t thr, bool fuse_trivial, cudaStream_t s);
cudaError_t launch_trivial(uint8_t* g, int w, int h, cudaStream_t s);
cudaError_t launch_heuristics(const GraphBatch& b, int nframes, cudaStream_t s);
cudaError_t launch_labels(const uint8_t* g, int32_t* labels, int w, int h, int nframes, size_t frame_stride,
                          cudaStream_t s);

cudaError_t launch_yuv_words(const uint8_t* px3, size_t n, uint32_t* out, cudaStream_t s);

// geometry stage
cudaError_t init_tables(cudaStream_t s);
cudaError_t copy_tables(uint64_t* hull, uint64_t* tri);
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
cudaError_t build_scale_masks(int scale, uint32_t* lut, cudaStream_t s);
cudaError_t launch_mask_raster(const RasterBatch& b, int nframes, const uint32_t* lut, cudaStream_t s);


}  // namespace depix
