/*
 * depix.h -- C ABI of the GB300 depixelization library (libdepix.so).
 *
 * The library implements the reference's frame path (kernel.cu:286-526 of
 * marcoc2/pixel-art-remaster-gpu): similarity graph, crossing resolution,
 * reshaped cells, corner-cutting subdivision, ear-clip triangulation, the
 * "mapped buffer" VBO output, plus a headless rasterizer that replaces the
 * OpenGL draw and a connected-component labelling stage.
 *
 * Conventions (all entry points):
 *  - every function returns a depix_status; nothing calls exit();
 *  - pointers named d_* are device pointers, h_* host pointers; the caller
 *    owns all memory passed in;
 *  - work is enqueued on the given stream and the call returns without
 *    synchronising, except where a function says otherwise;
 *  - images are rows of pixels with row 0 at the bottom (the y-up order the
 *    reference works in after its loader flips rows, Image.cpp:21-38);
 *  - node byte bit e set means "similar to the neighbour in direction e":
 *        bit  0      1      2      3      4      5       6      7
 *        (di,dj) (-1,+1) (0,+1) (+1,+1) (-1,0) (+1,0) (-1,-1) (0,-1) (+1,-1)
 *    (graph_functions.cu:162-235 of the reference).
 */
#ifndef DEPIX_H
#define DEPIX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* depix_stream; /* a cudaStream_t; NULL = legacy default stream */

typedef enum depix_status {
    DEPIX_OK = 0,
    DEPIX_ERR_INVALID_ARG = 1, /* bad size, stride, scale or NULL pointer */
    DEPIX_ERR_CUDA = 2,        /* a CUDA runtime call or launch failed */
    DEPIX_ERR_ALLOC = 3,       /* device or host allocation failed */
    DEPIX_ERR_TOO_LARGE = 4,   /* request exceeds a context's or buffer's capacity */
    DEPIX_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up */
    DEPIX_ERR_CAPTURING = 6,   /* one-time set-up was needed while the stream was being captured */
    DEPIX_ERR_STATE = 7        /* a device-side consistency check failed */
} depix_status;

/* Pixel layout of an input image. */
typedef enum depix_layout {
    /* the reference's layout: 3 bytes per pixel, B,G,R order, rows
     * `widthstep` bytes apart (Image.cpp:42-48) */
    DEPIX_LAYOUT_BGR = 0,
    /* 4 bytes per pixel R,G,B,A (alpha ignored), rows `widthstep` bytes
     * apart; handled as the BGR image the reference would have loaded, with
     * a 4-byte-aligned row stride and zero row padding */
    DEPIX_LAYOUT_RGBA = 1
} depix_layout;

/* How the luma y of the packed Y/U/V word is evaluated. The reference
 * computes y = int(0.299 r + 0.587 g + 0.114 b) in double
 * (graph_functions.cu:90); its two builds round that sum differently for
 * 2490 of the 2^24 colours (42 of them grey levels), all with an exact
 * integer sum, where one build's y is one below the other's. */
typedef enum depix_yuv {
    /* the reference's CUDA build (depixel_gpu.pro, nvcc with its default FMA
     * contraction): fma(0.114, b, fma(0.299, r, 0.587 g)). The parity target
     * of the frame path and the default. */
    DEPIX_YUV_CUDA = 0,
    /* the reference's stage bodies built for the host CPU: IEEE double with no
     * contraction, (0.299 r + 0.587 g) + 0.114 b */
    DEPIX_YUV_HOST = 1
} depix_yuv;

typedef struct depix_params {
    /* similarity thresholds in units of the packed Y/U/V byte fields
     * (graph_functions.cu:11-19): defaults Y 48, U 7, V 6; the reference's
     * active build uses Y 5 */
    int tr_y, tr_u, tr_v;
    int subdivide; /* run the corner-cutting stage (simpleVBO.cpp:41 default off) */
    int scale;     /* raster scale factor, 1..64 */
    /* heuristic crossing resolution: 0 (default) the reference's ordered
     * tests (processHeuristics2, graph_functions.cu:761-849); 1 the weighted
     * vote of Kopf and Lischinski, "Depixelizing Pixel Art" (2011) sec. 3.2:
     * curves, sparse pixels (component sizes in the 8x8 window around the
     * block) and islands, the diagonal with fewer votes removed, both on a
     * tie. Not in the reference; no parity target beyond the oracle. */
    int vote;
    int yuv; /* depix_yuv: arithmetic of the luma (default DEPIX_YUV_CUDA) */
} depix_params;

void depix_default_params(depix_params* p);
const char* depix_status_string(depix_status s);
/* Last CUDA error text seen by this thread ("" if none). */
const char* depix_last_error(void);

/* One-time per-device set-up (builds the 4096-entry cell-pattern tables on
 * the current device). Every entry point does it on first use on a device;
 * call it once before capturing any stream into a CUDA graph. */
depix_status depix_init_device(void);
/* Sticky device-side faults of the current device since the last call,
 * then cleared: a bounded wait for a TMA tile load gave up and that tile
 * was left unwritten, bit 0 in the raster, bit 1 in the graph stage, bit 2
 * in the heuristics stage. Returns DEPIX_ERR_TIMEOUT when any bit is set
 * (the outputs of the launches since the last call are then incomplete),
 * DEPIX_OK otherwise. Synchronous. */
depix_status depix_take_device_faults(int* flags);

/* Testing hooks: fault injection for the error paths, not for production.
 *  - depix_debug_fail_allocations(after): after `after` more device
 *    allocations by the library succeed, every later one fails (without
 *    calling cudaMalloc) until called again with after < 0;
 *  - depix_debug_live_allocations: device allocations the library holds now
 *    (context scratch and staging, per-device tables, queue descriptors,
 *    refiner buffers);
 *  - depix_debug_tma_timeout(1): the TMA graph kernel issues no tile load
 *    and gives up its bounded wait after a few polls, with nothing in flight,
 *    so a frame's graph stage fails the way a lost load would: bit 1 of
 *    depix_take_device_faults and DEPIX_ERR_TIMEOUT. (0) restores it. */
depix_status depix_debug_fail_allocations(int after);
depix_status depix_debug_live_allocations(long long* count);
depix_status depix_debug_tma_timeout(int enable);

/* ---------------------------------------------------------------------
 * Stage entry points: each mirrors one reference kernel, on device memory.
 * --------------------------------------------------------------------- */

/* Similarity graph (graph_Kernel, kernel.cu:140-159). With fuse_trivial != 0
 * the trivial crossing removal (trivial_cross_Kernel, kernel.cu:162-177) is
 * applied in the same pass. d_graph: w*h bytes. */
depix_status depix_graph(const uint8_t* d_img, int w, int h, int widthstep, depix_layout layout,
                         const depix_params* p, int fuse_trivial, uint8_t* d_graph, depix_stream s);

/* Trivial crossing removal in place (trivial_cross_Kernel, kernel.cu:162-177). */
depix_status depix_resolve_trivial(uint8_t* d_graph, int w, int h, depix_stream s);

/* Heuristic crossing resolution (ambiguous_cross_Kernel, kernel.cu:180-189):
 * reads the snapshot d_snapshot (the graph after trivial removal), writes the
 * resolved graph to d_out. The two buffers must not overlap. */
depix_status depix_resolve_heuristics(const uint8_t* d_snapshot, int w, int h, uint8_t* d_out, depix_stream s);

/* The same with the weighted vote (depix_params.vote = 1) instead of the
 * reference's ordered tests. No counterpart in the reference. */
depix_status depix_resolve_heuristics_vote(const uint8_t* d_snapshot, int w, int h, uint8_t* d_out,
                                           depix_stream s);

/* Reshaped cells (cells_Kernel, kernel.cu:192-213) in the reference's
 * 45-slot layout: d_diagram gets w*h*45 (x,y) float pairs, local cell
 * coordinates, count+1 points per cell (the last repeats the first), the
 * other slots zero; d_edge_count gets the vertex count. */
depix_status depix_cells(const uint8_t* d_graph, int w, int h, float* d_diagram, int* d_edge_count, depix_stream s);

/* One corner-cutting round (subdivision_Kernel, kernel.cu:216-261): reads
 * the cell snapshot (d_diagram_snap / d_edge_count_snap, as written by
 * depix_cells), writes new polygons into d_diagram / d_edge_count; interior
 * nodes (byte 90) are left untouched, as in the reference. */
depix_status depix_subdivide(const uint8_t* d_img, int w, int h, int widthstep, depix_layout layout,
                             const uint8_t* d_graph, const float* d_diagram_snap, const int* d_edge_count_snap,
                             float* d_diagram, int* d_edge_count, depix_stream s);

/* Ear-clip triangulation in place (triangulate_Kernel, kernel.cu:264-282):
 * each cell's first 3*(count-2) slots become triangle corners plus the
 * cell's (i, j) offset; the remaining slots get (-100,-100). */
depix_status depix_triangulate(float* d_diagram, const int* d_edge_count, int w, int h, depix_stream s);

/* Mapped-buffer output (position_kernel + color_kernel, kernel.cu:67-137):
 * d_pos w*h*45 float pairs (unused slots (-100,-100)), d_col w*h*45 RGBA8
 * (the pixel's R,G,B and alpha 255). Either may be NULL. */
depix_status depix_emit_vbo(const uint8_t* d_img, int w, int h, int widthstep, depix_layout layout,
                            const float* d_diagram, const int* d_edge_count, float* d_pos, uint8_t* d_col,
                            depix_stream s);

/* Connected components of a resolved graph over its set bits: every node
 * gets the minimum linear index of its component. d_labels: w*h int32.
 * (New stage: the reference has only a sequential border walk,
 * cc_functions.cu:348-503, which depix_border_walks provides.) */
depix_status depix_label_components(const uint8_t* d_graph, int w, int h, int32_t* d_labels, depix_stream s);

/* Border walks of the components of nframes resolved graphs (frame f at
 * d_graph + f*w*h), the input of the reference's spline export
 * (extractBorderPoints, cc_functions.cu:348-503), as its recorded output
 * alex_png.txt lists them: nodes in scan order start walks unless internal
 * (byte 90) or already listed; a walk leaves by the node's first link in the
 * reference's clockwise link order and turns clockwise at every node until
 * it closes on its start; a walk that enters an internal, listed or
 * discarded node first is dropped (its last node discarded, its start left
 * unlisted). A node without links is a walk of its own.
 *  - d_scratch: w*h*nframes bytes of state, overwritten;
 *  - walk k of frame f: nodes (linear indices) d_nodes[f*max_nodes +
 *    d_offsets[f*(max_walks+1) + k] ...] up to offset k+1, and per node the
 *    link it leaves by in d_edges (int8, -1 for a node without links);
 *  - d_counts[3*f ..]: walks, nodes, and 1 when max_nodes or max_walks ran
 *    out (the outputs then hold the walks completed before).
 * The walks of a frame depend on each other in scan order: one warp per
 * frame walks them sequentially, so a batch of frames is the efficient
 * call. */
depix_status depix_border_walks(const uint8_t* d_graph, int w, int h, int nframes, uint8_t* d_scratch, int32_t* d_nodes,
                                int8_t* d_edges, int32_t* d_offsets, int max_nodes, int max_walks, int32_t* d_counts,
                                depix_stream s);

/* Headless raster of a resolved graph (replaces glDrawArrays over the VBO,
 * simpleVBO.cpp:236-285): rebuilds every cell's (optionally subdivided,
 * p->subdivide) triangles and writes a (w*scale) x (h*scale) RGBA8 image,
 * row 0 at the bottom, rows (w*scale*4) bytes apart. Coverage contract:
 * output pixel (X,Y) samples (X+0.5, Y+0.5); a triangle covers it when its
 * edge functions are > 0, or == 0 on a top or left edge; the latest triangle
 * in VBO order wins; uncovered samples are (0,0,0,255). */
depix_status depix_raster(const uint8_t* d_img, int w, int h, int widthstep, depix_layout layout,
                          const uint8_t* d_graph, const depix_params* p, uint8_t* d_out, depix_stream s);

/* Diagnostics. The packed Y/U/V word the graph stage compares (RGBtoYUV,
 * graph_functions.cu:80-131) for n pixels of 3 bytes in the reference's
 * memory order (d_px3: 3n bytes, d_words: n uint32), with the luma
 * arithmetic yuv (depix_yuv). */
depix_status depix_yuv_words(const uint8_t* d_px3, size_t n, int yuv, uint32_t* d_words, depix_stream s);

/* Copies the per-device cell-pattern tables to host arrays of 4096 entries
 * each: hull (count in bits 0-3, then 8 vertices of 6 bits: x+1 | (y+1)<<3
 * in quarter cells) and its ear clip (3 bits per corner index). Synchronous. */
depix_status depix_pattern_tables(uint64_t* h_hull, uint64_t* h_tri);

/* Heuristic crossing resolution IN PLACE, allocating nothing. No counterpart
 * in the reference: it is depix_resolve_heuristics with the snapshot the
 * heuristics read (the reference's graph_aux copy, kernel.cu:415) kept in a
 * fixed device array inside the library instead of a caller buffer, for
 * callers that cannot allocate device memory: real-time or embedded hosts
 * that forbid allocation after start-up, plugins running under a host
 * application that owns the device memory pool, code that must not call
 * cudaMalloc while other work is in flight.
 *  - d_graph (w*h bytes) holds the graph after trivial removal on entry and
 *    the resolved graph on return;
 *  - w*h must not exceed DEPIX_STATIC_MAX_PIXELS (4 MiB of snapshot, e.g.
 *    2048x2048); larger frames return DEPIX_ERR_TOO_LARGE;
 *  - every device that loads the library holds the 4 MiB array until the
 *    process exits;
 *  - the first call on a device looks up the array's device address (no
 *    allocation); make that first call before capturing any stream. The
 *    address is kept per device and looked up again when the calling
 *    thread's current context is not the one it was found in (after
 *    cudaDeviceReset);
 *  - all calls share the one array: calls whose work overlaps on the GPU
 *    (different streams, no ordering between them) race on it. */
#define DEPIX_STATIC_MAX_PIXELS 4194304
depix_status depix_resolve_heuristics_static(uint8_t* d_graph, int w, int h, depix_stream s);

/* ---------------------------------------------------------------------
 * Frame path with a context that owns its scratch (no allocation per call).
 * --------------------------------------------------------------------- */

typedef struct depix_context depix_context;

/* Scratch for frames of up to max_pixels pixels each and up to max_frames
 * frames per batch call. */
depix_status depix_context_create(depix_context** ctx, size_t max_pixels, int max_frames);
depix_status depix_context_destroy(depix_context* ctx);

/* Whole path on one device-resident frame: graph + trivial -> heuristics ->
 * [labels] -> raster. d_graph_out (w*h) and d_labels (w*h int32) may be NULL. */
depix_status depix_frame(depix_context* ctx, const uint8_t* d_img, int w, int h, int widthstep,
                         depix_layout layout, const depix_params* p, uint8_t* d_out, uint8_t* d_graph_out,
                         int32_t* d_labels, depix_stream s);

/* A batch of frames, each with its own size. Frame k reads its image at
 * d_img + in_offset[k] (RGBA8, rows w[k]*4 bytes apart) and writes its raster
 * at d_out + out_offset[k] (rows w[k]*scale*4 bytes apart); offsets are in
 * bytes and must be multiples of 16. With d_labels set, frame k's component
 * labels go to d_labels + (w[0]*h[0] + ... + w[k-1]*h[k-1]). Host arrays w,
 * h, in_offset, out_offset have n entries. Frames of one size at a constant
 * stride go through one launch per stage for the whole batch; other batches
 * (scale up to 12, stream not capturing) through persistent kernels that pull
 * tiles of all frames from one queue per stage, replayed as a CUDA graph. */
depix_status depix_batch(depix_context* ctx, int n, const int* w, const int* h, const uint64_t* in_offset,
                         const uint64_t* out_offset, const uint8_t* d_img, const depix_params* p, uint8_t* d_out,
                         int32_t* d_labels, depix_stream s);

/* depix_batch on HOST buffers: copies h_img (in_bytes) to the device, runs
 * the batch, copies the rasters back to h_out (out_bytes) and, when h_labels
 * is set, the labels. Device staging is owned by the context (allocated on
 * the first call that needs more). Synchronous. Pinned host memory gives the
 * full copy bandwidth. */
depix_status depix_batch_host(depix_context* ctx, int n, const int* w, const int* h, const uint64_t* in_offset,
                              const uint64_t* out_offset, const uint8_t* h_img, size_t in_bytes,
                              const depix_params* p, uint8_t* h_out, size_t out_bytes, int32_t* h_labels,
                              depix_stream s);

/* Launch shape of the queue path (uneven batches): tiles pulled per queue
 * step, 1, 2, 4 or 8 (0: tuned, the default), and the raster tile in cells,
 * 32x32, 32x16, 16x16, or 0x0: each frame in the shape with the fewest cells
 * to process (one raster launch per shape). Tuning runs on the first batch of each bucket of
 * frame count and mean frame size (powers of two), scale and label choice, by
 * timing the candidate shapes on that batch (it synchronises the stream). */
depix_status depix_context_set_launch_shape(depix_context* ctx, int gran, int tile_w, int tile_h);
/* The shape the last queue-path batch ran with: gran[4] per stage (graph,
 * heuristics, labels, raster) and the raster tile; any pointer may be NULL. */
depix_status depix_context_launch_shape(depix_context* ctx, int* gran, int* tile_w, int* tile_h);

/* Per-stage device timing of a context's frame and batch calls. */
enum {
    DEPIX_STAGE_GRAPH = 0,      /* similarity graph + trivial removal */
    DEPIX_STAGE_HEURISTICS = 1, /* heuristic crossing resolution */
    DEPIX_STAGE_LABELS = 2,     /* component labels: merge across tiles and flatten (with labels on, the
                                   heuristics stage also makes each tile's local labels) */
    DEPIX_STAGE_RASTER = 3,     /* cells, subdivision, coverage masks, block resolution, output */
    DEPIX_STAGE_COUNT = 4
};
/* Turns CUDA-event timing of every stage launch on or off (off by default). */
depix_status depix_context_set_timing(depix_context* ctx, int enable);
/* Accumulated device milliseconds, kernel launches and stage calls per stage
 * since the last reset (arrays of DEPIX_STAGE_COUNT; any may be NULL), then
 * resets. Waits for the recorded events. */
depix_status depix_context_stage_times(depix_context* ctx, double* ms, long long* launches, long long* calls);

/* ---------------------------------------------------------------------
 * Spline refinement (no reference counterpart: the reference's frame path
 * ends at the VBO fill). Node positions of the colour boundaries are
 * optimised on the GPU with Adam against curvature, deviation and a soft
 * coverage loss at the output scale; the topology is frozen at setup.
 * --------------------------------------------------------------------- */

typedef struct depix_refiner depix_refiner;
typedef struct depix_refine_params {
    float w_curvature; /* 1.0: mean squared second difference of the Chaikin points at free nodes */
    float w_deviation; /* 0.25: mean squared distance of free nodes from their start */
    float w_coverage;  /* 1.0: mean squared RGB error of the soft raster against the x scale target */
    float sigma;       /* 0.5: coverage Gaussian, output pixels (fixed at setup) */
    float lr;          /* 0.05: Adam step, source pixels */
    int steps;         /* 200 */
} depix_refine_params;

void depix_refine_default_params(depix_refine_params* p);
/* Scratch for frames of up to max_pixels pixels. */
depix_status depix_refiner_create(depix_refiner** r, size_t max_pixels);
depix_status depix_refiner_destroy(depix_refiner* r);
/* Extracts and freezes one frame's topology from its image and resolved
 * graph (p: thresholds of the curve test, output scale 1..12; d_graph NULL:
 * the refiner resolves the graph itself): nodes, curve edges, Chaikin
 * segments, the output samples near each segment and their targets, and a
 * signature per 16x16-pixel tile (graph bytes and colours of the tile and its
 * one-pixel ring). Reads two counts back once (edges and nodes, which size
 * the node and segment arrays), so the call waits for the stream's work up
 * to that point; the rest of the setup is queued on s without waiting (later
 * calls on s see the frame; work on another stream waits for an event
 * recorded on s). Nodes are vertices of the (4w+3) x (4h+3) quarter-pixel
 * grid, so position buffers of that many float2 always hold a frame. */
depix_status depix_refine_setup(depix_refiner* r, const uint8_t* d_img, int w, int h, int widthstep,
                                depix_layout layout, const uint8_t* d_graph, const depix_params* p,
                                const depix_refine_params* rp, depix_stream s);
/* nodes, free nodes, curve edges, segment slots, assigned samples (the
 * first call after a setup synchronises the device to read the counts the
 * setup left on it) */
depix_status depix_refine_counts(depix_refiner* r, long long counts[5]);
/* The frozen topology to host arrays (any may be NULL): node quarter-pixel
 * coordinates (2 per node), flags (bit 0 pinned, 1 frame, 2 corner, degree
 * << 4), neighbours of degree-2 nodes (2 per node, -1 otherwise), edges (u,
 * v, left cell, right cell), segment slots (3 nodes, type), slot colours
 * (left, right as 0xBBGGRR) and samples (output index, slot). Synchronous. */
depix_status depix_refine_export(depix_refiner* r, int32_t* node_q, int32_t* node_flags, int32_t* node_nbr,
                                 int32_t* edges, int32_t* segs, uint32_t* seg_colors, int32_t* samples);
/* Start positions (float x, y per node, source pixels) to d_pos. */
depix_status depix_refine_initial(depix_refiner* r, float* d_pos, depix_stream s);
/* Warm start from the previous frame of a stream (same size): nodes in tiles
 * whose signature is unchanged take prev's position (d_prev_pos, prev's node
 * order) of the node at the same quarter-pixel coordinates; every other node
 * its start position. Writes r's start positions to d_pos; reused_tiles (may
 * be NULL; reading it synchronises) gets the number of unchanged tiles. */
depix_status depix_refine_warm_start(depix_refiner* r, const depix_refiner* prev, const float* d_prev_pos,
                                     float* d_pos, int* reused_tiles, depix_stream s);
/* Energy terms (curvature, deviation, coverage, total) at d_pos and, when
 * d_grad is set, dE/d position per node (zero at pinned nodes): the adjoint.
 * Synchronous. */
depix_status depix_refine_energy_grad(depix_refiner* r, const depix_refine_params* p, const float* d_pos,
                                      float* d_grad, double energy[4], depix_stream s);
/* p->steps Adam steps (beta 0.9 / 0.999, eps 1e-8) from d_pos (NULL: the
 * start positions); the result goes back to d_pos when set. Energies before
 * and after when the pointers are set (those evaluations synchronise). */
depix_status depix_refine_run(depix_refiner* r, const depix_refine_params* p, float* d_pos, double before[4],
                              double after[4], depix_stream s);

/* ---------------------------------------------------------------------
 * Drop-in replacement of the reference's frame driver.
 * --------------------------------------------------------------------- */

typedef struct depix_point { float x, y; } depix_point; /* Point, point.cu:2-11 */

/* Same arguments and layout as launch_kernel (kernel.cu:286-288), plus the
 * thresholds: pos / colorPos are caller-owned DEVICE buffers of w*h*45
 * float2 / uchar4; img_data is a host BGR image (stride img_widthstep);
 * edge_count_h (w*h int) and graph_h (w*h bytes) are host outputs; time is
 * unused; p NULL means the reference build's thresholds (Y 5, U 7, V 6) and
 * luma arithmetic (DEPIX_YUV_CUDA); p->subdivide / p->scale are ignored. Returns a malloc'd host array of
 * w*h*45 points (the triangulated cells, unused slots (-100,-100)) that the
 * caller frees, or NULL on error (see depix_last_error). Synchronous; scratch
 * is kept per process between calls and guarded by a lock. */
depix_point* depix_launch_kernel_compat(void* pos, void* colorPos, float time, char* img_data, int img_width,
                                        int img_height, int img_widthstep, int* edge_count_h, char* graph_h,
                                        int subdivide, const depix_params* p);

#ifdef __cplusplus
#define DEPIX_BOOL bool
#else
#define DEPIX_BOOL _Bool
#endif
/* The reference's own symbol (kernel.cu:286), forwarding to the function
 * above with the reference build's thresholds. */
depix_point* launch_kernel(void* pos, void* colorPos, float time, char* img_data, int img_width, int img_height,
                           int img_widthstep, int* edge_count_h, char* graph_h, DEPIX_BOOL subdivide);

#ifdef __cplusplus
}
#endif

#endif /* DEPIX_H */
