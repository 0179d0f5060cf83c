// GPU build of the reference's own per-pixel stage bodies.
//
// TEST INFRASTRUCTURE ONLY. oracle/build_ref.sh compiles this translation
// unit with nvcc for sm_103a and the reference's own device flags
// (depixel_gpu.pro:48: -use_fast_math, -fno-strict-aliasing; nvcc's default
// FMA contraction) against the reference's stage files, which the script
// stages into the git-ignored oracle/_ref/src/ (never committed). The
// result, oracle/_ref/libdepix_refgpu{5,48}.so, is the parity target the
// product is checked against on the GPU: the reference's CUDA arithmetic,
// not its host build.
//
// The kernels below are this harness's own: each runs one reference stage
// body per pixel exactly as the reference kernel of the same name does
// (kernel.cu:67-282), on zero guard-banded buffers, in the order of the
// reference frame driver (kernel.cu:402-475). Two things differ from
// kernel.cu, neither of which changes a result:
//  - blocks are 16x16 threads instead of 2x2 (every stage body reads only
//    snapshots or bits no thread changes, so the block shape is invisible);
//  - subdivision_Kernel's __syncthreads after a divergent return
//    (kernel.cu:231-243) is left out: nothing after it reads shared state.
// The heuristic walk (calcVal2PathSize) recurses up to 31 levels, so the
// per-thread stack limit is raised before the first launch.

#include <cstdint>
#include <cstdio>
#include <cstring>

#include <cuda_runtime.h>

#include "point.cu"
#define CELL_SIZE 45
#include "graph_functions.cu"
#include "diagram_functions.cu"
#include "triangulate_functions.cu"
#include "subdivision_functions.cu"

namespace {

constexpr int kBlock = 16;

__global__ void h_yuv_words(uint32_t* out)
{
    unsigned c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (1u << 24)) return;
    // diff() packs the pixel's three bytes in memory order (graph_functions.cu:190)
    char b0 = (char)(c & 0xFF), b1 = (char)((c >> 8) & 0xFF), b2 = (char)((c >> 16) & 0xFF);
    out[c] = RGBtoYUV((int)DATAtoINT(b0, b1, b2));
}

// graph_Kernel body (kernel.cu:140-159)
__global__ void h_graph(char* img, int w, int h, int ws, char* graph)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i < w && j < h) {
        for (int e = 0; e < 8; e++) {
            if (diff(i, j, e, w, h, ws, img)) {
                SET_BIT(graph[(j * w) + i], e, 0);
            } else {
                SET_BIT(graph[(j * w) + i], e, 1);
            }
        }
    }
}

// trivial_cross_Kernel body (kernel.cu:162-177)
__global__ void h_trivial(int w, int h, char* graph)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i < w && j < h) crossCheck_4(graph, w, h, i, j);
}

// ambiguous_cross_Kernel body (kernel.cu:180-189)
__global__ void h_heuristics(int w, int h, char* graph, char* graph_aux, bool* flag)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i < w && j < h) crossCheck_Heuristics(graph, graph_aux, w, h, i, j, flag);
}

// cells_Kernel body (kernel.cu:192-213): linear idx-1 / idx+1 neighbours
__global__ void h_cells(int w, int h, char* graph, Point* diagram, int* ec)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i < w && j < h) {
        int node = j * w + i;
        ec[node] = createCellFromPattern<Point>(graph[node], graph[node - 1], graph[node + 1], diagram,
                                                node * CELL_SIZE, i, j);
    }
}

// subdivision_Kernel body (kernel.cu:216-261)
__global__ void h_subdivision(char* img, int w, int ws, int h, char* graph, Point* diagram, Point* diagram_aux,
                              int* ec, int* ec_old, bool* edge_status, int* link_index)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i < w && j < h) {
        int cell = (j * w + i) * CELL_SIZE;
        int node = j * w + i;
        if (graph[node] == 90) return;
        int n = subdivision(img, &diagram[cell], diagram_aux, ec_old, node, w, ws, h, i, j, graph[node],
                            &edge_status[cell], &link_index[cell]);
        ec[node] = n;
    }
}

// triangulate_Kernel body (kernel.cu:264-282)
__global__ void h_triangulate(int w, int h, Point* diagram, int* ec)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i < w && j < h) {
        int node = j * w + i;
        triangulate_polygon(&diagram[node * CELL_SIZE], ec, node, CELL_SIZE, i, j);
    }
}

// color_kernel + position_kernel bodies (kernel.cu:67-137)
__global__ void h_emit(float2* pos, uchar4* col, Point* diagram, int* ec, int w, int h, char* img, int ws)
{
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i < (unsigned)w && j < (unsigned)h) {
        int node = (j * w) + i;
        int cell = node * CELL_SIZE;
        for (int t = 0; t < CELL_SIZE; t++) {
            col[cell + t].x = (unsigned char)img[PIXEL(i, j, ws, 3) + 2];
            col[cell + t].y = (unsigned char)img[PIXEL(i, j, ws, 3) + 1];
            col[cell + t].z = (unsigned char)img[PIXEL(i, j, ws, 3) + 0];
            col[cell + t].w = (unsigned char)255;
            if (t < ((ec[node] - 2) * 3)) {
                pos[cell + t].x = diagram[cell + t].x;
                pos[cell + t].y = diagram[cell + t].y;
            } else {
                pos[cell + t].x = -100.0f;
                pos[cell + t].y = -100.0f;
            }
        }
    }
}

char g_err[256];

int fail(const char* what, cudaError_t e)
{
    snprintf(g_err, sizeof g_err, "%s: %s", what, cudaGetErrorString(e));
    return (int)e;
}

#define CK(call)                                   \
    do {                                           \
        cudaError_t e_ = (call);                   \
        if (e_ != cudaSuccess) return fail(#call, e_); \
    } while (0)

int raise_stack()
{
    static bool done = false;
    if (done) return 0;
    CK(cudaDeviceSetLimit(cudaLimitStackSize, 8192));
    done = true;
    return 0;
}

// Device allocations of one frame run, zero guard bands on both sides.
struct Bufs {
    char* img_base = nullptr;
    char* graph_base = nullptr;
    char* aux_base = nullptr;
    Point* diag_base = nullptr;
    Point* diag_aux_base = nullptr;
    int* ec = nullptr;
    int* ec_aux = nullptr;
    bool* flag = nullptr;
    bool* edge_status = nullptr;
    int* link_index = nullptr;
    float2* pos = nullptr;
    uchar4* col = nullptr;
    ~Bufs()
    {
        cudaFree(img_base); cudaFree(graph_base); cudaFree(aux_base); cudaFree(diag_base);
        cudaFree(diag_aux_base); cudaFree(ec); cudaFree(ec_aux); cudaFree(flag); cudaFree(edge_status);
        cudaFree(link_index); cudaFree(pos); cudaFree(col);
    }
};

}  // namespace

extern "C" {

const char* refgpu_last_error(void) { return g_err; }

// The packed YUV word of all 2^24 byte triples (index b0 | b1 << 8 | b2 << 16)
// as the reference's CUDA build computes it. h_out: 2^24 uint32.
int refgpu_yuv_words(uint32_t* h_out)
{
    uint32_t* d = nullptr;
    CK(cudaMalloc(&d, sizeof(uint32_t) << 24));
    h_yuv_words<<<(1 << 24) / 256, 256>>>(d);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(h_out, d, sizeof(uint32_t) << 24, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return fail("yuv words", e);
    return 0;
}

// The reference's stages on one BGR frame (rows bottom-up, stride ws) on the
// GPU, with the same outputs as ref_frame in ref_driver.cpp (any may be
// NULL): graph after trivial removal, resolved graph, cell counts and 45-slot
// cells, counts and cells after subdivision (the cells before subdivision
// when it is off), and the VBO (pos w*h*45*2 floats, col w*h*45*4 bytes).
// graph_in, when set, replaces the graph stages by a given resolved graph.
int refgpu_frame(const uint8_t* bgr, int w, int h, int ws, int subdivide, const uint8_t* graph_in,
                 uint8_t* graph_trivial_out, uint8_t* graph_resolved_out, int* ec_cells_out, float* diag_cells_out,
                 int* ec_final_out, float* diag_final_out, float* pos_out, uint8_t* col_out)
{
    if (w <= 0 || h <= 0 || ws < 3 * w) {
        snprintf(g_err, sizeof g_err, "bad frame size");
        return -1;
    }
    if (int r = raise_stack()) return r;
    const size_t n = (size_t)w * h;
    const size_t img_bytes = (size_t)ws * h, img_guard = (size_t)ws + 64;
    const size_t g_guard = (size_t)w + 64;
    const size_t cells = n * CELL_SIZE, c_guard = ((size_t)w + 2) * CELL_SIZE;
    Bufs b;
    CK(cudaMalloc(&b.img_base, img_bytes + 2 * img_guard));
    CK(cudaMalloc(&b.graph_base, n + 2 * g_guard));
    CK(cudaMalloc(&b.aux_base, n + 2 * g_guard));
    CK(cudaMalloc(&b.diag_base, (cells + 2 * c_guard) * sizeof(Point)));
    CK(cudaMalloc(&b.diag_aux_base, (cells + 2 * c_guard) * sizeof(Point)));
    CK(cudaMalloc(&b.ec, n * sizeof(int)));
    CK(cudaMalloc(&b.ec_aux, n * sizeof(int)));
    CK(cudaMalloc(&b.flag, n));
    CK(cudaMalloc(&b.edge_status, cells));
    CK(cudaMalloc(&b.link_index, cells * sizeof(int)));
    CK(cudaMalloc(&b.pos, cells * sizeof(float2)));
    CK(cudaMalloc(&b.col, cells * sizeof(uchar4)));
    CK(cudaMemset(b.img_base, 0, img_bytes + 2 * img_guard));
    CK(cudaMemset(b.graph_base, 0, n + 2 * g_guard));
    CK(cudaMemset(b.aux_base, 0, n + 2 * g_guard));
    CK(cudaMemset(b.diag_base, 0, (cells + 2 * c_guard) * sizeof(Point)));
    CK(cudaMemset(b.diag_aux_base, 0, (cells + 2 * c_guard) * sizeof(Point)));
    CK(cudaMemset(b.ec, 0, n * sizeof(int)));
    CK(cudaMemset(b.ec_aux, 0, n * sizeof(int)));
    CK(cudaMemset(b.flag, 0, n));
    CK(cudaMemset(b.edge_status, 0, cells));
    CK(cudaMemset(b.link_index, 0, cells * sizeof(int)));
    char* img = b.img_base + img_guard;
    char* g = b.graph_base + g_guard;
    char* ga = b.aux_base + g_guard;
    Point* diag = b.diag_base + c_guard;
    Point* diag_aux = b.diag_aux_base + c_guard;
    if (bgr) CK(cudaMemcpy(img, bgr, img_bytes, cudaMemcpyHostToDevice));

    dim3 blk(kBlock, kBlock), grd((w + kBlock - 1) / kBlock, (h + kBlock - 1) / kBlock);
    if (graph_in) {
        CK(cudaMemcpy(g, graph_in, n, cudaMemcpyHostToDevice));
        if (graph_trivial_out) memcpy(graph_trivial_out, graph_in, n);
    } else {
        h_graph<<<grd, blk>>>(img, w, h, ws, g);
        CK(cudaGetLastError());
        h_trivial<<<grd, blk>>>(w, h, g);
        CK(cudaGetLastError());
        CK(cudaMemcpy(ga, g, n, cudaMemcpyDeviceToDevice));
        if (graph_trivial_out) CK(cudaMemcpy(graph_trivial_out, ga, n, cudaMemcpyDeviceToHost));
        h_heuristics<<<grd, blk>>>(w, h, g, ga, b.flag);
        CK(cudaGetLastError());
    }
    if (graph_resolved_out) CK(cudaMemcpy(graph_resolved_out, g, n, cudaMemcpyDeviceToHost));
    h_cells<<<grd, blk>>>(w, h, g, diag, b.ec);
    CK(cudaGetLastError());
    CK(cudaMemcpy(diag_aux, diag, cells * sizeof(Point), cudaMemcpyDeviceToDevice));
    CK(cudaMemcpy(b.ec_aux, b.ec, n * sizeof(int), cudaMemcpyDeviceToDevice));
    if (ec_cells_out) CK(cudaMemcpy(ec_cells_out, b.ec, n * sizeof(int), cudaMemcpyDeviceToHost));
    if (diag_cells_out) CK(cudaMemcpy(diag_cells_out, diag, cells * sizeof(Point), cudaMemcpyDeviceToHost));
    if (subdivide) {
        h_subdivision<<<grd, blk>>>(img, w, ws, h, g, diag, diag_aux, b.ec, b.ec_aux, b.edge_status,
                                    b.link_index);
        CK(cudaGetLastError());
    }
    if (ec_final_out) CK(cudaMemcpy(ec_final_out, b.ec, n * sizeof(int), cudaMemcpyDeviceToHost));
    if (diag_final_out) CK(cudaMemcpy(diag_final_out, diag, cells * sizeof(Point), cudaMemcpyDeviceToHost));
    h_triangulate<<<grd, blk>>>(w, h, diag, b.ec);
    CK(cudaGetLastError());
    h_emit<<<grd, blk>>>(b.pos, b.col, diag, b.ec, w, h, img, ws);
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    if (pos_out) CK(cudaMemcpy(pos_out, b.pos, cells * sizeof(float2), cudaMemcpyDeviceToHost));
    if (col_out) CK(cudaMemcpy(col_out, b.col, cells * sizeof(uchar4), cudaMemcpyDeviceToHost));
    return 0;
}

}  // extern "C"
