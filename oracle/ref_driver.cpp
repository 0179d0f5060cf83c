// Host build of the reference's own per-pixel stage bodies.
//
// TEST INFRASTRUCTURE ONLY. This translation unit is compiled by
// oracle/build_ref.sh directly against the reference checkout (the stage
// files are #included from there, never copied into this repository) into
// oracle/_ref/libdepix_ref{5,48}.so. It is used to pin the C restatement in
// oracle/depix_oracle.c and to generate the committed golden fixtures; no
// product code links or loads it.
//
// The per-stage loops below replay the order of the reference frame driver
// (kernel.cu:402-475: graph -> trivial -> snapshot -> heuristics -> cells ->
// snapshot -> subdivision -> triangulation -> colour/position fill) with one
// host loop per kernel launch. Out-of-buffer reads made by the reference at
// image borders land in zero-filled guard bands, which is the parity contract
// for those reads.

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#define __device__
#define __global__
#define __align__(n) __attribute__((aligned(n)))

#include "point.cu"
#define CELL_SIZE 45
#include "graph_functions.cu"
#include "diagram_functions.cu"
#include "triangulate_functions.cu"
#include "subdivision_functions.cu"

namespace {

struct Guarded {
    std::vector<char> buf;
    size_t guard;
    char* base() { return buf.data() + guard; }
    Guarded(size_t n, size_t g) : buf(n + 2 * g, 0), guard(g) {}
};

}  // namespace

extern "C" {

// Runs the reference stages on one BGR frame (rows bottom-up, stride ws).
// graph_in: if non-NULL, the graph stages are skipped and this resolved graph
// is used instead (lets the known-answer graph dumps drive the cell stages).
// Every output pointer may be NULL. Array sizes: graphs W*H, edge counts W*H,
// diagrams W*H*45*2 floats, pos W*H*45*2 floats, col W*H*45*4 bytes.
int ref_frame(const uint8_t* bgr, int w, int h, int ws, int subdivide,
              const uint8_t* graph_in,
              uint8_t* graph_trivial_out, uint8_t* graph_resolved_out,
              int* ec_cells_out, float* diag_cells_out,
              int* ec_final_out, float* diag_final_out,
              float* pos_out, uint8_t* col_out)
{
    const int n = w * h;
    const size_t img_size = (size_t)ws * h;
    Guarded img((size_t)img_size, (size_t)ws + 64);
    if (bgr) memcpy(img.base(), bgr, img_size);
    Guarded graph((size_t)n, (size_t)w + 64);
    Guarded graph_aux((size_t)n, (size_t)w + 64);
    char* g = graph.base();
    char* ga = graph_aux.base();

    if (graph_in) {
        memcpy(g, graph_in, n);
        if (graph_trivial_out) memcpy(graph_trivial_out, graph_in, n);
    } else {
        // graph_Kernel body (kernel.cu:140-159)
        for (int j = 0; j < h; j++)
            for (int i = 0; i < w; i++)
                for (int e = 0; e < 8; e++) {
                    if (diff(i, j, e, w, h, ws, img.base())) {
                        SET_BIT(g[(j * w) + i], e, 0);
                    } else {
                        SET_BIT(g[(j * w) + i], e, 1);
                    }
                }
        // trivial_cross_Kernel body (kernel.cu:162-177)
        for (int j = 0; j < h; j++)
            for (int i = 0; i < w; i++) crossCheck_4(g, w, h, i, j);
        memcpy(ga, g, n);
        if (graph_trivial_out) memcpy(graph_trivial_out, g, n);
        // ambiguous_cross_Kernel body (kernel.cu:180-189)
        bool flag = false;
        for (int j = 0; j < h; j++)
            for (int i = 0; i < w; i++) crossCheck_Heuristics(g, ga, w, h, i, j, &flag);
    }
    if (graph_resolved_out) memcpy(graph_resolved_out, g, n);

    std::vector<Point> diagram((size_t)n * CELL_SIZE);
    std::vector<Point> diagram_aux((size_t)n * CELL_SIZE);
    memset(diagram.data(), 0, diagram.size() * sizeof(Point));
    std::vector<int> ec(n, 0), ec_aux(n, 0);
    std::vector<char> edge_status((size_t)n * CELL_SIZE, 0);
    std::vector<int> link_index((size_t)n * CELL_SIZE, 0);

    // cells_Kernel body (kernel.cu:192-213); graph[idx-1] / graph[idx+1]
    // read the zero guard at the two ends of the buffer.
    for (int j = 0; j < h; j++)
        for (int i = 0; i < w; i++) {
            int node_index = j * w + i;
            ec[node_index] = createCellFromPattern<Point>(
                g[node_index], g[node_index - 1], g[node_index + 1],
                diagram.data(), node_index * CELL_SIZE, i, j);
        }
    if (ec_cells_out) memcpy(ec_cells_out, ec.data(), n * sizeof(int));
    if (diag_cells_out) memcpy(diag_cells_out, diagram.data(), (size_t)n * CELL_SIZE * sizeof(Point));
    diagram_aux = diagram;
    ec_aux = ec;

    // subdivision_Kernel body (kernel.cu:216-261)
    if (subdivide) {
        for (int j = 0; j < h; j++)
            for (int i = 0; i < w; i++) {
                int node_index = j * w + i;
                int cell_index = node_index * CELL_SIZE;
                if (g[node_index] == 90) continue;
                int ne = subdivision(img.base(), &diagram[cell_index], diagram_aux.data(), ec_aux.data(),
                                     node_index, w, ws, h, i, j, g[node_index],
                                     (bool*)&edge_status[cell_index], &link_index[cell_index]);
                ec[node_index] = ne;
            }
    }
    if (ec_final_out) memcpy(ec_final_out, ec.data(), n * sizeof(int));
    if (diag_final_out) memcpy(diag_final_out, diagram.data(), (size_t)n * CELL_SIZE * sizeof(Point));

    // triangulate_Kernel body (kernel.cu:264-282)
    for (int j = 0; j < h; j++)
        for (int i = 0; i < w; i++) {
            int node_index = j * w + i;
            triangulate_polygon(&diagram[(size_t)node_index * CELL_SIZE], ec.data(), node_index, CELL_SIZE, i, j);
        }

    // position_kernel / color_kernel bodies (kernel.cu:67-137)
    for (int j = 0; j < h; j++)
        for (int i = 0; i < w; i++) {
            int node_index = j * w + i;
            size_t ci = (size_t)node_index * CELL_SIZE;
            for (int t = 0; t < CELL_SIZE; t++) {
                if (pos_out) {
                    if (t < ((ec[node_index] - 2) * 3)) {
                        pos_out[2 * (ci + t)] = diagram[ci + t].x;
                        pos_out[2 * (ci + t) + 1] = diagram[ci + t].y;
                    } else {
                        pos_out[2 * (ci + t)] = -100.0f;
                        pos_out[2 * (ci + t) + 1] = -100.0f;
                    }
                }
                if (col_out) {
                    const char* px = img.base() + PIXEL(i, j, ws, 3);
                    col_out[4 * (ci + t) + 0] = (uint8_t)px[2];
                    col_out[4 * (ci + t) + 1] = (uint8_t)px[1];
                    col_out[4 * (ci + t) + 2] = (uint8_t)px[0];
                    col_out[4 * (ci + t) + 3] = 255;
                }
            }
        }
    return 0;
}

// The reference's packed-YUV word for one BGR pixel (graph_functions.cu:80-131).
uint32_t ref_yuv_word(uint8_t b0, uint8_t b1, uint8_t b2)
{
    return RGBtoYUV((int)DATAtoINT((char)b0, (char)b1, (char)b2));
}

// Bulk form over n pixels of 3 bytes each.
void ref_yuv_words(const uint8_t* px, long n, uint32_t* out)
{
    for (long k = 0; k < n; k++) out[k] = ref_yuv_word(px[3 * k], px[3 * k + 1], px[3 * k + 2]);
}

}  // extern "C"
