// depix_refine.cu -- spline refinement: node positions of the colour
// boundaries optimised against curvature, deviation and a soft-coverage
// raster loss, with a hand-written adjoint.
//
// The reference has no such stage (its frame path ends at the VBO fill,
// kernel.cu:439-520). Its definition here:
//
// Topology, extracted once per frame and frozen:
//   * cells are the hulls of the resolved graph's cell patterns (the hull
//     table); split at every hull vertex lying inside an edge, the cells'
//     edges pair up exactly with reversed twins in 8-neighbour cells;
//   * a split edge whose twin belongs to a dissimilar cell is a curve edge,
//     kept once (from the lower-indexed cell, along its counter-clockwise
//     hull: its colour on the left);
//   * nodes are curve-edge vertices in global quarter-pixel units, numbered
//     in vertex-grid order; pinned when not of degree 2, on an edge without
//     a twin (the frame), or where the two edges turn by 90 degrees or more;
//   * one Chaikin round gives the segments: the middle of each edge (slot
//     3e+1), the piece from a pinned end to the first cut point (3e, 3e+2)
//     and the cut corner of each free node (3E + node);
//   * every output sample within 1.5 output pixels of a segment is assigned
//     to the nearest one (exact integer distances, one rounded division;
//     ties to the lower slot).
// Energy (every term a mean): w_curv * 1/F sum_free |a - 2p + b|^2 / 8
//   + w_dev * 1/F sum_free |p - p0|^2
//   + w_cov * 1/(3 Ws Hs) sum_samples sum_rgb ((r - t)/255)^2,
//   r = cR + (cL - cR) Phi(d / sigma), d the sample's signed distance from
//   its segment's line, t the nearest-neighbour target under the same
//   Gaussian coverage. The adjoint recomputes each segment's Chaikin points
//   from the nodes in the backward pass instead of storing them.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "depix_internal.h"

namespace depix {

namespace {

constexpr int kBand = 48;          // 1.5 output pixels in 1/(32 s) source pixel
constexpr int kMaxRefineScale = 12;
enum SegType { SEG_NONE = 0, SEG_MID = 1, SEG_PIN_U = 2, SEG_PIN_V = 3, SEG_CORNER = 4 };
// weights (x4) of a segment's ends over its three node slots, per type, as
// 4-bit fields (type * 12 + slot * 4): A {-, 3 1 0, 4 0 0, 1 3 0, 1 3 0},
// B {-, 1 3 0, 3 1 0, 0 4 0, 0 3 1}
constexpr unsigned long long kSegWA = 0x031031004013000ull;
constexpr unsigned long long kSegWB = 0x130040013031000ull;
__host__ __device__ constexpr int seg_wa(int type, int k) { return (int)((kSegWA >> (type * 12 + k * 4)) & 0xF); }
__host__ __device__ constexpr int seg_wb(int type, int k) { return (int)((kSegWB >> (type * 12 + k * 4)) & 0xF); }
static_assert(seg_wa(1, 0) == 3 && seg_wa(1, 1) == 1 && seg_wa(2, 0) == 4 && seg_wa(3, 1) == 3 && seg_wa(4, 1) == 3,
              "segment weights A");
static_assert(seg_wb(1, 1) == 3 && seg_wb(2, 0) == 3 && seg_wb(2, 1) == 1 && seg_wb(3, 1) == 4 && seg_wb(4, 2) == 1 &&
              seg_wb(4, 1) == 3 && seg_wb(4, 0) == 0, "segment weights B");

// vertex grid word: bit 0 a hull vertex, bit 1 on an edge without a twin,
// bits 8.. the number of curve edges
constexpr uint32_t kVUsed = 1, kVFrame = 2;
constexpr int kNoSeg = 0x7F7F7F7F; // a byte fill of 0x7F: no segment
constexpr int kDegShift = 8;

struct Geo {
    const uint8_t* img;
    int ws, layout;
    const uint8_t* g;
    int w, h;
    int gw, gh;         // vertex grid: (4w + 3) x (4h + 3), origin at quarter (-1, -1)
    const uint64_t* lut;
    const uint32_t* box; // per-pattern hull boxes (k_rf_boxes)
    uint32_t thr;
};

__device__ __forceinline__ uint64_t cell_hull(const Geo& G, int idx)
{
    const int n = G.w * G.h;
    const unsigned node = G.g[idx];
    const unsigned left = idx > 0 ? G.g[idx - 1] : 0u;
    const unsigned right = idx + 1 < n ? G.g[idx + 1] : 0u;
    return __ldg(&G.lut[cell_pattern(node, left, right)]);
}

// hull vertex t in global quarter units
__device__ __forceinline__ int qvx(uint64_t e, int t, int i) { return 4 * i + (int)((e >> (4 + 6 * t)) & 7u) - 1; }
__device__ __forceinline__ int qvy(uint64_t e, int t, int j) { return 4 * j + (int)((e >> (7 + 6 * t)) & 7u) - 1; }
__device__ __forceinline__ int vindex(const Geo& G, int x, int y) { return (y + 1) * G.gw + (x + 1); }

__device__ __forceinline__ int igcd(int a, int b)
{
    a = abs(a);
    b = abs(b);
    while (b) {
        int t = a % b;
        a = b;
        b = t;
    }
    return a;
}

// v -> u lies on p -> q in the same direction
__device__ __forceinline__ bool reversed_on(int px, int py, int qx, int qy, int ux, int uy, int vx, int vy)
{
    const int ex = qx - px, ey = qy - py;
    if (ex * (vy - py) - ey * (vx - px) != 0 || ex * (uy - py) - ey * (ux - px) != 0) return false;
    if (ex * (ux - vx) + ey * (uy - vy) <= 0) return false;
    const int L = ex * ex + ey * ey;
    const int tv = ex * (vx - px) + ey * (vy - py), tu = ex * (ux - px) + ey * (uy - py);
    return tv >= 0 && tu <= L;
}

__device__ __forceinline__ uint32_t cell_word(const Geo& G, int i, int j)
{
    return word_of_bgr(load_bgr(G.img, G.ws, G.layout, i, j), G.thr);
}

// Walks the split edges of cell idx; for each, the twin's owner: the first
// 8-neighbour (in bit order) with a hull edge that holds the reversed split
// edge. A neighbour is only searched when its hull's bounding box (the
// per-pattern box table) holds the split edge. fn(ux, uy, vx, vy, owner, B).
template <typename Fn>
__device__ void walk_split_edges(const Geo& G, const uint32_t* vgrid, int idx, Fn fn)
{
    const int i = idx % G.w, j = idx / G.w;
    const uint64_t e = cell_hull(G, idx);
    const int k = (int)(e & 0xF);
    int npat[8];
    uint32_t nbox[8]; // x0, x1, y0, y1 in global quarter units, 8 bits each after a +8 bias
#pragma unroll
    for (int d = 0; d < 8; d++) {
        const int ni = i + dir_di(d), nj = j + dir_dj(d);
        npat[d] = -1;
        nbox[d] = 0;
        if (ni >= 0 && ni < G.w && nj >= 0 && nj < G.h) {
            const int nidx = nj * G.w + ni;
            const int n = G.w * G.h;
            npat[d] = cell_pattern(G.g[nidx], nidx > 0 ? G.g[nidx - 1] : 0u, nidx + 1 < n ? G.g[nidx + 1] : 0u);
            nbox[d] = __ldg(&G.box[npat[d]]);
        }
    }
    for (int t = 0; t < k; t++) {
        const int t1 = t + 1 == k ? 0 : t + 1;
        const int ax = qvx(e, t, i), ay = qvy(e, t, j), bx = qvx(e, t1, i), by = qvy(e, t1, j);
        const int gcd = igcd(bx - ax, by - ay);
        const int sx = (bx - ax) / gcd, sy = (by - ay) / gcd;
        int px = ax, py = ay;
        for (int st = 1; st <= gcd; st++) {
            const int cx = ax + st * sx, cy = ay + st * sy;
            if (st < gcd && !(vgrid[vindex(G, cx, cy)] & kVUsed)) continue;
            int owner = -1;
            // the split edge relative to the cell's own quarter origin
            const int lx0 = min(px, cx) - 4 * i, lx1 = max(px, cx) - 4 * i;
            const int ly0 = min(py, cy) - 4 * j, ly1 = max(py, cy) - 4 * j;
            for (int d = 0; d < 8 && owner < 0; d++) {
                if (npat[d] < 0) continue;
                const uint32_t bb = nbox[d];
                const int ox = 4 * dir_di(d), oy = 4 * dir_dj(d);
                if (lx0 < (int)(bb & 0xFF) - 8 + ox || lx1 > (int)((bb >> 8) & 0xFF) - 8 + ox ||
                    ly0 < (int)((bb >> 16) & 0xFF) - 8 + oy || ly1 > (int)(bb >> 24) - 8 + oy)
                    continue;
                const int ni = i + dir_di(d), nj = j + dir_dj(d);
                const uint64_t ne = __ldg(&G.lut[npat[d]]);
                const int nk = (int)(ne & 0xF);
                for (int s = 0; s < nk; s++) {
                    const int s1 = s + 1 == nk ? 0 : s + 1;
                    if (reversed_on(qvx(ne, s, ni), qvy(ne, s, nj), qvx(ne, s1, ni), qvy(ne, s1, nj), px, py, cx, cy)) {
                        owner = d;
                        break;
                    }
                }
            }
            const int B = owner < 0 ? -1 : (j + dir_dj(owner)) * G.w + (i + dir_di(owner));
            fn(px, py, cx, cy, owner, B);
            px = cx;
            py = cy;
        }
    }
}

// per pattern: the hull's bounding box in local quarter units, each bound + 8
__global__ void k_rf_boxes(const uint64_t* lut, uint32_t* box)
{
    const int pat = blockIdx.x * blockDim.x + threadIdx.x;
    if (pat >= 4096) return;
    const uint64_t e = lut[pat];
    const int k = (int)(e & 0xF);
    int x0 = 99, x1 = -99, y0 = 99, y1 = -99;
    for (int t = 0; t < k; t++) {
        const int x = qvx(e, t, 0), y = qvy(e, t, 0);
        x0 = min(x0, x);
        x1 = max(x1, x);
        y0 = min(y0, y);
        y1 = max(y1, y);
    }
    box[pat] = k ? (uint32_t)(x0 + 8) | (uint32_t)(x1 + 8) << 8 | (uint32_t)(y0 + 8) << 16 | (uint32_t)(y1 + 8) << 24
                 : 0xFFu; // empty: x0 beyond every edge
}

__global__ void k_rf_mark_vertices(Geo G, uint32_t* vgrid)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= G.w * G.h) return;
    const int i = idx % G.w, j = idx / G.w;
    const uint64_t e = cell_hull(G, idx);
    const int k = (int)(e & 0xF);
    for (int t = 0; t < k; t++) atomicOr(&vgrid[vindex(G, qvx(e, t, i), qvy(e, t, j))], kVUsed);
}

// pass 0: curve edges per cell, and the frame marks
__global__ void k_rf_count_edges(Geo G, uint32_t* vgrid, int* count)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= G.w * G.h) return;
    const int i = idx % G.w, j = idx / G.w;
    const uint32_t me = cell_word(G, i, j);
    int c = 0;
    walk_split_edges(G, vgrid, idx, [&](int ux, int uy, int vx, int vy, int owner, int B) {
        if (owner < 0) {
            atomicOr(&vgrid[vindex(G, ux, uy)], kVFrame);
            atomicOr(&vgrid[vindex(G, vx, vy)], kVFrame);
        } else if (B > idx && !similar(me, cell_word(G, B % G.w, B / G.w), G.thr)) {
            c++;
        }
    });
    count[idx] = c;
}

// pass 1: the curve edges at their offsets; degrees and up to two
// neighbours (vertex, edge) per vertex
__global__ void k_rf_emit_edges(Geo G, uint32_t* vgrid, const int* off, int4* edges, int2* nb_v, int2* nb_e)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= G.w * G.h) return;
    const int i = idx % G.w, j = idx / G.w;
    const uint32_t me = cell_word(G, i, j);
    int o = off[idx];
    walk_split_edges(G, vgrid, idx, [&](int ux, int uy, int vx, int vy, int owner, int B) {
        if (owner < 0 || B <= idx || similar(me, cell_word(G, B % G.w, B / G.w), G.thr)) return;
        const int u = vindex(G, ux, uy), v = vindex(G, vx, vy);
        edges[o] = make_int4(u, v, idx, B);
        const uint32_t su = atomicAdd(&vgrid[u], 1u << kDegShift) >> kDegShift;
        const uint32_t sv = atomicAdd(&vgrid[v], 1u << kDegShift) >> kDegShift;
        if (su < 2) {
            (&nb_v[u].x)[su] = v;
            (&nb_e[u].x)[su] = o;
        }
        if (sv < 2) {
            (&nb_v[v].x)[sv] = u;
            (&nb_e[v].x)[sv] = o;
        }
        o++;
    });
}

__global__ void k_rf_node_flags(const uint32_t* vgrid, int nv, int* is_node)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < nv) is_node[v] = (vgrid[v] >> kDegShift) > 0;
}

struct NodeOut {
    int2* q;        // quarter coordinates
    int* flags;     // bit 0 pinned, 1 frame, 2 corner; degree << 4
    int2* nbr;      // neighbours of degree-2 nodes (ascending), else -1
    int2* nbr_edge; // the edges to them
    float2* pos0;
};

__global__ void k_rf_nodes(Geo G, const uint32_t* vgrid, const int* nid, const int2* nb_v, const int2* nb_e, NodeOut N)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= G.gw * G.gh) return;
    const uint32_t word = vgrid[v];
    const int deg = (int)(word >> kDegShift);
    if (deg == 0) return;
    const int k = nid[v];
    const int x = v % G.gw - 1, y = v / G.gw - 1;
    int f = min(deg, 15) << 4;
    if (word & kVFrame) f |= 2;
    int2 nb = make_int2(-1, -1), ne = make_int2(-1, -1);
    if (deg == 2) {
        int a = nid[nb_v[v].x], b = nid[nb_v[v].y];
        int ea = nb_e[v].x, eb = nb_e[v].y;
        const int va = nb_v[v].x, vb = nb_v[v].y;
        int vax = va % G.gw - 1, vay = va / G.gw - 1, vbx = vb % G.gw - 1, vby = vb / G.gw - 1;
        if (a > b) {
            int t = a; a = b; b = t;
            t = ea; ea = eb; eb = t;
            t = vax; vax = vbx; vbx = t;
            t = vay; vay = vby; vby = t;
        }
        nb = make_int2(a, b);
        ne = make_int2(ea, eb);
        if ((x - vax) * (vbx - x) + (y - vay) * (vby - y) <= 0) f |= 4;
    }
    if (deg != 2 || (f & 6)) f |= 1;
    N.q[k] = make_int2(x, y);
    N.flags[k] = f;
    N.nbr[k] = nb;
    N.nbr_edge[k] = ne;
    N.pos0[k] = make_float2(0.25f * x, 0.25f * y);
}

struct SegOut {
    int4* seg;    // n0, n1, n2, type
    uint2* col;   // left, right RGB (0xBBGGRR)
};

__device__ __forceinline__ uint32_t cell_rgb(const Geo& G, int idx)
{
    const uint32_t c = load_bgr(G.img, G.ws, G.layout, idx % G.w, idx / G.w); // b0 | b1 << 8 | b2 << 16
    // reference bytes (b0, b1, b2) = (B, G, R) -> R | G << 8 | B << 16
    return ((c >> 16) & 0xFFu) | (c & 0xFF00u) | ((c & 0xFFu) << 16);
}

// segment slots: 3 per edge, then one per node
__global__ void k_rf_segments(Geo G, const int* nid, int4* edges, int E, int Nn, const int* flags, const int2* nbr,
                              const int2* nbr_edge, SegOut S)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < E) {
        int4 ed = edges[t];
        const int u = nid[ed.x], v = nid[ed.y];
        const uint2 col = make_uint2(cell_rgb(G, ed.z), cell_rgb(G, ed.w));
        const bool pu = flags[u] & 1, pv = flags[v] & 1;
        S.seg[3 * t] = pu ? make_int4(u, v, -1, SEG_PIN_U) : make_int4(-1, -1, -1, SEG_NONE);
        S.seg[3 * t + 1] = make_int4(u, v, -1, SEG_MID);
        S.seg[3 * t + 2] = pv ? make_int4(u, v, -1, SEG_PIN_V) : make_int4(-1, -1, -1, SEG_NONE);
        S.col[3 * t] = S.col[3 * t + 1] = S.col[3 * t + 2] = col;
    } else if (t < E + Nn) {
        const int p = t - E;
        const int s = 3 * E + p;
        if (flags[p] & 1) {
            S.seg[s] = make_int4(-1, -1, -1, SEG_NONE);
            S.col[s] = make_uint2(0, 0);
            return;
        }
        const int a = nbr[p].x, b = nbr[p].y;
        const int e = nbr_edge[p].x; // the edge between a and p
        const int4 ed = edges[e];
        const uint32_t l = cell_rgb(G, ed.z), r = cell_rgb(G, ed.w);
        const bool flip = nid[ed.x] != a; // stored as p -> a
        S.seg[s] = make_int4(a, p, b, SEG_CORNER);
        S.col[s] = flip ? make_uint2(r, l) : make_uint2(l, r);
    }
}

// exact segment ends at the start, in 1/(32 s) source pixel
__device__ __forceinline__ void seg_ends(const int4 sg, const int2* q, int scale, long long& ax, long long& ay,
                                         long long& bx, long long& by)
{
    ax = ay = bx = by = 0;
    const int nodes[3] = {sg.x, sg.y, sg.z};
#pragma unroll
    for (int k = 0; k < 3; k++) {
        if (nodes[k] < 0) continue;
        const int2 p = q[nodes[k]];
        ax += (long long)seg_wa(sg.w, k) * p.x;
        ay += (long long)seg_wa(sg.w, k) * p.y;
        bx += (long long)seg_wb(sg.w, k) * p.x;
        by += (long long)seg_wb(sg.w, k) * p.y;
    }
    const long long m = 2 * scale; // weights x4, quarter -> 1/(32 s): x 8 s / 4
    ax *= m;
    ay *= m;
    bx *= m;
    by *= m;
}

// squared distance, or -1 beyond the band (decided in integers first, so the
// rounded division only runs for samples inside it)
__device__ __forceinline__ double seg_dist2(long long ax, long long ay, long long bx, long long by, long long X,
                                            long long Y)
{
    const long long band2 = (long long)kBand * kBand;
    const long long ex = bx - ax, ey = by - ay, wx = X - ax, wy = Y - ay;
    const long long L = ex * ex + ey * ey, dot = ex * wx + ey * wy;
    if (dot <= 0) {
        const long long d = wx * wx + wy * wy;
        return d <= band2 ? (double)d : -1.0;
    }
    if (dot >= L) {
        const long long d = (X - bx) * (X - bx) + (Y - by) * (Y - by);
        return d <= band2 ? (double)d : -1.0;
    }
    const long long cr = ex * wy - ey * wx;
    if (cr * cr > band2 * L) return -1.0;
    return __ddiv_rn((double)(cr * cr), (double)L);
}

__device__ __forceinline__ long long floor_div_ll(long long a, long long b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }

// samples of a segment's box (+ band): fn(sample index, d2)
template <typename Fn>
__device__ void seg_samples(const int4 sg, const int2* q, int scale, int ow, int oh, Fn fn)
{
    long long ax, ay, bx, by;
    seg_ends(sg, q, scale, ax, ay, bx, by);
    // sample Xo sits at 16 (2 Xo + 1)
    const long long x0 = max(0LL, -floor_div_ll(-(min(ax, bx) - kBand - 16), 32));
    const long long x1 = min((long long)ow - 1, floor_div_ll(max(ax, bx) + kBand - 16, 32));
    const long long y0 = max(0LL, -floor_div_ll(-(min(ay, by) - kBand - 16), 32));
    const long long y1 = min((long long)oh - 1, floor_div_ll(max(ay, by) + kBand - 16, 32));
    for (long long yo = y0; yo <= y1; yo++)
        for (long long xo = x0; xo <= x1; xo++) {
            const double d2 = seg_dist2(ax, ay, bx, by, 16 * (2 * xo + 1), 16 * (2 * yo + 1));
            if (d2 >= 0.0) fn((int)(yo * ow + xo), d2);
        }
}

__global__ void k_rf_assign_dist(const int4* seg, int S, const int2* q, int scale, int ow, int oh,
                                 unsigned long long* best)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    const int4 sg = seg[s];
    if (sg.w == SEG_NONE) return;
    seg_samples(sg, q, scale, ow, oh, [&](int x, double d2) {
        atomicMin(&best[x], (unsigned long long)__double_as_longlong(d2));
    });
}

__global__ void k_rf_assign_seg(const int4* seg, int S, const int2* q, int scale, int ow, int oh,
                                const unsigned long long* best, int* bseg)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    const int4 sg = seg[s];
    if (sg.w == SEG_NONE) return;
    seg_samples(sg, q, scale, ow, oh, [&](int x, double d2) {
        if ((unsigned long long)__double_as_longlong(d2) == best[x]) atomicMin(&bseg[x], s);
    });
}

__global__ void k_rf_count_samples(const int* bseg, int n, int* seg_count)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x < n && bseg[x] != kNoSeg) atomicAdd(&seg_count[bseg[x]], 1);
}

__global__ void k_rf_scatter_samples(const int* bseg, int n, const int* seg_off, int* cursor, int* samp)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n || bseg[x] == kNoSeg) return;
    const int s = bseg[x];
    samp[seg_off[s] + atomicAdd(&cursor[s], 1)] = x;
}

// each segment's samples in ascending order (summation order fixed)
__global__ void k_rf_sort_samples(const int* seg_off, int S, int* samp)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    const int a = seg_off[s], b = seg_off[s + 1];
    for (int i = a + 1; i < b; i++) {
        const int v = samp[i];
        int j = i - 1;
        while (j >= a && samp[j] > v) {
            samp[j + 1] = samp[j];
            j--;
        }
        samp[j + 1] = v;
    }
}

// the nearest-neighbour target under the coverage Gaussian, per sample
// (separable: three column and three row weights)
__global__ void k_rf_targets(Geo G, int scale, float sig, const int* samp, const int* pM, float4* tgt)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= *pM) return;
    const int ow = G.w * scale;
    const int yo = samp[m] / ow, xo = samp[m] - yo * ow;
    const float x = ((float)xo + 0.5f) / (float)scale, y = ((float)yo + 0.5f) / (float)scale;
    const int ix = xo / scale, iy = yo / scale;
    const float inv = 1.f / sig;
    float cx[3], cy[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const int ii = ix + d - 1, jj = iy + d - 1;
        cx[d] = (ii >= 0 && ii < G.w) ? normcdff((x - (float)ii) * inv) - normcdff((x - (float)ii - 1.f) * inv) : 0.f;
        cy[d] = (jj >= 0 && jj < G.h) ? normcdff((y - (float)jj) * inv) - normcdff((y - (float)jj - 1.f) * inv) : 0.f;
    }
    float r = 0.f, g = 0.f, b = 0.f;
#pragma unroll
    for (int dj = 0; dj < 3; dj++) {
        const int jj = iy + dj - 1;
        if (jj < 0 || jj >= G.h) continue;
#pragma unroll
        for (int di = 0; di < 3; di++) {
            const int ii = ix + di - 1;
            if (ii < 0 || ii >= G.w) continue;
            const float wgt = cx[di] * cy[dj];
            const uint32_t c = cell_rgb(G, jj * G.w + ii);
            r += wgt * (float)(c & 0xFF);
            g += wgt * (float)((c >> 8) & 0xFF);
            b += wgt * (float)((c >> 16) & 0xFF);
        }
    }
    tgt[m] = make_float4(r, g, b, 0.f);
}

// ------------------------------------------------------------ warm start

constexpr int kWarmTile = 16; // source pixels per tile side

// Tile signature: FNV-1a (64-bit) over the resolved graph byte and the RGB of
// every pixel of the tile and its one-pixel ring (row-major, pixels outside
// the frame skipped): everything the tile's cells, curve edges and targets
// depend on.
__global__ void k_rf_tile_hash(Geo G, int tiles_x, int tiles, uint64_t* hash)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= tiles) return;
    const int x0 = (t % tiles_x) * kWarmTile - 1, y0 = (t / tiles_x) * kWarmTile - 1;
    uint64_t hsh = 0xcbf29ce484222325ull;
    auto mix = [&](uint32_t byte) {
        hsh ^= byte;
        hsh *= 0x100000001b3ull;
    };
    for (int y = max(y0, 0); y < min(y0 + kWarmTile + 2, G.h); y++)
        for (int x = max(x0, 0); x < min(x0 + kWarmTile + 2, G.w); x++) {
            const int idx = y * G.w + x;
            const uint32_t c = cell_rgb(G, idx);
            mix(G.g[idx]);
            mix(c & 0xFF);
            mix((c >> 8) & 0xFF);
            mix((c >> 16) & 0xFF);
        }
    hash[t] = hsh;
}

__global__ void k_rf_warm_scatter(const int2* q, const float2* pos, int N, int gw, float2* grid, int* stamp, int epoch)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    const int v = (q[k].y + 1) * gw + (q[k].x + 1);
    grid[v] = pos[k];
    stamp[v] = epoch;
}

__global__ void k_rf_warm_gather(const int2* q, const float2* pos0, int N, int w, int h, int gw, int tiles_x,
                                 const uint64_t* hash, const uint64_t* prev_hash, const float2* grid,
                                 const int* stamp, int epoch, float2* out)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    const int2 c = q[k];
    const int px = min(max(c.x >> 2, 0), w - 1), py = min(max(c.y >> 2, 0), h - 1);
    const int t = (py / kWarmTile) * tiles_x + px / kWarmTile;
    const int v = (c.y + 1) * gw + (c.x + 1);
    out[k] = (hash[t] == prev_hash[t] && stamp[v] == epoch) ? grid[v] : pos0[k];
}

__global__ void k_rf_same_tiles(const uint64_t* a, const uint64_t* b, int tiles, int* count)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const bool same = t < tiles && a[t] == b[t];
    const unsigned m = __ballot_sync(0xFFFFFFFFu, same);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(count, __popc(m));
}

// ---------------------------------------------------------------- scans

constexpr int kScanBlock = 1024, kScanItems = 4, kScanTile = kScanBlock * kScanItems;

__device__ __forceinline__ int block_exclusive_scan(int v, int* warp_sums)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int s = lane < (blockDim.x >> 5) ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xFFFFFFFFu, s, o);
            if (lane >= o) s += y;
        }
        warp_sums[lane] = s; // inclusive
    }
    __syncthreads();
    const int base = warp > 0 ? warp_sums[warp - 1] : 0;
    return base + x - v;
}

__global__ void __launch_bounds__(kScanBlock) k_scan_tiles(const int* in, int* out, int n, int* tile_sums)
{
    __shared__ int ws[32];
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int v[kScanItems], s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        v[k] = base + k < n ? in[base + k] : 0;
        s += v[k];
    }
    int ex = block_exclusive_scan(s, ws);
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        if (base + k < n) out[base + k] = ex;
        ex += v[k];
    }
    if (threadIdx.x == blockDim.x - 1) tile_sums[blockIdx.x] = ex;
}

__global__ void __launch_bounds__(kScanBlock) k_scan_sums(int* tile_sums, int tiles, int* total)
{
    __shared__ int ws[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int b = 0; b < tiles; b += kScanBlock) {
        const int k = b + threadIdx.x;
        const int v = k < tiles ? tile_sums[k] : 0;
        const int ex = block_exclusive_scan(v, ws);
        const int c = carry;
        if (k < tiles) tile_sums[k] = c + ex;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = c + ex + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void k_scan_add(int* out, int n, const int* tile_sums)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] += tile_sums[k / kScanTile];
}

// exclusive scan of n ints; the sum lands in *total (device)
cudaError_t exclusive_scan(const int* in, int* out, int n, int* tile_sums, int* total, cudaStream_t s)
{
    const int tiles = (n + kScanTile - 1) / kScanTile;
    if (tiles > 0) k_scan_tiles<<<tiles, kScanBlock, 0, s>>>(in, out, n, tile_sums);
    k_scan_sums<<<1, kScanBlock, 0, s>>>(tile_sums, tiles, total);
    if (n > 0) k_scan_add<<<(n + 255) / 256, 256, 0, s>>>(out, n, tile_sums);
    return cudaGetLastError();
}

// ------------------------------------------------------- energy and adjoint

// Frame sizes the step kernels read from device memory, so that a captured
// graph of the Adam loop serves every frame of the same buffers.
struct RefineFrame {
    int N;      // nodes
    int L;      // live segments (with samples)
    int ow, oh; // output raster
    int scale;
    int F;      // free nodes
    float inv_samples3; // 1 / (3 ow oh), rounded once on the host
};

// A live segment, packed for one load: its nodes and type, its sample
// range and its colours.
struct LiveSeg {
    int4 nodes;  // n0, n1, n2, type
    int4 range;  // first sample, end, left colour, right colour (0xBBGGRR)
};

// A free node and the nodes its curvature gradient reads: its neighbours
// a, b and, where a neighbour is free, that neighbour's neighbours (-1 when
// pinned), packed for one load.
struct FreeNode {
    int4 k_a_b_aa; // node, a, b, a's first neighbour
    int4 ab_ba_bb; // a's second neighbour, b's neighbours, unused
};

struct StepArgs {
    const float2* x;     // positions read
    float2* y;           // positions written (Adam)
    float2* gcov;        // coverage gradient (atomics), zeroed by the node pass
    float2* gout;        // gradient out (energy/gradient call), or NULL
    const float2* x0;
    const int4* seg;
    const uint2* col;
    const int* seg_off;
    const int* samp;
    const float4* tgt;
    const int* flags;
    const int2* nbr;
    const LiveSeg* live;
    const float2* sxy;   // sample positions (source pixels), in segment order
    const FreeNode* fnodes;
    const RefineFrame* fr;
    float2* m;
    float2* v;
    double* energy;      // [3] when not NULL
    float sigma;         // output pixels
    float w_curv, w_dev, w_cov;
    float lr, bc1, bc2;  // Adam step and bias corrections 1 - beta^t
    int update;
};

constexpr float kBeta1 = 0.9f, kBeta2 = 0.999f, kEps = 1e-8f;
constexpr float kInvSqrt2Pi = 0.3989422804014327f;
constexpr int kSegLanes = 4; // lanes per segment in the coverage pass

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}

__device__ __forceinline__ float group_sum(float v, unsigned mask)
{
#pragma unroll
    for (int o = kSegLanes / 2; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o);
    return v;
}

// Four lanes per live segment: Chaikin ends recomputed from the nodes, each
// assigned sample's soft colour, loss and d loss / d ends, reduced in the
// group and pushed to the segment's free nodes.
__global__ void __launch_bounds__(256) k_rf_coverage(StepArgs a)
{
    const RefineFrame F = *a.fr;
    const float inv_sig = (float)F.scale / a.sigma;
    const float cov_norm = a.w_cov * F.inv_samples3;
    const int lane = threadIdx.x & 31, gl = lane & (kSegLanes - 1);
    const unsigned gmask = ((1u << kSegLanes) - 1u) << (lane & ~(kSegLanes - 1));
    const int groups = (gridDim.x * blockDim.x) / kSegLanes;
    float eloss = 0.f;
    for (int l = (blockIdx.x * blockDim.x + threadIdx.x) / kSegLanes; l < F.L; l += groups) {
        const LiveSeg ls = a.live[l];
        const int4 sg = ls.nodes;
        const int b0 = ls.range.x, b1 = ls.range.y;
        const int nodes[3] = {sg.x, sg.y, sg.z};
        float2 A = make_float2(0.f, 0.f), B = make_float2(0.f, 0.f);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            if (nodes[k] < 0) continue;
            const float2 p = a.x[nodes[k]];
            const float wa = 0.25f * seg_wa(sg.w, k), wb = 0.25f * seg_wb(sg.w, k);
            A.x += wa * p.x;
            A.y += wa * p.y;
            B.x += wb * p.x;
            B.y += wb * p.y;
        }
        const uint32_t cl = (uint32_t)ls.range.z, crr = (uint32_t)ls.range.w;
        const float dl[3] = {(float)(int)(cl & 0xFF) - (float)(int)(crr & 0xFF),
                             (float)(int)((cl >> 8) & 0xFF) - (float)(int)((crr >> 8) & 0xFF),
                             (float)(int)((cl >> 16) & 0xFF) - (float)(int)((crr >> 16) & 0xFF)};
        const float cr[3] = {(float)(crr & 0xFF), (float)((crr >> 8) & 0xFF), (float)((crr >> 16) & 0xFF)};
        const float ex = B.x - A.x, ey = B.y - A.y;
        const float invL = rsqrtf(ex * ex + ey * ey);
        float gax = 0.f, gay = 0.f, gbx = 0.f, gby = 0.f;
        for (int m = b0 + gl; m < b1; m += kSegLanes) {
            const float2 X = a.sxy[m];
            const float wx = X.x - A.x, wy = X.y - A.y;
            const float d = (ex * wy - ey * wx) * invL;
            const float z = d * inv_sig;
            const float Phi = normcdff(z);
            const float4 t = a.tgt[m];
            const float r0 = (cr[0] + dl[0] * Phi - t.x) * (1.f / 255.f);
            const float r1 = (cr[1] + dl[1] * Phi - t.y) * (1.f / 255.f);
            const float r2 = (cr[2] + dl[2] * Phi - t.z) * (1.f / 255.f);
            eloss += r0 * r0 + r1 * r1 + r2 * r2;
            const float phi = expf(-0.5f * z * z) * kInvSqrt2Pi * inv_sig;
            const float dEdd = 2.f * cov_norm * (1.f / 255.f) * (r0 * dl[0] + r1 * dl[1] + r2 * dl[2]) * phi;
            // d d / d e = (wy, -wx) / L - d e / L^2 ; d d / d w = (-ey, ex) / L
            const float dex = wy * invL - d * ex * invL * invL, dey = -wx * invL - d * ey * invL * invL;
            const float dwx = -ey * invL, dwy = ex * invL;
            gbx += dEdd * dex;
            gby += dEdd * dey;
            gax += dEdd * (-dex - dwx);
            gay += dEdd * (-dey - dwy);
        }
        gax = group_sum(gax, gmask);
        gay = group_sum(gay, gmask);
        gbx = group_sum(gbx, gmask);
        gby = group_sum(gby, gmask);
        const int my = gl == 0 ? sg.x : (gl == 1 ? sg.y : (gl == 2 ? sg.z : -1));
        if (my >= 0 && !(a.flags[my] & 1)) {
            const float wa = 0.25f * seg_wa(sg.w, gl), wb = 0.25f * seg_wb(sg.w, gl);
            atomicAdd(&a.gcov[my].x, wa * gax + wb * gbx);
            atomicAdd(&a.gcov[my].y, wa * gay + wb * gby);
        }
    }
    if (a.energy) {
        eloss = warp_sum(eloss);
        if (lane == 0 && eloss != 0.f) atomicAdd(&a.energy[2], (double)eloss * (double)cov_norm);
    }
}

// One thread per node: curvature and deviation gradients (gathered from the
// node's own and its free neighbours' second differences), the coverage
// gradient, then an Adam step (or the gradient written out).
__global__ void __launch_bounds__(256) k_rf_nodes_step(StepArgs a)
{
    const RefineFrame F = *a.fr;
    const float curv_k = a.w_curv / (float)max(F.F, 1), dev_k = a.w_dev / (float)max(F.F, 1);
    float ec = 0.f, ed = 0.f;
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < F.F; f += gridDim.x * blockDim.x) {
        const FreeNode fn = a.fnodes[f];
        const int k = fn.k_a_b_aa.x;
        const float2 p = a.x[k], pa = a.x[fn.k_a_b_aa.y], pb = a.x[fn.k_a_b_aa.z];
        const int q_nb[4] = {fn.k_a_b_aa.w, fn.ab_ba_bb.x, fn.ab_ba_bb.y, fn.ab_ba_bb.z};
        float2 qn[4];
#pragma unroll
        for (int t = 0; t < 4; t++) qn[t] = q_nb[t] >= 0 ? a.x[q_nb[t]] : make_float2(0.f, 0.f);
        const float tx = pa.x - 2.f * p.x + pb.x, ty = pa.y - 2.f * p.y + pb.y;
        float gx = -2.f * tx, gy = -2.f * ty;
        if (q_nb[0] >= 0) { // a is free: its second difference reads p
            gx += qn[0].x - 2.f * pa.x + qn[1].x;
            gy += qn[0].y - 2.f * pa.y + qn[1].y;
        }
        if (q_nb[2] >= 0) {
            gx += qn[2].x - 2.f * pb.x + qn[3].x;
            gy += qn[2].y - 2.f * pb.y + qn[3].y;
        }
        const float2 p0 = a.x0[k];
        const float dx = p.x - p0.x, dy = p.y - p0.y;
        const float2 gc = a.gcov[k];
        gx = 0.25f * curv_k * gx + 2.f * dev_k * dx + gc.x;
        gy = 0.25f * curv_k * gy + 2.f * dev_k * dy + gc.y;
        a.gcov[k] = make_float2(0.f, 0.f);
        if (a.energy) {
            ec += 0.125f * (tx * tx + ty * ty);
            ed += dx * dx + dy * dy;
        }
        if (a.gout) a.gout[k] = make_float2(gx, gy);
        if (a.update) {
            float2 m = a.m[f], v = a.v[f];
            m.x = kBeta1 * m.x + (1.f - kBeta1) * gx;
            m.y = kBeta1 * m.y + (1.f - kBeta1) * gy;
            v.x = kBeta2 * v.x + (1.f - kBeta2) * gx * gx;
            v.y = kBeta2 * v.y + (1.f - kBeta2) * gy * gy;
            a.m[f] = m;
            a.v[f] = v;
            a.y[k] = make_float2(p.x - a.lr * (m.x / a.bc1) / (sqrtf(v.x / a.bc2) + kEps),
                                 p.y - a.lr * (m.y / a.bc1) / (sqrtf(v.y / a.bc2) + kEps));
        }
    }
    if (a.energy) {
        ec = warp_sum(ec);
        ed = warp_sum(ed);
        if ((threadIdx.x & 31) == 0) {
            if (ec != 0.f) atomicAdd(&a.energy[0], (double)ec * (double)curv_k);
            if (ed != 0.f) atomicAdd(&a.energy[1], (double)ed * (double)dev_k);
        }
    }
}

// live segments: a slot with a type and at least one sample
__global__ void k_rf_live_flags(const int4* seg, const int* seg_off, int S, int* flag)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < S) flag[s] = seg[s].w != SEG_NONE && seg_off[s + 1] > seg_off[s];
}

__global__ void k_rf_live_scatter(const int* flag, const int* pos, int S, const int4* seg, const int* seg_off,
                                  const uint2* col, LiveSeg* live)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < S && flag[s])
        live[pos[s]] = LiveSeg{seg[s], make_int4(seg_off[s], seg_off[s + 1], (int)col[s].x, (int)col[s].y)};
}

__global__ void k_rf_sample_xy(const int* samp, const int* pM, int ow, int scale, float2* sxy)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= *pM) return;
    const int yo = samp[m] / ow, xo = samp[m] - yo * ow;
    sxy[m] = make_float2(((float)xo + 0.5f) / (float)scale, ((float)yo + 0.5f) / (float)scale);
}

// start of an Adam run: both position buffers from src, moments zeroed
__global__ void k_rf_begin(const float2* src, float2* x, float2* y, float2* m, float2* v, int N)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const float2 q = src[i];
        x[i] = q;
        y[i] = q; // pinned nodes never move: both buffers start equal
        m[i] = make_float2(0.f, 0.f);
        v[i] = make_float2(0.f, 0.f);
    }
}

// the step kernels' frame record, from the scan totals on the device (F in
// slot 3, L in slot 4)
__global__ void k_rf_frame(const int* totals, int N, int ow, int oh, int scale, float inv_samples3, RefineFrame* fr)
{
    *fr = RefineFrame{N, totals[4], ow, oh, scale, totals[3], inv_samples3};
}

__global__ void k_rf_free_flags(const int* flags, int N, int* is_free)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < N) is_free[k] = !(flags[k] & 1);
}

__global__ void k_rf_free_nodes(const int* flags, const int2* nbr, const int* is_free, const int* pos, int N,
                                FreeNode* out)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N || !is_free[k]) return;
    const int2 nb = nbr[k];
    const int2 na = (flags[nb.x] & 1) ? make_int2(-1, -1) : nbr[nb.x];
    const int2 nbb = (flags[nb.y] & 1) ? make_int2(-1, -1) : nbr[nb.y];
    out[pos[k]] = FreeNode{make_int4(k, nb.x, nb.y, na.x), make_int4(na.y, nbb.x, nbb.y, 0)};
}

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t cap = 0;
    // grows with a quarter of headroom, so that frames of about the same
    // size reuse the buffer (a free in between would synchronize the device)
    cudaError_t reserve(size_t n)
    {
        if (n <= cap && p) return cudaSuccess;
        dev_free(p);
        p = nullptr;
        cap = 0;
        const size_t want = std::max<size_t>(n + n / 4, 1);
        cudaError_t e = dev_alloc(&p, want * sizeof(T));
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release()
    {
        dev_free(p);
        p = nullptr;
        cap = 0;
    }
};

}  // namespace

}  // namespace depix

using namespace depix;

struct depix_refiner {
    int device = 0;
    size_t max_pixels = 0;
    int sms = 0;
    const uint64_t* lut = nullptr;
    // frame
    int w = 0, h = 0, scale = 0, ow = 0, oh = 0;
    int E = 0, N = 0, F = 0, S = 0, M = 0; // F, M and L: -1 until read back (fetch_counts)
    int max_split = 0; // split curve edges a cell can own at most (its hull box's lattice steps)
    float sigma = 0.5f; // coverage sigma of the targets (output pixels)
    DevBuf<uint32_t> vgrid;
    DevBuf<uint32_t> box;
    DevBuf<uint8_t> own_graph, own_snap; // resolved graph when the caller gives none
    DevBuf<uint64_t> tile_hash;
    DevBuf<float2> warm_grid;
    DevBuf<int> warm_stamp;
    int tiles_x = 0, tiles = 0, warm_epoch = 0;
    DevBuf<int> cell_count, cell_off, is_node, nid, tile_sums, scalars;
    DevBuf<int2> nb_v, nb_e;
    DevBuf<int4> edges;
    DevBuf<int2> node_q, node_nbr, node_nbr_edge;
    DevBuf<int> node_flags;
    DevBuf<float2> pos0, pos_a, pos_b, gcov, adam_m, adam_v;
    DevBuf<int4> seg;
    DevBuf<uint2> seg_col;
    DevBuf<unsigned long long> best;
    DevBuf<int> bseg, seg_count, seg_off, cursor, samp;
    DevBuf<float4> tgt;
    DevBuf<double> energy;
    DevBuf<LiveSeg> live;
    DevBuf<int> live_flag, live_pos, free_flag, free_pos;
    DevBuf<FreeNode> fnodes;
    DevBuf<float2> sxy;
    DevBuf<RefineFrame> frame;
    int L = 0;
    int* h_scalars = nullptr; // pinned
    double* h_energy = nullptr;
    bool ready = false;
    // the Adam loop as a graph, replayed while its parameters and buffers stay
    cudaStream_t capture_stream = nullptr;
    cudaGraphExec_t loop = nullptr;
    StepArgs loop_args{};
    int loop_steps = -1;
    int loop_cov_blocks = 0, loop_node_blocks = 0;
};

namespace {

depix_status rf_fail(cudaError_t e, const char* where)
{
    set_last_error(std::string(where) + ": " + cudaGetErrorString(e));
    return DEPIX_ERR_CUDA;
}

#define DEPIX_TRY_RF(call)                                              \
    do {                                                                \
        depix_status st_ = (call);                                      \
        if (st_ != DEPIX_OK) return st_;                                \
    } while (0)

#define RF_CK(call)                                                     \
    do {                                                                \
        cudaError_t e_ = (call);                                        \
        if (e_ != cudaSuccess) return rf_fail(e_, #call);               \
    } while (0)

int blocks_for(long long n, int t = 256) { return (int)std::max<long long>(1, (n + t - 1) / t); }

// scan totals in slots [slot, slot + n), read back to the host (synchronous)
depix_status read_totals(depix_refiner* r, int slot, int n, int* out, cudaStream_t s)
{
    RF_CK(cudaMemcpyAsync(r->h_scalars + slot, r->scalars.p + slot, n * sizeof(int), cudaMemcpyDeviceToHost, s));
    RF_CK(cudaStreamSynchronize(s));
    for (int k = 0; k < n; k++) out[k] = r->h_scalars[slot + k];
    return DEPIX_OK;
}

// M, F and L of the set-up frame (scan totals left on the device by the
// setup), read back when a caller asks for them
depix_status fetch_counts(depix_refiner* r)
{
    if (r->M >= 0) return DEPIX_OK;
    RF_CK(cudaDeviceSynchronize());
    RF_CK(cudaMemcpy(r->h_scalars + 2, r->scalars.p + 2, 3 * sizeof(int), cudaMemcpyDeviceToHost));
    r->M = r->h_scalars[2];
    r->F = r->h_scalars[3];
    r->L = r->h_scalars[4];
    return DEPIX_OK;
}

depix_status check_refiner(depix_refiner* r)
{
    if (!r) {
        set_last_error("NULL refiner");
        return DEPIX_ERR_INVALID_ARG;
    }
    if (!r->ready) {
        set_last_error("refiner has no frame: call depix_refine_setup first");
        return DEPIX_ERR_INVALID_ARG;
    }
    return DEPIX_OK;
}

StepArgs step_args(depix_refiner* r, const depix_refine_params* p)
{
    StepArgs a{};
    a.gcov = r->gcov.p;
    a.x0 = r->pos0.p;
    a.seg = r->seg.p;
    a.col = r->seg_col.p;
    a.seg_off = r->seg_off.p;
    a.samp = r->samp.p;
    a.tgt = r->tgt.p;
    a.flags = r->node_flags.p;
    a.nbr = r->node_nbr.p;
    a.live = r->live.p;
    a.sxy = r->sxy.p;
    a.fnodes = r->fnodes.p;
    a.fr = r->frame.p;
    a.m = r->adam_m.p;
    a.v = r->adam_v.p;
    a.sigma = r->sigma;
    a.w_curv = p->w_curvature;
    a.w_dev = p->w_deviation;
    a.w_cov = p->w_coverage;
    a.lr = p->lr;
    return a;
}

depix_status check_rparams(const depix_refine_params* p)
{
    if (!p || !(p->sigma > 0.f) || !(p->lr >= 0.f) || p->steps < 0 || !(p->w_curvature >= 0.f) ||
        !(p->w_deviation >= 0.f) || !(p->w_coverage >= 0.f)) {
        set_last_error("refine params: sigma > 0, lr, weights >= 0, steps >= 0");
        return DEPIX_ERR_INVALID_ARG;
    }
    return DEPIX_OK;
}

depix_status check_sigma(const depix_refiner* r, const depix_refine_params* p)
{
    if (p->sigma != r->sigma) {
        set_last_error("coverage sigma differs from the one the targets were set up with");
        return DEPIX_ERR_INVALID_ARG;
    }
    return DEPIX_OK;
}

// grids: enough blocks for the frame rounded up to a power of two (the
// kernels stride over the sizes they read on the device, so a captured loop
// serves every frame whose rounded grids match), at most 8 blocks per SM
int pow2_at_least(long long n)
{
    int p = 1;
    while (p < n) p <<= 1;
    return p;
}
int cov_blocks(const depix_refiner* r)
{
    return std::min(r->sms * 8, pow2_at_least(((long long)r->S * kSegLanes + 255) / 256)); // L <= S
}
int node_blocks(const depix_refiner* r) { return std::min(r->sms * 8, pow2_at_least(((long long)r->N + 255) / 256)); } // F <= N

bool same_loop(const StepArgs& a, const StepArgs& b)
{
    return a.gcov == b.gcov && a.x0 == b.x0 && a.seg == b.seg && a.col == b.col && a.seg_off == b.seg_off &&
           a.samp == b.samp && a.tgt == b.tgt && a.flags == b.flags && a.nbr == b.nbr && a.live == b.live && a.sxy == b.sxy && a.fnodes == b.fnodes &&
           a.fr == b.fr && a.m == b.m && a.v == b.v && a.sigma == b.sigma && a.w_curv == b.w_curv &&
           a.w_dev == b.w_dev && a.w_cov == b.w_cov && a.lr == b.lr;
}

// launches the Adam steps from pos_a (result in pos_a after an even number
// of steps, pos_b after an odd one)
cudaError_t launch_steps(depix_refiner* r, const StepArgs& base, int steps, cudaStream_t s)
{
    StepArgs a = base;
    a.update = 1;
    float2* x = r->pos_a.p;
    float2* y = r->pos_b.p;
    double b1 = 1.0, b2 = 1.0;
    for (int t = 1; t <= steps; t++) {
        b1 *= (double)kBeta1;
        b2 *= (double)kBeta2;
        a.x = x;
        a.y = y;
        a.bc1 = (float)(1.0 - b1);
        a.bc2 = (float)(1.0 - b2);
        k_rf_coverage<<<cov_blocks(r), 256, 0, s>>>(a);
        k_rf_nodes_step<<<node_blocks(r), 256, 0, s>>>(a);
        std::swap(x, y);
    }
    return cudaGetLastError();
}

// energy (and gradient when gout) at positions x, without an update
depix_status eval(depix_refiner* r, const depix_refine_params* p, const float2* x, float2* gout, double out[4],
                  cudaStream_t s)
{
    StepArgs a = step_args(r, p);
    a.x = x;
    a.gout = gout;
    a.energy = r->energy.p;
    a.update = 0;
    RF_CK(cudaMemsetAsync(r->energy.p, 0, 3 * sizeof(double), s));
    if (gout) RF_CK(cudaMemsetAsync(gout, 0, (size_t)r->N * sizeof(float2), s)); // pinned nodes stay zero
    k_rf_coverage<<<cov_blocks(r), 256, 0, s>>>(a);
    k_rf_nodes_step<<<node_blocks(r), 256, 0, s>>>(a);
    RF_CK(cudaGetLastError());
    RF_CK(cudaMemcpyAsync(r->h_energy, r->energy.p, 3 * sizeof(double), cudaMemcpyDeviceToHost, s));
    RF_CK(cudaStreamSynchronize(s));
    out[0] = r->h_energy[0];
    out[1] = r->h_energy[1];
    out[2] = r->h_energy[2];
    out[3] = out[0] + out[1] + out[2];
    return DEPIX_OK;
}

}  // namespace

extern "C" {

void depix_refine_default_params(depix_refine_params* p)
{
    if (!p) return;
    p->w_curvature = 1.0f;
    p->w_deviation = 0.25f;
    p->w_coverage = 1.0f;
    p->sigma = 0.5f;
    p->lr = 0.05f;
    p->steps = 200;
}

depix_status depix_refiner_create(depix_refiner** out, size_t max_pixels)
{
    if (!out) {
        set_last_error("NULL refiner pointer");
        return DEPIX_ERR_INVALID_ARG;
    }
    *out = nullptr;
    if (max_pixels < 1) {
        set_last_error("capacity must be >= 1");
        return DEPIX_ERR_INVALID_ARG;
    }
    depix_status st = depix_init_device();
    if (st != DEPIX_OK) return st;
    depix_refiner* r = new (std::nothrow) depix_refiner();
    if (!r) return DEPIX_ERR_ALLOC;
    r->max_pixels = max_pixels;
    cudaError_t e = cudaGetDevice(&r->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&r->sms, cudaDevAttrMultiProcessorCount, r->device);
    if (e == cudaSuccess) e = hull_table_address(&r->lut);
    if (e == cudaSuccess) e = r->box.reserve(4096);
    if (e == cudaSuccess) {
        k_rf_boxes<<<16, 256>>>(r->lut, r->box.p);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
    }
    if (e == cudaSuccess) {
        // A cell's split curve edges lie on its convex hull, at most one per
        // quarter-unit lattice step: at most 2 (width + height) of the hull's
        // box, over all patterns.
        std::vector<uint32_t> box(4096);
        e = cudaMemcpy(box.data(), r->box.p, 4096 * sizeof(uint32_t), cudaMemcpyDeviceToHost);
        for (uint32_t b : box) {
            if (b == 0xFFu) continue;
            const int x0 = (int)(b & 0xFF), x1 = (int)((b >> 8) & 0xFF), y0 = (int)((b >> 16) & 0xFF), y1 = (int)(b >> 24);
            r->max_split = std::max(r->max_split, 2 * ((x1 - x0) + (y1 - y0)));
        }
        r->max_split = std::max(r->max_split, 1);
    }
    if (e == cudaSuccess) e = r->scalars.reserve(8);
    if (e == cudaSuccess) e = r->energy.reserve(3);
    if (e == cudaSuccess) e = cudaHostAlloc(&r->h_scalars, 8 * sizeof(int), cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaHostAlloc(&r->h_energy, 4 * sizeof(double), cudaHostAllocDefault);
    if (e == cudaSuccess) e = r->frame.reserve(1);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&r->capture_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        cudaGetLastError();
        depix_refiner_destroy(r);
        set_last_error(std::string("refiner set-up: ") + cudaGetErrorString(e));
        return DEPIX_ERR_ALLOC;
    }
    *out = r;
    return DEPIX_OK;
}

depix_status depix_refiner_destroy(depix_refiner* r)
{
    if (!r) return DEPIX_OK;
    r->vgrid.release();
    r->box.release();
    r->own_graph.release(); r->own_snap.release(); r->tile_hash.release(); r->warm_grid.release();
    r->warm_stamp.release();
    r->cell_count.release(); r->cell_off.release(); r->is_node.release(); r->nid.release();
    r->tile_sums.release(); r->scalars.release();
    r->nb_v.release(); r->nb_e.release(); r->edges.release();
    r->node_q.release(); r->node_nbr.release(); r->node_nbr_edge.release(); r->node_flags.release();
    r->pos0.release(); r->pos_a.release(); r->pos_b.release(); r->gcov.release();
    r->adam_m.release(); r->adam_v.release();
    r->seg.release(); r->seg_col.release(); r->best.release(); r->bseg.release();
    r->seg_count.release(); r->seg_off.release(); r->cursor.release(); r->samp.release(); r->tgt.release();
    r->energy.release();
    r->live.release(); r->live_flag.release(); r->live_pos.release(); r->frame.release();
    r->free_flag.release(); r->free_pos.release(); r->fnodes.release(); r->sxy.release();
    if (r->loop) cudaGraphExecDestroy(r->loop);
    if (r->capture_stream) cudaStreamDestroy(r->capture_stream);
    cudaFreeHost(r->h_scalars);
    cudaFreeHost(r->h_energy);
    delete r;
    return DEPIX_OK;
}

depix_status depix_refine_setup(depix_refiner* r, const uint8_t* d_img, int w, int h, int widthstep,
                                depix_layout layout, const uint8_t* d_graph, const depix_params* p,
                                const depix_refine_params* rp, depix_stream s_)
{
    DEPIX_TRY_RF(check_rparams(rp));
    if (!r || !d_img || !p || w < 1 || h < 1) {
        set_last_error("refine setup: NULL argument or size below 1");
        return DEPIX_ERR_INVALID_ARG;
    }
    if ((size_t)w * h > r->max_pixels) {
        set_last_error("frame larger than the refiner capacity");
        return DEPIX_ERR_TOO_LARGE;
    }
    if (p->scale < 1 || p->scale > kMaxRefineScale) {
        set_last_error("refine scale must be in 1..12");
        return DEPIX_ERR_INVALID_ARG;
    }
    if (p->vote != 0 && p->vote != 1) {
        set_last_error("vote must be 0 or 1");
        return DEPIX_ERR_INVALID_ARG;
    }
    if (layout == DEPIX_LAYOUT_RGBA ? (widthstep < 4 * w || (widthstep & 3)) : (layout != DEPIX_LAYOUT_BGR || widthstep < 3 * w)) {
        set_last_error("refine setup: bad layout or widthstep");
        return DEPIX_ERR_INVALID_ARG;
    }
    cudaStream_t s = reinterpret_cast<cudaStream_t>(s_);
    r->ready = false;
    const int n = w * h, gw = 4 * w + 3, gh = 4 * h + 3, nv = gw * gh;
    if (!d_graph) {
        // the frame's resolved graph: similarity + trivial, then heuristics
        RF_CK(r->own_graph.reserve(n));
        RF_CK(r->own_snap.reserve(n));
        const FrameBatch fb{d_img, 0, r->own_snap.p, 0, w, h, widthstep, (int)layout};
        RF_CK(launch_graph(fb, 1, pack_thresholds(p->tr_y, p->tr_u, p->tr_v, p->yuv), true, s));
        RF_CK(launch_heuristics(GraphBatch{r->own_snap.p, r->own_graph.p, 0, w, h, p->vote}, 1, s));
        d_graph = r->own_graph.p;
    }
    Geo G{d_img, widthstep, (int)layout, d_graph, w, h, gw, gh, r->lut, r->box.p,
          pack_thresholds(p->tr_y, p->tr_u, p->tr_v, p->yuv)};
    RF_CK(r->vgrid.reserve(nv));
    RF_CK(r->cell_count.reserve(n));
    RF_CK(r->cell_off.reserve(n));
    RF_CK(r->is_node.reserve(nv));
    RF_CK(r->nid.reserve(nv));
    RF_CK(r->nb_v.reserve(nv));
    RF_CK(r->nb_e.reserve(nv));
    RF_CK(r->tile_sums.reserve((size_t)nv / kScanTile + 2));
    RF_CK(cudaMemsetAsync(r->vgrid.p, 0, (size_t)nv * sizeof(uint32_t), s));
    k_rf_mark_vertices<<<blocks_for(n), 256, 0, s>>>(G, r->vgrid.p);
    k_rf_count_edges<<<blocks_for(n, 128), 128, 0, s>>>(G, r->vgrid.p, r->cell_count.p);
    RF_CK(cudaGetLastError());
    RF_CK(exclusive_scan(r->cell_count.p, r->cell_off.p, n, r->tile_sums.p, r->scalars.p + 0, s));
    // edges reserved for the most a frame can have, so that E and N come
    // back together: the one read back of the setup (they size the node and
    // segment arrays; the later counts stay on the device)
    RF_CK(r->edges.reserve((size_t)n * r->max_split));
    k_rf_emit_edges<<<blocks_for(n, 128), 128, 0, s>>>(G, r->vgrid.p, r->cell_off.p, r->edges.p, r->nb_v.p, r->nb_e.p);
    k_rf_node_flags<<<blocks_for(nv), 256, 0, s>>>(r->vgrid.p, nv, r->is_node.p);
    RF_CK(cudaGetLastError());
    RF_CK(exclusive_scan(r->is_node.p, r->nid.p, nv, r->tile_sums.p, r->scalars.p + 1, s));
    int EN[2];
    DEPIX_TRY_RF(read_totals(r, 0, 2, EN, s));
    const int E = EN[0], N = EN[1];
    RF_CK(r->node_q.reserve(N));
    RF_CK(r->node_flags.reserve(N));
    RF_CK(r->node_nbr.reserve(N));
    RF_CK(r->node_nbr_edge.reserve(N));
    RF_CK(r->pos0.reserve(N));
    RF_CK(r->pos_a.reserve(N));
    RF_CK(r->pos_b.reserve(N));
    RF_CK(r->gcov.reserve(N));
    RF_CK(r->adam_m.reserve(N));
    RF_CK(r->adam_v.reserve(N));
    NodeOut no{r->node_q.p, r->node_flags.p, r->node_nbr.p, r->node_nbr_edge.p, r->pos0.p};
    k_rf_nodes<<<blocks_for(nv), 256, 0, s>>>(G, r->vgrid.p, r->nid.p, r->nb_v.p, r->nb_e.p, no);
    RF_CK(cudaGetLastError());
    const int S = 3 * E + N;
    RF_CK(r->seg.reserve(S));
    RF_CK(r->seg_col.reserve(S));
    k_rf_segments<<<blocks_for((long long)E + N), 256, 0, s>>>(G, r->nid.p, r->edges.p, E, N, r->node_flags.p,
                                                              r->node_nbr.p, r->node_nbr_edge.p,
                                                              SegOut{r->seg.p, r->seg_col.p});
    // sample assignment
    const int ow = w * p->scale, oh = h * p->scale, no_px = ow * oh;
    RF_CK(r->best.reserve(no_px));
    RF_CK(r->bseg.reserve(no_px));
    RF_CK(r->seg_count.reserve((size_t)S + 1));
    RF_CK(r->seg_off.reserve((size_t)S + 1));
    RF_CK(r->cursor.reserve((size_t)S + 1));
    RF_CK(r->tile_sums.reserve((size_t)std::max(nv, S + 1) / kScanTile + 2));
    RF_CK(cudaMemsetAsync(r->best.p, 0xFF, (size_t)no_px * sizeof(unsigned long long), s));
    RF_CK(cudaMemsetAsync(r->bseg.p, 0x7F, (size_t)no_px * sizeof(int), s)); // kNoSeg
    k_rf_assign_dist<<<blocks_for(S, 128), 128, 0, s>>>(r->seg.p, S, r->node_q.p, p->scale, ow, oh, r->best.p);
    k_rf_assign_seg<<<blocks_for(S, 128), 128, 0, s>>>(r->seg.p, S, r->node_q.p, p->scale, ow, oh, r->best.p,
                                                       r->bseg.p);
    RF_CK(cudaMemsetAsync(r->seg_count.p, 0, ((size_t)S + 1) * sizeof(int), s));
    k_rf_count_samples<<<blocks_for(no_px), 256, 0, s>>>(r->bseg.p, no_px, r->seg_count.p);
    RF_CK(cudaGetLastError());
    RF_CK(exclusive_scan(r->seg_count.p, r->seg_off.p, S + 1, r->tile_sums.p, r->scalars.p + 2, s));
    // samples (M on the device): at most one per output pixel
    RF_CK(r->samp.reserve(no_px));
    RF_CK(r->tgt.reserve(no_px));
    RF_CK(cudaMemsetAsync(r->cursor.p, 0, ((size_t)S + 1) * sizeof(int), s));
    k_rf_scatter_samples<<<blocks_for(no_px), 256, 0, s>>>(r->bseg.p, no_px, r->seg_off.p, r->cursor.p, r->samp.p);
    k_rf_sort_samples<<<blocks_for(S), 256, 0, s>>>(r->seg_off.p, S, r->samp.p);
    k_rf_targets<<<blocks_for(no_px), 256, 0, s>>>(G, p->scale, rp->sigma / (float)p->scale, r->samp.p,
                                                   r->scalars.p + 2, r->tgt.p);
    RF_CK(cudaGetLastError());
    RF_CK(r->sxy.reserve(no_px));
    k_rf_sample_xy<<<blocks_for(no_px), 256, 0, s>>>(r->samp.p, r->scalars.p + 2, ow, p->scale, r->sxy.p);
    // free nodes and their curvature stencils
    RF_CK(r->free_flag.reserve(N));
    RF_CK(r->free_pos.reserve(N));
    RF_CK(r->fnodes.reserve(N));
    k_rf_free_flags<<<blocks_for(N), 256, 0, s>>>(r->node_flags.p, N, r->free_flag.p);
    RF_CK(cudaGetLastError());
    RF_CK(exclusive_scan(r->free_flag.p, r->free_pos.p, N, r->tile_sums.p, r->scalars.p + 3, s));
    k_rf_free_nodes<<<blocks_for(N), 256, 0, s>>>(r->node_flags.p, r->node_nbr.p, r->free_flag.p, r->free_pos.p, N,
                                                  r->fnodes.p);
    RF_CK(cudaGetLastError());
    RF_CK(cudaMemsetAsync(r->gcov.p, 0, (size_t)std::max(N, 1) * sizeof(float2), s));
    r->w = w;
    r->h = h;
    r->scale = p->scale;
    r->ow = ow;
    r->oh = oh;
    r->E = E;
    r->N = N;
    r->S = S;
    r->F = r->M = r->L = -1; // on the device until fetch_counts
    r->sigma = rp->sigma;
    // live segments
    RF_CK(r->live_flag.reserve(S));
    RF_CK(r->live_pos.reserve(S));
    RF_CK(r->live.reserve(S));
    k_rf_live_flags<<<blocks_for(S), 256, 0, s>>>(r->seg.p, r->seg_off.p, S, r->live_flag.p);
    RF_CK(cudaGetLastError());
    RF_CK(exclusive_scan(r->live_flag.p, r->live_pos.p, S, r->tile_sums.p, r->scalars.p + 4, s));
    k_rf_live_scatter<<<blocks_for(S), 256, 0, s>>>(r->live_flag.p, r->live_pos.p, S, r->seg.p, r->seg_off.p,
                                                    r->seg_col.p, r->live.p);
    RF_CK(cudaGetLastError());
    r->tiles_x = (w + kWarmTile - 1) / kWarmTile;
    r->tiles = r->tiles_x * ((h + kWarmTile - 1) / kWarmTile);
    RF_CK(r->tile_hash.reserve(r->tiles));
    k_rf_tile_hash<<<blocks_for(r->tiles, 64), 64, 0, s>>>(G, r->tiles_x, r->tiles, r->tile_hash.p);
    RF_CK(cudaGetLastError());
    k_rf_frame<<<1, 1, 0, s>>>(r->scalars.p, N, ow, oh, p->scale, (float)(1.0 / (3.0 * (double)ow * (double)oh)),
                               r->frame.p);
    RF_CK(cudaGetLastError());
    r->ready = true; // the rest is ordered on s: later calls on s see the frame, others wait on an event of s
    return DEPIX_OK;
}

depix_status depix_refine_counts(depix_refiner* r, long long counts[5])
{
    DEPIX_TRY_RF(check_refiner(r));
    if (!counts) {
        set_last_error("NULL counts");
        return DEPIX_ERR_INVALID_ARG;
    }
    DEPIX_TRY_RF(fetch_counts(r));
    counts[0] = r->N;
    counts[1] = r->F;
    counts[2] = r->E;
    counts[3] = r->S;
    counts[4] = r->M;
    return DEPIX_OK;
}

depix_status depix_refine_export(depix_refiner* r, int32_t* node_q, int32_t* node_flags, int32_t* node_nbr,
                                 int32_t* edges, int32_t* segs, uint32_t* seg_colors, int32_t* samples)
{
    DEPIX_TRY_RF(check_refiner(r));
    DEPIX_TRY_RF(fetch_counts(r));
    if (node_q) RF_CK(cudaMemcpy(node_q, r->node_q.p, (size_t)r->N * sizeof(int2), cudaMemcpyDeviceToHost));
    if (node_flags) RF_CK(cudaMemcpy(node_flags, r->node_flags.p, (size_t)r->N * sizeof(int), cudaMemcpyDeviceToHost));
    if (node_nbr) RF_CK(cudaMemcpy(node_nbr, r->node_nbr.p, (size_t)r->N * sizeof(int2), cudaMemcpyDeviceToHost));
    if (edges) {
        // vertex indices -> node ids on the host copy
        std::vector<int4> ev(r->E);
        std::vector<int> nid((size_t)(4 * r->w + 3) * (4 * r->h + 3));
        RF_CK(cudaMemcpy(ev.data(), r->edges.p, (size_t)r->E * sizeof(int4), cudaMemcpyDeviceToHost));
        RF_CK(cudaMemcpy(nid.data(), r->nid.p, nid.size() * sizeof(int), cudaMemcpyDeviceToHost));
        for (int e = 0; e < r->E; e++) {
            edges[4 * e] = nid[ev[e].x];
            edges[4 * e + 1] = nid[ev[e].y];
            edges[4 * e + 2] = ev[e].z;
            edges[4 * e + 3] = ev[e].w;
        }
    }
    if (segs) RF_CK(cudaMemcpy(segs, r->seg.p, (size_t)r->S * sizeof(int4), cudaMemcpyDeviceToHost));
    if (seg_colors) RF_CK(cudaMemcpy(seg_colors, r->seg_col.p, (size_t)r->S * sizeof(uint2), cudaMemcpyDeviceToHost));
    if (samples) {
        std::vector<int> off((size_t)r->S + 1), smp(r->M);
        RF_CK(cudaMemcpy(off.data(), r->seg_off.p, off.size() * sizeof(int), cudaMemcpyDeviceToHost));
        RF_CK(cudaMemcpy(smp.data(), r->samp.p, smp.size() * sizeof(int), cudaMemcpyDeviceToHost));
        for (int sg = 0; sg < r->S; sg++)
            for (int m = off[sg]; m < off[sg + 1]; m++) {
                samples[2 * m] = smp[m];
                samples[2 * m + 1] = sg;
            }
    }
    return DEPIX_OK;
}

depix_status depix_refine_initial(depix_refiner* r, float* d_pos, depix_stream s)
{
    DEPIX_TRY_RF(check_refiner(r));
    if (!d_pos) {
        set_last_error("NULL positions");
        return DEPIX_ERR_INVALID_ARG;
    }
    RF_CK(cudaMemcpyAsync(d_pos, r->pos0.p, (size_t)r->N * sizeof(float2), cudaMemcpyDeviceToDevice,
                          reinterpret_cast<cudaStream_t>(s)));
    return DEPIX_OK;
}

depix_status depix_refine_warm_start(depix_refiner* r, const depix_refiner* prev, const float* d_prev_pos,
                                     float* d_pos, int* reused_tiles, depix_stream s_)
{
    DEPIX_TRY_RF(check_refiner(r));
    if (!prev || !prev->ready || !d_prev_pos || !d_pos) {
        set_last_error("warm start: previous refiner without a frame, or NULL positions");
        return DEPIX_ERR_INVALID_ARG;
    }
    if (prev->w != r->w || prev->h != r->h) {
        set_last_error("warm start: the previous frame has another size");
        return DEPIX_ERR_INVALID_ARG;
    }
    cudaStream_t s = reinterpret_cast<cudaStream_t>(s_);
    const int gw = 4 * r->w + 3, nv = gw * (4 * r->h + 3);
    if (r->warm_grid.cap < (size_t)nv || !r->warm_grid.p) {
        RF_CK(r->warm_grid.reserve(nv));
        RF_CK(r->warm_stamp.reserve(nv));
        RF_CK(cudaMemsetAsync(r->warm_stamp.p, 0, (size_t)nv * sizeof(int), s));
        r->warm_epoch = 0;
    }
    const int epoch = ++r->warm_epoch;
    k_rf_warm_scatter<<<blocks_for(prev->N), 256, 0, s>>>(prev->node_q.p, reinterpret_cast<const float2*>(d_prev_pos),
                                                          prev->N, gw, r->warm_grid.p, r->warm_stamp.p, epoch);
    k_rf_warm_gather<<<blocks_for(r->N), 256, 0, s>>>(r->node_q.p, r->pos0.p, r->N, r->w, r->h, gw, r->tiles_x,
                                                      r->tile_hash.p, prev->tile_hash.p, r->warm_grid.p,
                                                      r->warm_stamp.p, epoch, reinterpret_cast<float2*>(d_pos));
    RF_CK(cudaGetLastError());
    if (reused_tiles) {
        RF_CK(cudaMemsetAsync(r->scalars.p + 5, 0, sizeof(int), s));
        k_rf_same_tiles<<<blocks_for(r->tiles), 256, 0, s>>>(r->tile_hash.p, prev->tile_hash.p, r->tiles,
                                                             r->scalars.p + 5);
        RF_CK(cudaGetLastError());
        DEPIX_TRY_RF(read_totals(r, 5, 1, reused_tiles, s));
    }
    return DEPIX_OK;
}

depix_status depix_refine_energy_grad(depix_refiner* r, const depix_refine_params* p, const float* d_pos,
                                      float* d_grad, double energy[4], depix_stream s)
{
    DEPIX_TRY_RF(check_refiner(r));
    DEPIX_TRY_RF(check_rparams(p));
    DEPIX_TRY_RF(check_sigma(r, p));
    if (!d_pos || !energy) {
        set_last_error("NULL positions or energy");
        return DEPIX_ERR_INVALID_ARG;
    }
    return eval(r, p, reinterpret_cast<const float2*>(d_pos), reinterpret_cast<float2*>(d_grad), energy,
                reinterpret_cast<cudaStream_t>(s));
}

depix_status depix_refine_run(depix_refiner* r, const depix_refine_params* p, float* d_pos, double before[4],
                              double after[4], depix_stream s_)
{
    DEPIX_TRY_RF(check_refiner(r));
    DEPIX_TRY_RF(check_rparams(p));
    DEPIX_TRY_RF(check_sigma(r, p));
    cudaStream_t s = reinterpret_cast<cudaStream_t>(s_);
    const size_t bytes = (size_t)r->N * sizeof(float2);
    float2* x = r->pos_a.p;
    float2* y = r->pos_b.p;
    k_rf_begin<<<std::min(blocks_for(r->N), r->sms * 4), 256, 0, s>>>(
        d_pos ? reinterpret_cast<const float2*>(d_pos) : r->pos0.p, x, y, r->adam_m.p, r->adam_v.p, r->N);
    RF_CK(cudaGetLastError());
    if (before) DEPIX_TRY_RF(eval(r, p, x, nullptr, before, s));
    const StepArgs a = step_args(r, p);
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    RF_CK(cudaStreamIsCapturing(s, &cs));
    if (p->steps > 0 && cs == cudaStreamCaptureStatusNone) {
        if (!r->loop || r->loop_steps != p->steps || !same_loop(a, r->loop_args) ||
            r->loop_args.x != r->pos_a.p || r->loop_args.y != r->pos_b.p || r->loop_cov_blocks != cov_blocks(r) ||
            r->loop_node_blocks != node_blocks(r)) {
            if (r->loop) cudaGraphExecDestroy(r->loop);
            r->loop = nullptr;
            RF_CK(cudaStreamBeginCapture(r->capture_stream, cudaStreamCaptureModeThreadLocal));
            cudaError_t e = launch_steps(r, a, p->steps, r->capture_stream);
            cudaGraph_t g = nullptr;
            const cudaError_t e2 = cudaStreamEndCapture(r->capture_stream, &g);
            if (e == cudaSuccess) e = e2;
            if (e == cudaSuccess) e = cudaGraphInstantiate(&r->loop, g, 0);
            if (g) cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                r->loop = nullptr;
                return rf_fail(e, "refine loop capture");
            }
            r->loop_args = a;
            r->loop_args.x = r->pos_a.p;
            r->loop_args.y = r->pos_b.p;
            r->loop_steps = p->steps;
            r->loop_cov_blocks = cov_blocks(r);
            r->loop_node_blocks = node_blocks(r);
        }
        RF_CK(cudaGraphLaunch(r->loop, s));
    } else {
        RF_CK(launch_steps(r, a, p->steps, s));
    }
    if (p->steps & 1) x = y;
    if (after) DEPIX_TRY_RF(eval(r, p, x, nullptr, after, s));
    if (d_pos) RF_CK(cudaMemcpyAsync(d_pos, x, bytes, cudaMemcpyDeviceToDevice, s));
    return DEPIX_OK;
}

}  // extern "C"
