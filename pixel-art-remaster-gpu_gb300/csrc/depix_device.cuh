// depix_device.cuh -- device-side building blocks shared by the kernels.
//
// Geometry is carried in exact integers: every coordinate the reference
// produces is a multiple of 1/64 of a cell (hull points are multiples of
// 1/4, one corner-cutting round and the neighbour midpoints add three more
// halvings), and its float and double arithmetic on such values is exact. So
// the hull, subdivision and ear-clip decisions below, made on integers in
// 1/64-cell units, are the reference's decisions bit for bit.
#pragma once

#include <cstdint>
#include <cuda.h> // CUtensorMap (the type only; the encoder comes through the runtime's driver entry point)
#include <cuda_runtime.h>

#include "../../include/depix.h"

namespace depix {

constexpr int kCell = 45;    // slots per cell in the VBO layout (kernel.cu:8)
constexpr int kMaxHull = 8;  // largest reshaped-cell hull over all 4096 patterns
constexpr int kMaxPoly = 16; // one subdivision round at most doubles the hull
constexpr int kUnit = 64;    // geometry units per cell

// neighbour offset of node bit e (graph_functions.cu:162-235), j upward
__host__ __device__ __forceinline__ int dir_di(int e) { return ((0x9224 >> (2 * e)) & 3) - 1; }
__host__ __device__ __forceinline__ int dir_dj(int e) { return ((0x016A >> (2 * e)) & 3) - 1; }
__host__ __device__ __forceinline__ int bitof(unsigned v, int k) { return (int)((v >> k) & 1u); }

// bits of a node whose neighbour lies inside the image
__device__ __forceinline__ unsigned inside_mask(int x, int y, int w, int h)
{
    unsigned m = 0xFFu;
    if (x == 0) m &= ~0x29u;     // 0, 3, 5
    if (x == w - 1) m &= ~0x94u; // 2, 4, 7
    if (y == 0) m &= ~0xE0u;     // 5, 6, 7
    if (y == h - 1) m &= ~0x07u; // 0, 1, 2
    return m;
}

// ------------------------------------------------------------------ colour

// Packed Y/U/V word of one pixel from its bytes in the reference's memory
// order (b0 plays "r", b2 plays "b": RGBtoYUV + DATAtoINT,
// graph_functions.cu:80-131). y is the truncated double 0.299 r + 0.587 g +
// 0.114 b, evaluated as one of the reference's two builds evaluates it
// (depix_params.yuv):
//  - DEPIX_YUV_CUDA: its CUDA build (nvcc contracts the sum into fused
//    multiply-adds): fma(0.114, b, fma(0.299, r, 0.587 g));
//  - DEPIX_YUV_HOST: its host build, IEEE with no contraction:
//    (0.299 r + 0.587 g) + 0.114 b.
// Off exact multiples of 1/1000 the sum is at least 0.001 away from an
// integer, and either evaluation truncates to the integer quotient of
// 299 r + 587 g + 114 b by 1000; only a zero remainder needs the double
// evaluation, where the two builds differ for 2490 of the 2^24 colours.
__device__ __forceinline__ uint32_t yuv_word(int r, int g, int b, int mode)
{
    int s = 299 * r + 587 * g + 114 * b;
    int y = s / 1000;
    if (s - y * 1000 == 0) {
        double t;
        if (mode == DEPIX_YUV_HOST) {
            t = __dadd_rn(__dmul_rn(0.299, (double)r), __dmul_rn(0.587, (double)g));
            t = __dadd_rn(t, __dmul_rn(0.114, (double)b));
        } else {
            t = __fma_rn(0.114, (double)b, __fma_rn(0.299, (double)r, __dmul_rn(0.587, (double)g)));
        }
        y = __double2int_rz(t);
    }
    int u = __float2int_rz(__fmul_rn((float)(b - y), 0.492f));
    int v = __float2int_rz(__fmul_rn((float)(r - y), 0.877f));
    return (uint32_t)(y * 65536 + u * 256 + v);
}

// Thresholds packed like a word (a field threshold above 255 can never be
// exceeded), with the y arithmetic (depix_params.yuv) in bits 24-31: the
// similarity test ignores that byte, so the kernels that build words carry
// the mode in the thresholds they already take.
__host__ __device__ __forceinline__ uint32_t pack_thresholds(int ty, int tu, int tv, int yuv)
{
    auto c = [](int t) { return (uint32_t)(t < 0 ? 0 : (t > 255 ? 255 : t)); };
    return ((uint32_t)(yuv & 0xFF) << 24) | (c(ty) << 16) | (c(tu) << 8) | c(tv);
}

__host__ __device__ __forceinline__ int yuv_mode_of(uint32_t thr) { return (int)(thr >> 24); }

// similarity of two words: every masked field within its threshold
// (graph_functions.cu:291-293)
__device__ __forceinline__ bool similar(uint32_t a, uint32_t b, uint32_t thr)
{
    return (__vcmpleu4(__vabsdiffu4(a, b), thr) & 0x00FFFFFFu) == 0x00FFFFFFu;
}

// Reference-layout bytes of one pixel (b0, b1, b2) packed little-endian.
__device__ __forceinline__ uint32_t load_bgr(const uint8_t* img, int ws, int layout, int i, int j)
{
    if (layout == DEPIX_LAYOUT_RGBA) {
        uint32_t p = __ldg(reinterpret_cast<const uint32_t*>(img + (size_t)j * ws) + i);
        // RGBA -> B,G,R
        return ((p >> 16) & 0xFFu) | (p & 0xFF00u) | ((p & 0xFFu) << 16);
    }
    const uint8_t* q = img + (size_t)j * ws + 3 * i;
    return (uint32_t)__ldg(q) | ((uint32_t)__ldg(q + 1) << 8) | ((uint32_t)__ldg(q + 2) << 16);
}

// word of packed bytes c = b0 | b1 << 8 | b2 << 16 under the y arithmetic
// carried in the packed thresholds thr
__device__ __forceinline__ uint32_t word_of_bgr(uint32_t c, uint32_t thr)
{
    return yuv_word((int)(c & 0xFF), (int)((c >> 8) & 0xFF), (int)((c >> 16) & 0xFF), yuv_mode_of(thr));
}

// Byte at linear offset `off` of the reference's BGR image (rows `vws` bytes,
// 3*w used, zero padding), zero outside the image. For RGBA input the
// reference image is the 4-byte-aligned BGR image it would have loaded.
__device__ __forceinline__ int ref_byte(const uint8_t* img, int w, int h, int ws, int layout, long long off)
{
    if (layout == DEPIX_LAYOUT_BGR) {
        if (off < 0 || off >= (long long)h * ws) return 0;
        return __ldg(img + off);
    }
    int vws = (3 * w + 3) & ~3;
    if (off < 0 || off >= (long long)h * vws) return 0;
    int row = (int)(off / vws), col = (int)(off % vws);
    if (col >= 3 * w) return 0;
    int px = col / 3, ch = col % 3; // ch 0 = B, 1 = G, 2 = R
    return __ldg(img + (size_t)row * ws + 4 * px + (2 - ch));
}

__device__ __forceinline__ int ref_stride(int w, int ws, int layout)
{
    return layout == DEPIX_LAYOUT_BGR ? ws : ((3 * w + 3) & ~3);
}

// 3-byte colour equality at two linear offsets (isColorEqual, subdivision_functions.cu:157-167)
__device__ __forceinline__ bool ref_color_eq(const uint8_t* img, int w, int h, int ws, int layout, long long a,
                                             long long b)
{
    return ref_byte(img, w, h, ws, layout, a) == ref_byte(img, w, h, ws, layout, b) &&
           ref_byte(img, w, h, ws, layout, a + 1) == ref_byte(img, w, h, ws, layout, b + 1) &&
           ref_byte(img, w, h, ws, layout, a + 2) == ref_byte(img, w, h, ws, layout, b + 2);
}

// T-junction test at vertex (cx, cy) of cell (i, j) (checkTJunction,
// subdivision_functions.cu:170-242): its bounds test (written with the width
// in place of the stride) answers true for any vertex; past it only the four
// corners can answer true. Reads the image through linear offsets.
static __device__ __noinline__ bool t_junction_global(const uint8_t* img, int w, int h, int ws, int layout, int i, int j,
                                               int cx, int cy)
{
    long long st = ref_stride(w, ws, layout);
    long long index = (long long)j * st + (long long)i * 3;
    if ((index - st - 1) < 0 || (index + w + 1) > ((long long)h * st - 1)) return true;
    long long c0 = index + st - 3, c1 = index + st, c2 = index + st + 3, c3 = index - 3, c4 = index + 3;
    long long c5 = index - st - 3, c6 = index - st, c7 = index - st + 3;
#define EQ(a, b) ref_color_eq(img, w, h, ws, layout, a, b)
    if (cx == 0 && cy == 0 && (!EQ(c3, c5) || !EQ(c5, c6))) return true;
    if (cx == kUnit && cy == 0 && (!EQ(c4, c7) || !EQ(c7, c6))) return true;
    if (cx == kUnit && cy == kUnit && (!EQ(c1, c2) || !EQ(c2, c4))) return true;
    if (cx == 0 && cy == kUnit && (!EQ(c0, c1) || !EQ(c1, c3))) return true;
#undef EQ
    return false;
}

// ------------------------------------------------------- cell pattern tables

// Pattern of a cell: node byte (bits 0-7), left neighbour bit 2 (8) and
// bit 7 (9), right neighbour bit 0 (10) and bit 5 (11): all that decides its
// reshaped polygon (createCellFromPattern, diagram_functions.cu:320-520).
__device__ __forceinline__ int cell_pattern(unsigned node, unsigned left, unsigned right)
{
    return (int)(node & 0xFF) | (bitof(left, 2) << 8) | (bitof(left, 7) << 9) | (bitof(right, 0) << 10) |
           (bitof(right, 5) << 11);
}

// A cell polygon in 1/64-cell units. Every vertex lies in [-0.75, 1.75] of
// its cell (hull points in [-0.25, 1.25]; subdivision midpoints pair an own
// point with a neighbour's), i.e. in [-48, 112]: int8 storage keeps the
// per-thread arrays small.
struct Poly {
    int n;
    int8_t x[kMaxPoly];
    int8_t y[kMaxPoly];
};

// Decodes a hull table entry (built once per device in depix_geom.cu):
// vertex count in bits 0-3, then 8 vertices of 6 bits (x+1 | (y+1) << 3,
// quarter units).
__device__ __forceinline__ void hull_from_lut(uint64_t e, Poly& p)
{
    p.n = (int)(e & 0xF);
#pragma unroll
    for (int t = 0; t < kMaxHull; t++) {
        unsigned v = (unsigned)(e >> (4 + 6 * t)) & 63u;
        p.x[t] = (int8_t)(((int)(v & 7) - 1) * (kUnit / 4));
        p.y[t] = (int8_t)(((int)(v >> 3) - 1) * (kUnit / 4));
    }
}

// ------------------------------------------------------------- subdivision

__device__ __forceinline__ int pmod(int i, int n) { return (n + (i % n)) % n; }

// Neighbour direction an edge is shared with, or -1 (isLinkedEdge,
// subdivision_functions.cu:245-424). In integer units the float slope test
// "== +-1" is dy == +-dx with dx != 0, and the 0.5 tests compare with 32.
__device__ __forceinline__ int edge_link(const Poly& c, unsigned node, int idx)
{
    int b = pmod(idx + 1, c.n);
    int ax = c.x[idx], ay = c.y[idx], bx = c.x[b], by = c.y[b];
    int dx = bx - ax, dy = by - ay, my2 = ay + by;
    const int half = kUnit / 2;
    if (ay == by && ay > half && bitof(node, 1)) return 1;
    if (ax == bx && ax > half && bitof(node, 4)) return 4;
    if (ay == by && ay < half && bitof(node, 6)) return 6;
    if (ax == bx && ax < half && bitof(node, 3)) return 3;
    bool s1 = dx != 0 && dy == dx, sm1 = dx != 0 && dy == -dx;
    if (s1 && my2 > kUnit && bitof(node, 0)) return 0;
    if (sm1 && my2 > kUnit && bitof(node, 2)) return 2;
    if (s1 && my2 < kUnit && bitof(node, 7)) return 7;
    if (sm1 && my2 < kUnit && bitof(node, 5)) return 5;
    return -1;
}

// corner-cutting points on edge i -> i+1 (getQ_i / getR_i,
// subdivision_functions.cu:42-122): 3/4-1/4 when the edge is at most one cell
// long, else 7/8-1/8.
__device__ __forceinline__ void qr_point(const Poly& c, int i, bool want_r, int& ox, int& oy)
{
    int a = i % c.n;
    if (a < 0) a += c.n;
    int b = (i + 1) % c.n;
    int px = c.x[a], py = c.y[a], nx = c.x[b], ny = c.y[b];
    int l2 = (nx - px) * (nx - px) + (ny - py) * (ny - py);
    if (l2 <= kUnit * kUnit) {
        if (want_r) { ox = (px + 3 * nx) / 4; oy = (py + 3 * ny) / 4; }
        else { ox = (3 * px + nx) / 4; oy = (3 * py + ny) / 4; }
    } else {
        if (want_r) { ox = (px + 7 * nx) / 8; oy = (py + 7 * ny) / 8; }
        else { ox = (7 * px + nx) / 8; oy = (7 * py + ny) / 8; }
    }
}

// Q (or R) point of a linked neighbour's hull around the vertex matching
// (px, py), mapped back to this cell (get{Q,R}_i_from_linked_cell,
// subdivision_functions.cu:125-154; getPointIndex falls back to index 0).
__device__ __forceinline__ void linked_point(const Poly& nb, int link, int px, int py, bool want_r, int& ox,
                                             int& oy)
{
    int tx = px - kUnit * dir_di(link), ty = py - kUnit * dir_dj(link);
    int op = 0;
    for (int t = 0; t < nb.n; t++)
        if (nb.x[t] == tx && nb.y[t] == ty) { op = t; break; }
    qr_point(nb, want_r ? op - 1 : op, want_r, ox, oy);
    ox += kUnit * dir_di(link);
    oy += kUnit * dir_dj(link);
}

// One corner-cutting round of a cell (subdivision, subdivision_functions.cu:564-669).
// NbHull(link, Poly&) fetches the hull of the neighbour in direction link;
// TJ(cx, cy) is the T-junction test at a cell corner.
template <typename NbHull, typename TJ>
__device__ void subdivide_cell(const Poly& c, unsigned node, NbHull nb_hull, TJ tj, Poly& out)
{
    int link[kMaxHull];
    for (int e = 0; e < c.n; e++) link[e] = edge_link(c, node, e);
    int m = 0;
    Poly nb;
    for (int v = 0; v < c.n; v++) {
        int lp = link[pmod(v - 1, c.n)];
        bool cur = link[v] >= 0, prev = lp >= 0;
        int px = c.x[v], py = c.y[v];
        if (!cur && !prev) {
            // the test's image-bounds check answers "keep" for any vertex of
            // the cells it covers, before it looks at corners
            if (tj(px, py)) {
                out.x[m] = (int8_t)px; out.y[m] = (int8_t)py; m++;
            } else {
                int rx, ry, qx, qy;
                qr_point(c, v - 1, true, rx, ry);
                qr_point(c, v, false, qx, qy);
                out.x[m] = (int8_t)rx; out.y[m] = (int8_t)ry; m++;
                out.x[m] = (int8_t)qx; out.y[m] = (int8_t)qy; m++;
            }
        } else if (!cur && prev) {
            int qx, qy, ax, ay;
            qr_point(c, v, false, qx, qy);
            nb_hull(lp, nb);
            linked_point(nb, lp, px, py, true, ax, ay);
            out.x[m] = (int8_t)((qx + ax) / 2); out.y[m] = (int8_t)((qy + ay) / 2); m++;
            out.x[m] = (int8_t)qx; out.y[m] = (int8_t)qy; m++;
        } else if (cur && !prev) {
            int rx, ry, ax, ay;
            nb_hull(link[v], nb);
            linked_point(nb, link[v], px, py, false, ax, ay);
            qr_point(c, v - 1, true, rx, ry);
            out.x[m] = (int8_t)rx; out.y[m] = (int8_t)ry; m++;
            out.x[m] = (int8_t)((rx + ax) / 2); out.y[m] = (int8_t)((ry + ay) / 2); m++;
        } else {
            out.x[m] = (int8_t)px; out.y[m] = (int8_t)py; m++;
        }
    }
    out.n = m;
}

// ----------------------------------------------------------- ear clipping

__device__ __forceinline__ bool inside_tri(int Ax, int Ay, int Bx, int By, int Cx, int Cy, int Px, int Py)
{
    int a = (Cx - Bx) * (Py - By) - (Cy - By) * (Px - Bx);
    int c = (Bx - Ax) * (Py - Ay) - (By - Ay) * (Px - Ax);
    int b = (Ax - Cx) * (Py - Cy) - (Ay - Cy) * (Px - Cx);
    return a >= 0 && b >= 0 && c >= 0;
}

// Ear clipping (process / snip / area, triangulate_functions.cu:6-217) in
// integer units: the reference's EPSILON test on an exact product of
// 1/64-multiples is "cross <= 0". Writes corner indices, returns the triangle
// count; ok = false when the reference's loop guard gives up.
__device__ __forceinline__ int ear_clip(const Poly& c, uint8_t* tri, bool& ok)
{
    ok = true;
    int n = c.n;
    if (n < 3) { ok = false; return 0; }
    int area = 0;
    for (int p = n - 1, q = 0; q < n; p = q++) area += c.x[p] * c.y[q] - c.x[q] * c.y[p];
    uint8_t V[kMaxPoly];
    for (int v = 0; v < n; v++) V[v] = (uint8_t)(area > 0 ? v : (n - 1) - v);
    int nv = n, nt = 0, count = 2 * nv;
    for (int v = nv - 1; nv > 2;) {
        if (0 >= (count--)) { ok = false; return nt; }
        int u = v;
        if (nv <= u) u = 0;
        v = u + 1;
        if (nv <= v) v = 0;
        int w = v + 1;
        if (nv <= w) w = 0;
        int Ax = c.x[V[u]], Ay = c.y[V[u]], Bx = c.x[V[v]], By = c.y[V[v]], Cx = c.x[V[w]], Cy = c.y[V[w]];
        bool ear = ((Bx - Ax) * (Cy - Ay) - (By - Ay) * (Cx - Ax)) > 0;
        if (ear) {
            // a point outside the triangle's bounding box cannot be inside or on it
            const int x0 = min(Ax, min(Bx, Cx)), x1 = max(Ax, max(Bx, Cx));
            const int y0 = min(Ay, min(By, Cy)), y1 = max(Ay, max(By, Cy));
            for (int p = 0; p < nv; p++) {
                if (p == u || p == v || p == w) continue;
                const int Px = c.x[V[p]], Py = c.y[V[p]];
                if (Px < x0 || Px > x1 || Py < y0 || Py > y1) continue;
                if (inside_tri(Ax, Ay, Bx, By, Cx, Cy, Px, Py)) { ear = false; break; }
            }
        }
        if (ear) {
            tri[3 * nt] = (uint8_t)V[u];
            tri[3 * nt + 1] = (uint8_t)V[v];
            tri[3 * nt + 2] = (uint8_t)V[w];
            nt++;
            for (int s = v, t = v + 1; t < nv; s++, t++) V[s] = V[t];
            nv--;
            count = 2 * nv;
        }
    }
    return nt;
}

// ------------------------------------------------------------------ raster

// Sample coverage of one triangle under the top-left rule, all in integer
// units of 1/256 output pixel relative to a common origin. The triangle is
// taken counter-clockwise (y up); zero area covers nothing.
__device__ __forceinline__ bool covers(int ax, int ay, int bx, int by, int cx, int cy, int sx, int sy)
{
    int area = (bx - ax) * (cy - ay) - (by - ay) * (cx - ax);
    if (area == 0) return false;
    if (area < 0) {
        int tx = bx, ty = by;
        bx = cx; by = cy; cx = tx; cy = ty;
    }
    int ex, ey, f;
    ex = bx - ax; ey = by - ay; f = ex * (sy - ay) - ey * (sx - ax);
    if (!(f > 0 || (f == 0 && (ey < 0 || (ey == 0 && ex < 0))))) return false;
    ex = cx - bx; ey = cy - by; f = ex * (sy - by) - ey * (sx - bx);
    if (!(f > 0 || (f == 0 && (ey < 0 || (ey == 0 && ex < 0))))) return false;
    ex = ax - cx; ey = ay - cy; f = ex * (sy - cy) - ey * (sx - cx);
    if (!(f > 0 || (f == 0 && (ey < 0 || (ey == 0 && ex < 0))))) return false;
    return true;
}

}  // namespace depix

namespace depix {

// ------------------------------------------- register-packed cell geometry
//
// The mask path keeps a cell's geometry in registers: a hull as its 64-bit
// pattern-table entry, a cut polygon as 16 signed-byte coordinates per axis in
// two 64-bit words. Same decisions as the Poly-based functions above.

struct Packed {
    uint64_t x0, x1, y0, y1; // vertex t: byte (t & 7) of (t < 8 ? *0 : *1)
    int n;
};

__device__ __forceinline__ int pk_get(uint64_t lo, uint64_t hi, int t)
{
    uint64_t w = t < 8 ? lo : hi;
    return (int)(int8_t)(uint8_t)(w >> ((t & 7) * 8));
}

__device__ __forceinline__ void pk_put(Packed& P, int t, int x, int y)
{
    const int sh = (t & 7) * 8;
    const uint64_t keep = ~(0xFFull << sh);
    const uint64_t bx = (uint64_t)(uint8_t)x << sh, by = (uint64_t)(uint8_t)y << sh;
    if (t < 8) {
        P.x0 = (P.x0 & keep) | bx;
        P.y0 = (P.y0 & keep) | by;
    } else {
        P.x1 = (P.x1 & keep) | bx;
        P.y1 = (P.y1 & keep) | by;
    }
}

// hull vertex t of a pattern-table entry, in 1/64 cell
__device__ __forceinline__ int hx(uint64_t e, int t) { return ((int)((e >> (4 + 6 * t)) & 7u) - 1) * (kUnit / 4); }
__device__ __forceinline__ int hy(uint64_t e, int t) { return ((int)((e >> (7 + 6 * t)) & 7u) - 1) * (kUnit / 4); }

// edge_link (isLinkedEdge) on a hull entry
__device__ __forceinline__ int hull_edge_link(uint64_t e, int n, unsigned node, int idx)
{
    int b = idx + 1 == n ? 0 : idx + 1;
    int ax = hx(e, idx), ay = hy(e, idx), bx = hx(e, b), by = hy(e, b);
    int dx = bx - ax, dy = by - ay, my2 = ay + by;
    const int half = kUnit / 2;
    if (ay == by && ay > half && bitof(node, 1)) return 1;
    if (ax == bx && ax > half && bitof(node, 4)) return 4;
    if (ay == by && ay < half && bitof(node, 6)) return 6;
    if (ax == bx && ax < half && bitof(node, 3)) return 3;
    bool s1 = dx != 0 && dy == dx, sm1 = dx != 0 && dy == -dx;
    if (s1 && my2 > kUnit && bitof(node, 0)) return 0;
    if (sm1 && my2 > kUnit && bitof(node, 2)) return 2;
    if (s1 && my2 < kUnit && bitof(node, 7)) return 7;
    if (sm1 && my2 < kUnit && bitof(node, 5)) return 5;
    return -1;
}

// getQ_i / getR_i on a hull entry (index i taken modulo n, as the reference)
__device__ __forceinline__ void hull_qr(uint64_t e, int n, int i, bool want_r, int& ox, int& oy)
{
    int a = i % n;
    if (a < 0) a += n;
    int b = (i + 1) % n;
    int px = hx(e, a), py = hy(e, a), nx = hx(e, b), ny = hy(e, b);
    int l2 = (nx - px) * (nx - px) + (ny - py) * (ny - py);
    int wp, wn, d;
    if (l2 <= kUnit * kUnit) {
        wp = want_r ? 1 : 3;
        wn = want_r ? 3 : 1;
        d = 4;
    } else {
        wp = want_r ? 1 : 7;
        wn = want_r ? 7 : 1;
        d = 8;
    }
    ox = (wp * px + wn * nx) / d;
    oy = (wp * py + wn * ny) / d;
}

// One corner-cutting round on a hull entry into a packed polygon
// (subdivision, subdivision_functions.cu:564-669). NbEntry(link) returns the
// pattern-table entry of the neighbour in that direction; TJ(px, py) is the
// corner test.
template <typename NbEntry, typename TJ>
__device__ __forceinline__ void subdivide_packed(uint64_t e, unsigned node, NbEntry nb_entry, TJ tj, Packed& out)
{
    const int n = (int)(e & 0xF);
    uint32_t links = 0; // 4 bits per edge: link direction, 15 = border
    for (int v = 0; v < n; v++) links |= (uint32_t)(hull_edge_link(e, n, node, v) & 15) << (4 * v);
    out.x0 = out.x1 = out.y0 = out.y1 = 0;
    int m = 0;
    for (int v = 0; v < n; v++) {
        const int lc = (int)((links >> (4 * v)) & 15u);
        const int lp = (int)((links >> (4 * (v == 0 ? n - 1 : v - 1))) & 15u);
        const bool cur = lc != 15, prev = lp != 15;
        const int px = hx(e, v), py = hy(e, v);
        int qx, qy, rx, ry;
        hull_qr(e, n, v, false, qx, qy);
        hull_qr(e, n, v - 1, true, rx, ry);
        if (cur == prev) {
            if (cur || tj(px, py)) {
                pk_put(out, m++, px, py);
            } else {
                pk_put(out, m++, rx, ry);
                pk_put(out, m++, qx, qy);
            }
            continue;
        }
        // exactly one adjacent edge is linked: the neighbour's R (previous
        // edge linked) or Q (current edge linked) around the matching vertex
        const int L = prev ? lp : lc;
        const uint64_t ne = nb_entry(L);
        const int nn = (int)(ne & 0xF);
        const int tx = px - kUnit * dir_di(L), ty = py - kUnit * dir_dj(L);
        int op = 0;
        for (int t = 0; t < nn; t++)
            if (hx(ne, t) == tx && hy(ne, t) == ty) {
                op = t;
                break;
            }
        int ax, ay;
        hull_qr(ne, nn, prev ? op - 1 : op, prev, ax, ay);
        ax += kUnit * dir_di(L);
        ay += kUnit * dir_dj(L);
        if (prev) { // current edge border: mid(Q, R_adjacent), Q
            pk_put(out, m++, (qx + ax) / 2, (qy + ay) / 2);
            pk_put(out, m++, qx, qy);
        } else { // current edge linked: R, mid(R, Q_adjacent)
            pk_put(out, m++, rx, ry);
            pk_put(out, m++, (rx + ax) / 2, (ry + ay) / 2);
        }
    }
    out.n = m;
}

// bit k set where byte k of m is 0xFF (m from a per-byte SIMD compare)
__device__ __forceinline__ unsigned byte_bits(uint32_t m) { return (((m >> 7) & 0x01010101u) * 0x10204080u) >> 28; }

// vertices (bit t) whose point lies in [x0,x1] x [y0,y1]
__device__ __forceinline__ unsigned in_box16(const Packed& P, int x0, int x1, int y0, int y1)
{
    const uint32_t bx0 = (uint8_t)x0 * 0x01010101u, bx1 = (uint8_t)x1 * 0x01010101u;
    const uint32_t by0 = (uint8_t)y0 * 0x01010101u, by1 = (uint8_t)y1 * 0x01010101u;
    unsigned m = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        uint32_t xw = (uint32_t)((k < 2 ? P.x0 : P.x1) >> (32 * (k & 1)));
        uint32_t yw = (uint32_t)((k < 2 ? P.y0 : P.y1) >> (32 * (k & 1)));
        uint32_t in = __vcmpges4(xw, bx0) & __vcmples4(xw, bx1) & __vcmpges4(yw, by0) & __vcmples4(yw, by1);
        m |= byte_bits(in) << (4 * k);
    }
    return m;
}

}  // namespace depix

namespace depix {

// Ear clipping (process / snip / area, triangulate_functions.cu:6-217) on a
// packed polygon. Index list V as 4-bit entries of one word; the inside test
// runs only for the vertices in the ear's bounding box (a vertex outside it
// cannot be inside or on the triangle). Each ear goes to on_tri(A, B, C) as
// it is found. Returns the ear count; ok = false when the reference's loop
// guard gives up.
template <typename OnTri>
__device__ __forceinline__ int ear_clip_packed(const Packed& P, OnTri on_tri, bool& ok)
{
    ok = true;
    const int n = P.n;
    if (n < 3) {
        ok = false;
        return 0;
    }
    int area = 0;
    for (int p = n - 1, q = 0; q < n; p = q++)
        area += pk_get(P.x0, P.x1, p) * pk_get(P.y0, P.y1, q) - pk_get(P.x0, P.x1, q) * pk_get(P.y0, P.y1, p);
    uint64_t V = 0;
    for (int v = 0; v < n; v++) V |= (uint64_t)(area > 0 ? v : n - 1 - v) << (4 * v);
    unsigned alive = (1u << n) - 1u;
    int nv = n, nt = 0, count = 2 * nv;
    for (int v = nv - 1; nv > 2;) {
        if (0 >= (count--)) {
            ok = false;
            return nt;
        }
        int u = v;
        if (nv <= u) u = 0;
        v = u + 1;
        if (nv <= v) v = 0;
        int w = v + 1;
        if (nv <= w) w = 0;
        const int A = (int)((V >> (4 * u)) & 15u), B = (int)((V >> (4 * v)) & 15u), C = (int)((V >> (4 * w)) & 15u);
        const int Ax = pk_get(P.x0, P.x1, A), Ay = pk_get(P.y0, P.y1, A);
        const int Bx = pk_get(P.x0, P.x1, B), By = pk_get(P.y0, P.y1, B);
        const int Cx = pk_get(P.x0, P.x1, C), Cy = pk_get(P.y0, P.y1, C);
        bool ear = ((Bx - Ax) * (Cy - Ay) - (By - Ay) * (Cx - Ax)) > 0;
        if (ear) {
            unsigned cand = alive & ~((1u << A) | (1u << B) | (1u << C)) &
                            in_box16(P, min(Ax, min(Bx, Cx)), max(Ax, max(Bx, Cx)), min(Ay, min(By, Cy)),
                                     max(Ay, max(By, Cy)));
            while (cand) {
                const int p = __ffs(cand) - 1;
                cand &= cand - 1u;
                if (inside_tri(Ax, Ay, Bx, By, Cx, Cy, pk_get(P.x0, P.x1, p), pk_get(P.y0, P.y1, p))) {
                    ear = false;
                    break;
                }
            }
        }
        if (ear) {
            on_tri(Ax, Ay, Bx, By, Cx, Cy);
            nt++;
            const uint64_t low = (1ull << (4 * v)) - 1ull;
            V = (V & low) | ((V >> 4) & ~low);
            alive &= ~(1u << B);
            nv--;
            count = 2 * nv;
        }
    }
    return nt;
}

}  // namespace depix

namespace depix {

__device__ __forceinline__ int floor_div(int a, int b) // b > 0
{
    int q = a / b;
    return (a % b != 0 && a < 0) ? q - 1 : q;
}

// floor(a / b) and a - b * floor(a / b) for b > 0, |a| < 2^30, |a / b| < 2^20:
// a float estimate (off by less than one: a loses at most 2^6 in the
// conversion, b >= 256 in every use, relative error 2^-23) corrected once in
// each direction with exact integer arithmetic.
__device__ __forceinline__ int floor_div_fast(int a, int b, int& rem)
{
    int q = __float2int_rd(__fdividef((float)a, (float)b));
    int r = a - q * b;
    if (r < 0) {
        q--;
        r += b;
    }
    if (r >= b) {
        q++;
        r -= b;
    }
    rem = r;
    return q;
}

// True when every edge turns strictly counter-clockwise around the cell
// centre (32, 32) and the polygon winds around it exactly once: the vertices
// are then in increasing angle around the centre, so the polygon is
// star-shaped about it, hence simple. For a simple polygon the reference's
// ear clip never gives up (every position is tried within nv attempts and a
// simple polygon always has an ear its test accepts) and its triangles tile
// the polygon exactly.
__device__ __forceinline__ bool star_simple(const Packed& P)
{
    const int n = P.n;
    if (n < 3) return false;
    int px = pk_get(P.x0, P.x1, n - 1) - kUnit / 2, py = pk_get(P.y0, P.y1, n - 1) - kUnit / 2;
    int wraps = 0;
    for (int i = 0; i < n; i++) {
        const int x = pk_get(P.x0, P.x1, i) - kUnit / 2, y = pk_get(P.y0, P.y1, i) - kUnit / 2;
        if (px * y - py * x <= 0) return false;
        // a counter-clockwise step of less than half a turn from the lower to
        // the upper half-plane passes angle 0
        const bool up_prev = py > 0 || (py == 0 && px > 0), up = y > 0 || (y == 0 && x > 0);
        wraps += (!up_prev && up) ? 1 : 0;
        px = x;
        py = y;
    }
    return wraps == 1;
}

// Footprint coverage of a simple polygon (vertices x u, in 1/256 output
// pixel) by crossing number at the sample point shifted by (+e, -e^2): the
// same set the top-left rule gives for any exact triangulation of it. Each
// edge toggles, on every sample row it crosses, the samples left of the
// crossing; the crossing column steps from row to row by an exact rational
// increment (quotient and remainder), so no division per row.
__device__ __forceinline__ void crossing_mask(const Packed& P, int u, int mlo, int F, uint32_t* rows, int rstride)
{
    const int n = P.n;
    int bx = pk_get(P.x0, P.x1, n - 1) * u, by = pk_get(P.y0, P.y1, n - 1) * u;
    for (int i = 0; i < n; i++) {
        int ax = bx, ay = by;
        bx = pk_get(P.x0, P.x1, i) * u;
        by = pk_get(P.y0, P.y1, i) * u;
        if (ay == by) continue;
        int lx = ax, ly = ay, hxx = bx, hyy = by;
        if (ly > hyy) {
            lx = bx; ly = by; hxx = ax; hyy = ay;
        }
        // rows whose sample height py = 256 row + 128 has ly < py <= hyy
        const int r0 = max(((ly - 128) >> 8) + 1, mlo), r1 = min((hyy - 128) >> 8, mlo + F - 1);
        if (r0 > r1) continue;
        const int D = hyy - ly, den = 256 * D;
        // samples left of the crossing: 256 m + 128 < x_cross  <=>  m < num / den
        int num = lx * D + (256 * r0 + 128 - ly) * (hxx - lx) - 128 * D;
        const int step = 256 * (hxx - lx);
        int r, sr;
        int q = floor_div_fast(num, den, r);
        const int sq = floor_div_fast(step, den, sr);
        for (int row = r0; row <= r1; row++) {
            const int k = q + (r > 0 ? 1 : 0) - mlo; // ceil(num / den) - mlo
            rows[(row - mlo) * rstride] ^= k <= 0 ? 0u : (k >= 32 ? 0xFFFFFFFFu : ((1u << k) - 1u));
            q += sq;
            r += sr;
            if (r >= den) {
                r -= den;
                q++;
            }
        }
    }
    const uint32_t fmask = F >= 32 ? 0xFFFFFFFFu : ((1u << F) - 1u);
    for (int row = 0; row < F; row++) rows[row * rstride] &= fmask;
}

// star_simple, the polygon's bounding box and crossing_mask in one pass over
// the vertices. Returns star_simple's answer; the rows are only meaningful
// when it is true (the caller clears them and ear-clips otherwise).
__device__ __forceinline__ bool star_crossing_mask(const Packed& P, int u, int mlo, int F, uint32_t* rows, int rstride,
                                                   int& mnx, int& mny, int& mxx, int& mxy)
{
    const int n = P.n;
    int px = pk_get(P.x0, P.x1, n - 1), py = pk_get(P.y0, P.y1, n - 1);
    mnx = mxx = px;
    mny = mxy = py;
    bool ok = n >= 3;
    int wraps = 0;
    for (int i = 0; i < n; i++) {
        const int x = pk_get(P.x0, P.x1, i), y = pk_get(P.y0, P.y1, i);
        mnx = min(mnx, x);
        mxx = max(mxx, x);
        mny = min(mny, y);
        mxy = max(mxy, y);
        // star test about the cell centre
        const int cx0 = px - kUnit / 2, cy0 = py - kUnit / 2, cx1 = x - kUnit / 2, cy1 = y - kUnit / 2;
        ok &= cx0 * cy1 - cy0 * cx1 > 0;
        const bool up_prev = cy0 > 0 || (cy0 == 0 && cx0 > 0), up = cy1 > 0 || (cy1 == 0 && cx1 > 0);
        wraps += (!up_prev && up) ? 1 : 0;
        // crossings of the edge prev -> this vertex
        const int ax = px * u, ay = py * u, bx = x * u, by = y * u;
        px = x;
        py = y;
        if (ay == by) continue;
        int lx = ax, ly = ay, hxx = bx, hyy = by;
        if (ly > hyy) {
            lx = bx; ly = by; hxx = ax; hyy = ay;
        }
        const int r0 = max(((ly - 128) >> 8) + 1, mlo), r1 = min((hyy - 128) >> 8, mlo + F - 1);
        if (r0 > r1) continue;
        const int D = hyy - ly, den = 256 * D;
        int num = lx * D + (256 * r0 + 128 - ly) * (hxx - lx) - 128 * D;
        const int step = 256 * (hxx - lx);
        int r, sr;
        int q = floor_div_fast(num, den, r);
        const int sq = floor_div_fast(step, den, sr);
        for (int row = r0; row <= r1; row++) {
            const int k = q + (r > 0 ? 1 : 0) - mlo;
            rows[(row - mlo) * rstride] ^= k <= 0 ? 0u : (k >= 32 ? 0xFFFFFFFFu : ((1u << k) - 1u));
            q += sq;
            r += sr;
            if (r >= den) {
                r -= den;
                q++;
            }
        }
    }
    const uint32_t fmask = F >= 32 ? 0xFFFFFFFFu : ((1u << F) - 1u);
    for (int row = 0; row < F; row++) rows[row * rstride] &= fmask;
    return ok && wraps == 1;
}

// ------------------------------------------------- TMA tile loads (sm_90+)

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// Waits for the phase with the given parity to complete, at most max_iter
// polls; false when it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int max_iter)
{
    for (int i = 0; i < max_iter; i++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Polls a block allows a TMA tile load before it gives up (about a second on
// GB300 at most; a load completes in microseconds).
constexpr int kTmaPolls = 1 << 22;

// Waits for the tile load completing on bar. When the wait gives up, it sets
// the stage's sticky fault flag and then waits again, bounded the same way,
// for the load it issued, so that a load still in flight does not land in
// shared memory after the block has left; the block then leaves its tile
// unwritten. False when the first wait gave up.
__device__ __forceinline__ bool tma_wait_or_flag(uint64_t* bar, int* fault, int polls = kTmaPolls)
{
    if (mbar_wait_bounded(bar, 0, polls)) return true;
    atomicExch(fault, 1);
    mbar_wait_bounded(bar, 0, polls);
    return false;
}

// One 3-D tile of a tensor map into shared memory, completing on bar. The
// innermost coordinate times the element size must be a multiple of 16
// bytes (the caller guarantees it); out-of-range elements read as zero.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

}  // namespace depix

namespace depix {

// Persistent work loop: the block pulls `gran` tile indices at a time from
// *counter until `total` is reached and runs body(t) on each; a barrier
// separates tiles (the bodies reuse shared memory). No block waits on
// another: a block stops when the counter passes the end.
template <typename Body>
__device__ __forceinline__ void queue_loop(int* counter, int total, int gran, Body body)
{
    __shared__ int s_first;
    for (;;) {
        if (threadIdx.x == 0) s_first = atomicAdd(counter, gran);
        __syncthreads();
        const int t0 = s_first;
        __syncthreads();
        if (t0 >= total) break;
        const int t1 = min(t0 + gran, total);
        for (int t = t0; t < t1; t++) {
            body(t);
            __syncthreads();
        }
    }
}

// The same with each warp pulling its own tiles (bodies that need no
// barrier: one warp per tile).
template <typename Body>
__device__ __forceinline__ void warp_queue_loop(int* counter, int total, int gran, Body body)
{
    const int lane = threadIdx.x & 31;
    for (;;) {
        int t0 = 0;
        if (lane == 0) t0 = atomicAdd(counter, gran);
        t0 = __shfl_sync(0xFFFFFFFFu, t0, 0);
        if (t0 >= total) break;
        const int t1 = min(t0 + gran, total);
        for (int t = t0; t < t1; t++) body(t);
    }
}

// the frame f with base[f] <= t < base[f + 1]
__device__ __forceinline__ int queue_frame(const uint32_t* base, int n, uint32_t t)
{
    int lo = 0, hi = n;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(base + mid) <= t) lo = mid;
        else hi = mid;
    }
    return lo;
}

}  // namespace depix
