// depix_geom.cu -- reshaped cells, subdivision, triangulation, VBO output
// and the headless rasterizer.
//
// A cell's hull depends only on 12 bits of the resolved graph (its node byte
// and two bits of each row neighbour), so the hull and its ear clip are
// computed once per device for all 4096 patterns by k_init_tables and looked
// up afterwards. Corner cutting and the ear clip of the cut polygon depend on
// neighbours and on the image, and are computed per cell.
#include "depix_internal.h"

namespace depix {

__device__ uint64_t g_hull_lut[4096];
__device__ uint64_t g_tri_lut[4096];
// Per pattern and hull vertex v: the corner-cutting case of v (bits 0-1:
// 0 both adjacent edges linked, 1 both border, 2 only the previous edge
// linked, 3 only the current edge linked) and, for 2 and 3, that edge's link
// direction (bits 2-4); 5 bits per vertex.
__device__ uint64_t g_vk_lut[4096];
// Per pattern and hull vertex v: Q on edge v -> v+1 near v and R on edge
// v-1 -> v near v (getQ_i(v), getR_i(v-1)), as int8 x, y, x, y in 1/64 cell.
__device__ __align__(16) uint32_t g_qr_lut[4096 * 8];
// Per pattern: bit e set when the hull reaches into the open square of
// neighbour e (hull bounding box test).
__device__ uint8_t g_spill_lut[4096];

// ------------------------------------------------------ pattern tables

struct QP {
    int x, y; // quarter units
};

// Cell points in emission order, directions 0,1,2,4,7,6,5,3
// (createCellFromPattern, diagram_functions.cu:320-520). The misses of bits 4
// and 6 emit (0.75,0.75) and (0.25,0.75) as the reference does.
__device__ int cell_points(unsigned nd, unsigned left, unsigned right, QP* p)
{
    int n = 0;
    auto put = [&](int x, int y) { p[n].x = x; p[n].y = y; n++; };
    // corner direction d between sides a (first) and b (second): both sides
    // present -> two points; one side -> the point on the other side's axis
    if (bitof(nd, 0)) {
        if (bitof(nd, 1) && !bitof(nd, 3)) put(-1, 3);
        else if (bitof(nd, 3) && !bitof(nd, 1)) put(1, 5);
        else { put(-1, 3); put(1, 5); }
    } else if (bitof(left, 2)) put(1, 3);
    else put(0, 4);
    if (bitof(nd, 1)) { put(0, 4); put(4, 4); }
    else put(2, 3);
    if (bitof(nd, 2)) {
        if (bitof(nd, 1) && !bitof(nd, 4)) put(5, 3);
        else if (bitof(nd, 4) && !bitof(nd, 1)) put(3, 5);
        else { put(3, 5); put(5, 3); }
    } else if (bitof(right, 0)) put(3, 3);
    else put(4, 4);
    if (bitof(nd, 4)) { put(4, 4); put(4, 0); }
    else put(3, 3);
    if (bitof(nd, 7)) {
        if (bitof(nd, 4) && !bitof(nd, 6)) put(3, -1);
        else if (bitof(nd, 6) && !bitof(nd, 4)) put(5, 1);
        else { put(5, 1); put(3, -1); }
    } else if (bitof(right, 5)) put(3, 1);
    else put(4, 0);
    if (bitof(nd, 6)) { put(4, 0); put(0, 0); }
    else put(1, 3);
    if (bitof(nd, 5)) {
        if (bitof(nd, 3) && !bitof(nd, 6)) put(1, -1);
        else if (bitof(nd, 6) && !bitof(nd, 3)) put(-1, 1);
        else { put(1, -1); put(-1, 1); }
    } else if (bitof(left, 7)) put(1, 1);
    else put(0, 0);
    if (bitof(nd, 3)) { put(0, 0); put(0, 4); }
    else put(1, 2);
    return n;
}

__device__ __forceinline__ void qswap(QP& a, QP& b)
{
    QP t = a;
    a = b;
    b = t;
}

// The reference's point ordering (sort + sort_y, diagram_functions.cu:37-129):
// gather all points with the smallest remaining x to the front, then bring
// the smallest y of that group to its front. Ties beyond two points stay in
// scan order, as in the reference.
__device__ void lex_order(QP* P, int n)
{
    int done = 0;
    while (done < n) {
        int lo = 1 << 20, tie = 0, idx[kMaxPoly];
        for (int i = done; i < n; i++) {
            if (P[i].x < lo) { lo = P[i].x; tie = 0; idx[0] = i; }
            else if (P[i].x == lo) idx[++tie] = i;
        }
        for (int t = 0; t <= tie; t++) qswap(P[done + t], P[idx[t]]);
        if (tie > 0) {
            int ly = 1 << 20, yt = 0, yidx[kMaxPoly];
            for (int i = done; i <= done + tie; i++) {
                if (P[i].y < ly) { ly = P[i].y; yt = 0; yidx[0] = i; }
                else if (P[i].y == ly) yidx[++yt] = i;
            }
            for (int t = 0; t <= yt; t++) qswap(P[done + t], P[yidx[t]]);
        }
        done += tie + 1;
    }
}

__device__ __forceinline__ int qcross(QP o, QP a, QP b) { return (a.x - o.x) * (b.y - o.y) - (a.y - o.y) * (b.x - o.x); }

// Monotone chain (convex_hull, diagram_functions.cu:239-316); returns the
// vertex count, H[0..count-1] counter-clockwise from the first sorted point.
__device__ int monotone_hull(QP* P, int n, QP* H)
{
    lex_order(P, n);
    int k = 0;
    for (int i = 0; i < n; i++) {
        while (k >= 2 && qcross(H[k - 2], H[k - 1], P[i]) <= 0) k--;
        H[k++] = P[i];
    }
    for (int i = n - 2, t = k + 1; i >= 0; i--) {
        while (k >= t && qcross(H[k - 2], H[k - 1], P[i]) <= 0) k--;
        H[k++] = P[i];
    }
    return k - 1;
}

__global__ void k_init_tables()
{
    int pat = blockIdx.x * blockDim.x + threadIdx.x;
    if (pat >= 4096) return;
    unsigned node = pat & 0xFF;
    unsigned left = ((unsigned)bitof(pat, 8) << 2) | ((unsigned)bitof(pat, 9) << 7);
    unsigned right = (unsigned)bitof(pat, 10) | ((unsigned)bitof(pat, 11) << 5);
    QP P[kMaxPoly], H[2 * kMaxPoly];
    int np = cell_points(node, left, right, P);
    int k = monotone_hull(P, np, H);
    uint64_t e = (uint64_t)k;
    for (int t = 0; t < k && t < kMaxHull; t++)
        e |= (uint64_t)((H[t].x + 1) | ((H[t].y + 1) << 3)) << (4 + 6 * t);
    g_hull_lut[pat] = e;
    Poly c;
    hull_from_lut(e, c);
    uint8_t tri[3 * kMaxPoly];
    bool ok;
    int nt = ear_clip(c, tri, ok);
    uint64_t te = 0;
    for (int q = 0; q < 3 * nt; q++) te |= (uint64_t)tri[q] << (3 * q);
    g_tri_lut[pat] = te;
    // vertex cases and corner-cutting points
    int links[kMaxHull];
    for (int v = 0; v < k; v++) links[v] = hull_edge_link(e, k, node, v);
    uint64_t vk = 0;
    for (int v = 0; v < kMaxHull; v++) {
        uint32_t qr = 0;
        if (v < k) {
            const int lc = links[v], lp = links[v == 0 ? k - 1 : v - 1];
            const bool cur = lc >= 0, prev = lp >= 0;
            const int kind = cur == prev ? (cur ? 0 : 1) : (prev ? 2 : 3);
            const int L = kind == 2 ? lp : (kind == 3 ? lc : 0);
            vk |= (uint64_t)(kind | (L << 2)) << (5 * v);
            int qx, qy, rx, ry;
            hull_qr(e, k, v, false, qx, qy);
            hull_qr(e, k, v - 1, true, rx, ry);
            qr = (uint32_t)(uint8_t)qx | ((uint32_t)(uint8_t)qy << 8) | ((uint32_t)(uint8_t)rx << 16) |
                 ((uint32_t)(uint8_t)ry << 24);
        }
        g_qr_lut[pat * 8 + v] = qr;
    }
    g_vk_lut[pat] = vk;
    int mnx = 1 << 20, mny = 1 << 20, mxx = -(1 << 20), mxy = -(1 << 20);
    for (int t = 0; t < k; t++) {
        mnx = min(mnx, hx(e, t)); mxx = max(mxx, hx(e, t));
        mny = min(mny, hy(e, t)); mxy = max(mxy, hy(e, t));
    }
    unsigned sp = 0;
    for (int d = 0; d < 8; d++) {
        int sx = kUnit * dir_di(d), sy = kUnit * dir_dj(d);
        if (mxx > sx && mnx < sx + kUnit && mxy > sy && mny < sy + kUnit) sp |= 1u << d;
    }
    g_spill_lut[pat] = (uint8_t)sp;
}

cudaError_t init_tables(cudaStream_t s)
{
    k_init_tables<<<16, 256, 0, s>>>();
    return cudaGetLastError();
}

cudaError_t hull_table_address(const uint64_t** out)
{
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_hull_lut);
    *out = static_cast<const uint64_t*>(p);
    return e;
}

cudaError_t copy_tables(uint64_t* hull, uint64_t* tri)
{
    cudaError_t e = cudaMemcpyFromSymbol(hull, g_hull_lut, sizeof(g_hull_lut));
    if (e == cudaSuccess) e = cudaMemcpyFromSymbol(tri, g_tri_lut, sizeof(g_tri_lut));
    return e;
}

// ------------------------------------------- 45-slot stage entry points

__device__ __forceinline__ unsigned linear_at(const uint8_t* g, int n, int idx)
{
    return (idx < 0 || idx >= n) ? 0u : (unsigned)g[idx];
}

// cells_Kernel (kernel.cu:192-213): row neighbours read linearly
__global__ void k_cells(const uint8_t* g, int w, int h, float2* diagram, int* ec)
{
    int idx = blockIdx.x * blockDim.x + threadIdx.x, n = w * h;
    if (idx >= n) return;
    int pat = cell_pattern(g[idx], linear_at(g, n, idx - 1), linear_at(g, n, idx + 1));
    Poly c;
    hull_from_lut(__ldg(&g_hull_lut[pat]), c);
    float2* cell = diagram + (size_t)idx * kCell;
    const float inv = 1.0f / kUnit;
    for (int t = 0; t < kCell; t++) {
        float2 v = make_float2(0.f, 0.f);
        if (t <= c.n) {
            int q = t < c.n ? t : 0;
            v = make_float2((float)c.x[q] * inv, (float)c.y[q] * inv);
        }
        cell[t] = v;
    }
    ec[idx] = c.n;
}

__device__ __forceinline__ bool poly_from_slots(const float2* cell, int n, int cap, Poly& p)
{
    if (n < 3 || n > cap) return false;
    p.n = n;
    for (int t = 0; t < n; t++) {
        float2 v = cell[t];
        p.x[t] = (int8_t)__float2int_rn(v.x * (float)kUnit);
        p.y[t] = (int8_t)__float2int_rn(v.y * (float)kUnit);
    }
    return true;
}

// subdivision_Kernel (kernel.cu:216-261): reads the snapshot, skips byte 90
__global__ void k_subdivide(const uint8_t* img, int w, int h, int ws, int layout, const uint8_t* g,
                            const float2* snap, const int* ec_snap, float2* diagram, int* ec)
{
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= w * h) return;
    unsigned node = g[idx];
    if (node == 90) return;
    int i = idx % w, j = idx / w;
    Poly c, out;
    if (!poly_from_slots(snap + (size_t)idx * kCell, ec_snap[idx], kMaxHull, c)) return;
    auto nb_hull = [&](int link, Poly& p) {
        // linear neighbour index as the reference computes it; a bit that
        // points past either end of the frame finds no cell
        int nb = idx + dir_dj(link) * w + dir_di(link);
        if (nb < 0 || nb >= w * h || !poly_from_slots(snap + (size_t)nb * kCell, ec_snap[nb], kMaxHull, p)) {
            p.n = 1;
            p.x[0] = p.y[0] = 0;
        }
    };
    auto tj = [&](int px, int py) { return t_junction_global(img, w, h, ws, layout, i, j, px, py); };
    subdivide_cell(c, node, nb_hull, tj, out);
    float2* cell = diagram + (size_t)idx * kCell;
    const float inv = 1.0f / kUnit;
    for (int t = 0; t < out.n; t++) cell[t] = make_float2((float)out.x[t] * inv, (float)out.y[t] * inv);
    ec[idx] = out.n;
}

// triangulate_Kernel (kernel.cu:264-282): triangle corners + (i, j) in the
// first 3*count slots; the remaining slots get (-100, -100)
__global__ void k_triangulate(float2* diagram, const int* ec, int w, int h)
{
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= w * h) return;
    int i = idx % w, j = idx / w;
    float2* cell = diagram + (size_t)idx * kCell;
    Poly c;
    int nt = 0;
    uint8_t tri[3 * kMaxPoly];
    if (poly_from_slots(cell, ec[idx], kMaxPoly, c)) {
        bool ok;
        nt = ear_clip(c, tri, ok);
    }
    const float inv = 1.0f / kUnit;
    for (int t = 0; t < kCell; t++) {
        float2 v = make_float2(-100.f, -100.f);
        if (t < 3 * nt) v = make_float2((float)c.x[tri[t]] * inv + (float)i, (float)c.y[tri[t]] * inv + (float)j);
        cell[t] = v;
    }
}

// position_kernel + color_kernel (kernel.cu:67-137)
__global__ void k_emit(const uint8_t* img, int w, int h, int ws, int layout, const float2* diagram, const int* ec,
                       float2* pos, uchar4* col)
{
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= w * h) return;
    int i = idx % w, j = idx / w;
    int lim = (ec[idx] - 2) * 3;
    size_t base = (size_t)idx * kCell;
    if (pos)
        for (int t = 0; t < kCell; t++) pos[base + t] = t < lim ? diagram[base + t] : make_float2(-100.f, -100.f);
    if (col) {
        uint32_t c = load_bgr(img, ws, layout, i, j);
        uchar4 v = make_uchar4((c >> 16) & 0xFF, (c >> 8) & 0xFF, c & 0xFF, 255);
        for (int t = 0; t < kCell; t++) col[base + t] = v;
    }
}

static dim3 grid1(int n, int b) { return dim3((n + b - 1) / b); }

cudaError_t launch_cells(const uint8_t* g, int w, int h, float* diagram, int* ec, cudaStream_t s)
{
    k_cells<<<grid1(w * h, 128), 128, 0, s>>>(g, w, h, reinterpret_cast<float2*>(diagram), ec);
    return cudaGetLastError();
}

cudaError_t launch_subdivide(const uint8_t* img, int w, int h, int ws, int layout, const uint8_t* g,
                             const float* snap, const int* ec_snap, float* diagram, int* ec, cudaStream_t s)
{
    k_subdivide<<<grid1(w * h, 128), 128, 0, s>>>(img, w, h, ws, layout, g, reinterpret_cast<const float2*>(snap),
                                                   ec_snap, reinterpret_cast<float2*>(diagram), ec);
    return cudaGetLastError();
}

cudaError_t launch_triangulate(float* diagram, const int* ec, int w, int h, cudaStream_t s)
{
    k_triangulate<<<grid1(w * h, 128), 128, 0, s>>>(reinterpret_cast<float2*>(diagram), ec, w, h);
    return cudaGetLastError();
}

cudaError_t launch_emit(const uint8_t* img, int w, int h, int ws, int layout, const float* diagram, const int* ec,
                        float* pos, uint8_t* col, cudaStream_t s)
{
    k_emit<<<grid1(w * h, 128), 128, 0, s>>>(img, w, h, ws, layout, reinterpret_cast<const float2*>(diagram), ec,
                                             reinterpret_cast<float2*>(pos), reinterpret_cast<uchar4*>(col));
    return cudaGetLastError();
}

// ------------------------------------------------------------------ raster
//
// One CTA per tile of kRTW x kRTH cells. Phase A stages the resolved graph
// (halo 3: a ring cell's linked neighbours need their own row neighbours) and
// the pixels (halo 2: corner tests of ring cells) in shared memory. Phase B
// builds the triangles of the tile's cells and of the ring around it (ring
// cells reach 0.25 cell into the tile). Phase C shades every output pixel of
// the tile as a gather: of the 3x3 cells around its sample, the one latest in
// VBO order (highest row, then highest column) whose triangles cover the
// sample gives the colour; rows of 4 pixels go out as one 16-byte store.

constexpr int kRTW = 32, kRTH = 8;
constexpr int kGW = kRTW + 2, kGH = kRTH + 2, kGN = kGW * kGH;
constexpr int kBW = kRTW + 6, kBH = kRTH + 6;
constexpr int kCW = kRTW + 4, kCH = kRTH + 4;
constexpr int kMaxTri = kMaxPoly - 2;

struct RasterShared {
    uint8_t graph[kBH][kBW];
    uint32_t pix[kCH][kCW];
    int8_t vx[kGN][kMaxPoly];
    int8_t vy[kGN][kMaxPoly];
    uint8_t tri[kGN][3 * kMaxTri];
    uint8_t nt[kGN];
    int8_t bb[kGN][4];
};


template <int LAYOUT>
__device__ void raster_tile(RasterShared& S, const uint8_t* img, int ws, const uint8_t* g, uint8_t* out, int w,
                            int h, int scale, bool subdivide, int x0, int y0)
{
    // ---- phase A
    for (int k = threadIdx.x; k < kBW * kBH; k += blockDim.x) {
        int gx = x0 - 3 + k % kBW, gy = y0 - 3 + k / kBW;
        unsigned v = 0;
        if (gx >= 0 && gy >= 0 && gx < w && gy < h) v = __ldg(g + (size_t)gy * w + gx) & inside_mask(gx, gy, w, h);
        S.graph[k / kBW][k % kBW] = (uint8_t)v;
    }
    for (int k = threadIdx.x; k < kCW * kCH; k += blockDim.x) {
        int gx = x0 - 2 + k % kCW, gy = y0 - 2 + k / kCW;
        uint32_t v = 0;
        if (gx >= 0 && gy >= 0 && gx < w && gy < h) v = load_bgr(img, ws, LAYOUT, gx, gy);
        S.pix[k / kCW][k % kCW] = v;
    }
    __syncthreads();

    // ---- phase B
    for (int k = threadIdx.x; k < kGN; k += blockDim.x) {
        int lx = k % kGW, ly = k / kGW;
        int ci = x0 - 1 + lx, cj = y0 - 1 + ly;
        if (ci < 0 || cj < 0 || ci >= w || cj >= h) {
            S.nt[k] = 0;
            continue;
        }
        const int bx = lx + 2, by = ly + 2;
        unsigned node = S.graph[by][bx];
        int pat = cell_pattern(node, S.graph[by][bx - 1], S.graph[by][bx + 1]);
        Poly c;
        hull_from_lut(__ldg(&g_hull_lut[pat]), c);
        int nt;
        if (subdivide && node != 90) {
            auto nb_hull = [&](int link, Poly& p) {
                int nx = bx + dir_di(link), ny = by + dir_dj(link);
                int np = cell_pattern(S.graph[ny][nx], S.graph[ny][nx - 1], S.graph[ny][nx + 1]);
                hull_from_lut(__ldg(&g_hull_lut[np]), p);
            };
            auto tj = [&](int px, int py) -> bool {
                long long st = LAYOUT == DEPIX_LAYOUT_BGR ? ws : ((3 * w + 3) & ~3);
                long long index = (long long)cj * st + (long long)ci * 3;
                if ((index - st - 1) < 0 || (index + w + 1) > ((long long)h * st - 1)) return true;
                if (ci == 0 || ci == w - 1 || cj >= h - 1)
                    return t_junction_global(img, w, h, ws, LAYOUT, ci, cj, px, py);
                const int qx = lx + 1, qy = ly + 1; // this pixel in S.pix
                auto C = [&](int dx, int dy) { return S.pix[qy + dy][qx + dx]; };
                if (px == 0 && py == 0) return C(-1, 0) != C(-1, -1) || C(-1, -1) != C(0, -1);
                if (px == kUnit && py == 0) return C(1, 0) != C(1, -1) || C(1, -1) != C(0, -1);
                if (px == kUnit && py == kUnit) return C(0, 1) != C(1, 1) || C(1, 1) != C(1, 0);
                if (px == 0 && py == kUnit) return C(-1, 1) != C(0, 1) || C(0, 1) != C(-1, 0);
                return false;
            };
            Poly sp;
            subdivide_cell(c, node, nb_hull, tj, sp);
            bool ok;
            nt = ear_clip(sp, S.tri[k], ok);
            c = sp;
        } else {
            uint64_t te = __ldg(&g_tri_lut[pat]);
            nt = c.n - 2;
            for (int q = 0; q < 3 * nt; q++) S.tri[k][q] = (uint8_t)((te >> (3 * q)) & 7u);
        }
        int mnx = 127, mny = 127, mxx = -128, mxy = -128;
        for (int t = 0; t < c.n; t++) {
            S.vx[k][t] = c.x[t];
            S.vy[k][t] = c.y[t];
            mnx = min(mnx, c.x[t]); mxx = max(mxx, c.x[t]);
            mny = min(mny, c.y[t]); mxy = max(mxy, c.y[t]);
        }
        S.nt[k] = (uint8_t)nt;
        S.bb[k][0] = (int8_t)mnx; S.bb[k][1] = (int8_t)mny;
        S.bb[k][2] = (int8_t)mxx; S.bb[k][3] = (int8_t)mxy;
    }
    __syncthreads();

    // ---- phase C
    const int s = scale, u = 4 * s;
    const int ow = w * s, oh = h * s;
    const int OW = kRTW * s, OH = kRTH * s;
    const int X0 = x0 * s, Y0 = y0 * s;
    const bool vec = (ow % 4) == 0 && ((reinterpret_cast<uintptr_t>(out) & 15) == 0);
    for (int q = threadIdx.x; q < (OW / 4) * OH; q += blockDim.x) {
        int r = q / (OW / 4), c4 = 4 * (q % (OW / 4));
        int Y = Y0 + r;
        if (Y >= oh) continue;
        int cj = Y / s;
        uint32_t v[4];
#pragma unroll
        for (int e = 0; e < 4; e++) {
            int X = X0 + c4 + e;
            uint32_t color = 0xFF000000u;
            if (X < ow) {
                int ci = X / s;
                int SX = 256 * X + 128, SY = 256 * Y + 128;
                bool hit = false;
                for (int dj = 1; dj >= -1 && !hit; dj--)
                    for (int di = 1; di >= -1 && !hit; di--) {
                        int lx = ci + di - (x0 - 1), ly = cj + dj - (y0 - 1);
                        int k = ly * kGW + lx;
                        int nt = S.nt[k];
                        if (nt == 0) continue;
                        int rx = SX - (ci + di) * 256 * s, ry = SY - (cj + dj) * 256 * s;
                        if (rx < S.bb[k][0] * u || rx > S.bb[k][2] * u || ry < S.bb[k][1] * u || ry > S.bb[k][3] * u)
                            continue;
                        for (int t = 0; t < nt; t++) {
                            int a = S.tri[k][3 * t], b = S.tri[k][3 * t + 1], cc = S.tri[k][3 * t + 2];
                            if (covers(S.vx[k][a] * u, S.vy[k][a] * u, S.vx[k][b] * u, S.vy[k][b] * u,
                                       S.vx[k][cc] * u, S.vy[k][cc] * u, rx, ry)) {
                                uint32_t p = S.pix[ly + 1][lx + 1]; // ring cell -> pixel tile
                                color = ((p >> 16) & 0xFFu) | (p & 0xFF00u) | ((p & 0xFFu) << 16) | 0xFF000000u;
                                hit = true;
                                break;
                            }
                        }
                    }
            }
            v[e] = color;
        }
        size_t o = ((size_t)Y * ow + (size_t)(X0 + c4)) * 4;
        if (vec && X0 + c4 + 3 < ow) {
            __stcs(reinterpret_cast<uint4*>(out + o), make_uint4(v[0], v[1], v[2], v[3]));
        } else {
            for (int e = 0; e < 4; e++)
                if (X0 + c4 + e < ow) reinterpret_cast<uint32_t*>(out + o)[e] = v[e];
        }
    }
}

template <int LAYOUT>
__global__ void __launch_bounds__(256) k_raster(RasterBatch b)
{
    __shared__ RasterShared S;
    size_t z = blockIdx.z;
    raster_tile<LAYOUT>(S, b.img + b.img_stride * z, b.ws, b.graph + b.graph_stride * z, b.out + b.out_stride * z,
                        b.w, b.h, b.scale, b.subdivide != 0, blockIdx.x * kRTW, blockIdx.y * kRTH);
}

cudaError_t launch_raster(const RasterBatch& b, int nframes, cudaStream_t s)
{
    dim3 grid((b.w + kRTW - 1) / kRTW, (b.h + kRTH - 1) / kRTH, nframes);
    if (b.layout == DEPIX_LAYOUT_RGBA)
        k_raster<DEPIX_LAYOUT_RGBA><<<grid, 256, 0, s>>>(b);
    else
        k_raster<DEPIX_LAYOUT_BGR><<<grid, 256, 0, s>>>(b);
    return cudaGetLastError();
}


// ------------------------------------------------------------ mask raster
//
// The gather above tests triangles per output pixel. This raster instead
// reduces every cell to a coverage bitmask over the samples its polygon can
// reach and resolves each output block with bit operations:
//
//  - a cell polygon lies inside [-0.75, 1.75]^2 of its own cell: hull points
//    lie in [-0.25, 1.25], subdivision adds midpoints of an own point and a
//    neighbour's point (neighbour hull shifted by one cell);
//  - footprint: output samples (X+0.5)/s in that box, offsets m = X - i*s in
//    [mlo, mlo + F); one 32-bit row word per footprint row (F <= 32, s <= 12);
//  - plain cells (no subdivision) take their rows from a per-scale table over
//    the 4096 hull patterns; subdivided cells are gathered into a list and
//    cut, ear-clipped and masked one per thread;
//  - an output block (the s x s samples of one cell) takes, per sample, the
//    latest covering cell in VBO order among the 3x3 cells around it. A cell
//    whose block its own mask fills and no neighbour polygon reaches is
//    filled without per-sample work.

struct MaskGeom {
    int s;
    int mlo, F;   // footprint of any cell polygon
    int hlo, HF;  // footprint of a hull (no subdivision): [-0.25, 1.25]
};

__host__ __device__ __forceinline__ MaskGeom mask_geom(int s)
{
    MaskGeom g;
    g.s = s;
    g.mlo = -((3 * s + 2) / 4);
    g.F = (7 * s - 2) / 4 - g.mlo + 1;
    g.hlo = -((s + 2) / 4);
    g.HF = (5 * s - 2) / 4 - g.hlo + 1;
    return g;
}

// Sets the footprint samples (offsets mlo.. in both axes, F of them) that the
// triangle covers under the top-left rule. Vertices in 1/256 output pixel
// relative to the cell origin.
__device__ __forceinline__ void tri_mask(int ax, int ay, int bx, int by, int cx, int cy, int mlo, int F,
                                         uint32_t* rows, int rstride = 1)
{
    int area = (bx - ax) * (cy - ay) - (by - ay) * (cx - ax);
    if (area == 0) return;
    if (area < 0) {
        int tx = bx, ty = by;
        bx = cx; by = cy; cx = tx; cy = ty;
    }
    // E(p) = A px + B py + C; covered iff E >= bias on all three edges, where
    // bias 0 on a top or left edge (dy < 0, or dy == 0 and dx < 0 with
    // dx = B, dy = -A) and 1 elsewhere: E > 0, or E == 0 on a top/left edge
    const int A0 = ay - by, B0 = bx - ax, C0 = -(A0 * ax + B0 * ay);
    const int A1 = by - cy, B1 = cx - bx, C1 = -(A1 * bx + B1 * by);
    const int A2 = cy - ay, B2 = ax - cx, C2 = -(A2 * cx + B2 * cy);
    const int b0 = (A0 > 0 || (A0 == 0 && B0 < 0)) ? 0 : 1;
    const int b1 = (A1 > 0 || (A1 == 0 && B1 < 0)) ? 0 : 1;
    const int b2 = (A2 > 0 || (A2 == 0 && B2 < 0)) ? 0 : 1;
    const int minx = min(ax, min(bx, cx)), maxx = max(ax, max(bx, cx));
    const int miny = min(ay, min(by, cy)), maxy = max(ay, max(by, cy));
    // sample offsets whose position 256 m + 128 lies inside the bounding box
    // (>> on a signed int is a floor division by 256)
    const int m0 = max(mlo, -((128 - minx) >> 8)), m1 = min(mlo + F - 1, (maxx - 128) >> 8);
    const int n0 = max(mlo, -((128 - miny) >> 8)), n1 = min(mlo + F - 1, (maxy - 128) >> 8);
    for (int n = n0; n <= n1; n++) {
        int py = 256 * n + 128;
        int e0 = B0 * py + C0, e1 = B1 * py + C1, e2 = B2 * py + C2;
        uint32_t bits = 0;
        for (int m = m0; m <= m1; m++) {
            int px = 256 * m + 128;
            if (A0 * px + e0 >= b0 && A1 * px + e1 >= b1 && A2 * px + e2 >= b2) bits |= 1u << (m - mlo);
        }
        if (bits) rows[(n - mlo) * rstride] |= bits;
    }
}

// Per-scale table: for each hull pattern, HF row words over the hull window.
__global__ void k_build_scale_masks(int s, uint32_t* lut)
{
    int pat = blockIdx.x * blockDim.x + threadIdx.x;
    if (pat >= 4096) return;
    MaskGeom g = mask_geom(s);
    Poly c;
    hull_from_lut(g_hull_lut[pat], c);
    uint64_t te = g_tri_lut[pat];
    uint32_t rows[32];
    for (int r = 0; r < g.HF; r++) rows[r] = 0;
    const int u = 4 * s;
    for (int t = 0; t < c.n - 2; t++) {
        int a = (int)((te >> (9 * t)) & 7), b = (int)((te >> (9 * t + 3)) & 7), d = (int)((te >> (9 * t + 6)) & 7);
        tri_mask(c.x[a] * u, c.y[a] * u, c.x[b] * u, c.y[b] * u, c.x[d] * u, c.y[d] * u, g.hlo, g.HF, rows);
    }
    for (int r = 0; r < g.HF; r++) lut[(size_t)pat * g.HF + r] = rows[r];
}

cudaError_t build_scale_masks(int s, uint32_t* lut, cudaStream_t st)
{
    k_build_scale_masks<<<16, 256, 0, st>>>(s, lut);
    return cudaGetLastError();
}

// set when a bounded wait for a TMA tile load gave up (the block then left
// its tile unwritten); read and cleared by depix_take_device_faults
__device__ int g_raster_fault;

// slots of a tile's table of distinct cut polygons (bounded probing: a
// polygon that finds no slot makes its own mask)
constexpr int kPolyTable = 1024, kPolyProbes = 16;

template <int TW, int TH>
struct MaskTile {
    static constexpr int GW = TW + 2, GH = TH + 2, GN = GW * GH; // cells with their ring
    static constexpr int BW = TW + 6, BH = TH + 6;               // graph, halo 3
    static constexpr int CW = TW + 4, CH = TH + 4;               // pixels, halo 2
    // pixels with halo 2, stored from two columns further left (x0 - 4) so
    // that a TMA box can start on a 16-byte boundary: pixel (lx, ly) of the
    // halo-2 window is pix[ly][lx + 2]
    __align__(128) uint32_t pix[CH][CW + 4];
    uint64_t bar;      // completion of the TMA pixel load
    int tma_ok;
    // graph bytes with halo 3, stored from 13 columns further left (x0 - 16)
    // so that a TMA box starts on a 16-byte boundary: graph byte (bx, by) of
    // the halo-3 window is graph[by][bx + kGOff]
    static constexpr int kGOff = 13, GRW = TW + 32;
    __align__(128) uint8_t graph[BH][GRW];
    uint8_t spill[GN]; // bit e: the polygon reaches into the open square of neighbour e
    uint8_t live[GN];  // the cell exists (inside the image)
    uint16_t list[GN]; // subdivided cells of the tile, then the blocks that need owner resolution
    uint16_t rep[GN];  // per subdivided cell: the list entry whose key, then whose polygon, it shares
    uint16_t reps[GN]; // list entries that build a polygon (one per distinct key)
    // distinct keys (first half), then distinct polygons (second half): hash
    // tag | (list entry + 1), 0 empty; the first half later holds the list
    // entries that make a mask
    unsigned long long table[kPolyTable];
    int count;
    int slow;          // blocks in list for the owner-resolution pass
    int nreps;
    int nmakers;
};

__device__ __forceinline__ uint32_t rgba_of(uint32_t p)
{
    return ((p >> 16) & 0xFFu) | (p & 0xFF00u) | ((p & 0xFFu) << 16) | 0xFF000000u;
}

// bit e set when the box [x0,x1]x[y0,y1] (1/64 units) overlaps the open unit
// square of neighbour e
__device__ __forceinline__ unsigned spill_bits(int x0, int y0, int x1, int y1)
{
    unsigned m = 0;
#pragma unroll
    for (int e = 0; e < 8; e++) {
        int sx = kUnit * dir_di(e), sy = kUnit * dir_dj(e);
        if (x1 > sx && x0 < sx + kUnit && y1 > sy && y0 < sy + kUnit) m |= 1u << e;
    }
    return m;
}

// One corner-cutting round (subdivision, subdivision_functions.cu:564-669)
// read off the per-pattern tables: each hull vertex's case, its own Q and R
// points and, on a linked/border transition, the linked neighbour's R (or Q)
// around the vertex matching this one (getPointIndex falls back to vertex 0).
// NbPattern(L) is the pattern of the neighbour in direction L; TJ(px, py) the
// corner test of a vertex between two border edges; Emit(t, x, y) receives
// cut vertex t. Returns the vertex count.
template <typename NbPattern, typename TJ, typename Emit>
__device__ __forceinline__ int subdivide_tables(int pat, uint64_t e, NbPattern nb_pattern, TJ tj, Emit emit)
{
    const int n = (int)(e & 0xF);
    const uint64_t vk = __ldg(&g_vk_lut[pat]);
    const uint32_t* qrs = g_qr_lut + pat * 8;
    int m = 0;
    for (int v = 0; v < n; v++) {
        const int code = (int)((vk >> (5 * v)) & 31u), kind = code & 3;
        const int px = hx(e, v), py = hy(e, v);
        const uint32_t qr = __ldg(qrs + v);
        const int qx = (int8_t)(qr & 0xFF), qy = (int8_t)((qr >> 8) & 0xFF);
        const int rx = (int8_t)((qr >> 16) & 0xFF), ry = (int8_t)(qr >> 24);
        if (kind == 0 || (kind == 1 && tj(px, py))) {
            emit(m++, px, py);
        } else if (kind == 1) {
            emit(m++, rx, ry);
            emit(m++, qx, qy);
        } else {
            const int L = code >> 2, ddx = dir_di(L), ddy = dir_dj(L);
            const int np = nb_pattern(L);
            const uint64_t ne = __ldg(&g_hull_lut[np]);
            const int nn = (int)(ne & 0xF);
            // index of the neighbour hull vertex at this vertex's position
            // (quarter units in the neighbour's frame), else 0
            const int tqx = (px - kUnit * ddx) / (kUnit / 4) + 1, tqy = (py - kUnit * ddy) / (kUnit / 4) + 1;
            int op = 0;
            if (tqx >= 0 && tqx < 8 && tqy >= 0 && tqy < 8) {
                const uint64_t key = (uint64_t)(tqx | (tqy << 3)) * 0x041041041041ull;
                const uint64_t x = ((ne >> 4) & 0xFFFFFFFFFFFFull) ^ key;
                uint64_t zero = (x - 0x041041041041ull) & ~x & 0x820820820820ull;
                zero &= (1ull << (6 * nn)) - 1ull; // only the hull's own vertices
                if (zero) op = (__ffsll((long long)zero) - 1) / 6;
            }
            const uint32_t nq = __ldg(&g_qr_lut[np * 8 + op]);
            int ax, ay;
            if (kind == 2) { // previous edge linked: the neighbour's R
                ax = (int8_t)((nq >> 16) & 0xFF);
                ay = (int8_t)(nq >> 24);
            } else { // current edge linked: the neighbour's Q
                ax = (int8_t)(nq & 0xFF);
                ay = (int8_t)((nq >> 8) & 0xFF);
            }
            ax += kUnit * ddx;
            ay += kUnit * ddy;
            if (kind == 2) {
                emit(m++, (qx + ax) / 2, (qy + ay) / 2);
                emit(m++, qx, qy);
            } else {
                emit(m++, rx, ry);
                emit(m++, (rx + ax) / 2, (ry + ay) / 2);
            }
        }
    }
    return m;
}

// Coverage of a polygon that is not star-shaped around its cell centre: the
// reference's own ear clip, triangle by triangle. Returns the ear count.
__device__ __noinline__ int ear_clip_mask(const Packed& P, int u, int mlo, int F, uint32_t* rows, int rstride)
{
    bool ok;
    return ear_clip_packed(
        P,
        [&](int ax, int ay, int bx, int by, int cx, int cy) {
            tri_mask(ax * u, ay * u, bx * u, by * u, cx * u, cy * u, mlo, F, rows, rstride);
        },
        ok);
}

// Footprint mask rows (F words at rows[r * rstride]) and spill bits of one
// subdivided cell. G(dx, dy) is the graph byte of the cell at that offset
// (0 outside the image, bits toward outside cleared); TJ(px, py) the corner
// test.
// The cut polygon of a subdivided cell (G(dx, dy): graph byte of the cell at
// that offset, 0 outside the image, bits toward outside cleared; TJ(px, py):
// the corner test).
template <typename GraphAt, typename TJ, typename Emit>
__device__ __forceinline__ int cell_polygon_emit(GraphAt G, TJ tj, Emit emit)
{
    const unsigned node = G(0, 0);
    const int pat = cell_pattern(node, G(-1, 0), G(1, 0));
    const uint64_t e = __ldg(&g_hull_lut[pat]);
    auto nb_pattern = [&](int L) -> int {
        const int dx = dir_di(L), dy = dir_dj(L);
        return cell_pattern(G(dx, dy), G(dx - 1, dy), G(dx + 1, dy));
    };
    return subdivide_tables(pat, e, nb_pattern, tj, emit);
}

// The cut polygon in registers.
template <typename GraphAt, typename TJ>
__device__ __forceinline__ void cell_polygon(GraphAt G, TJ tj, Packed& sp)
{
    sp.x0 = sp.x1 = sp.y0 = sp.y1 = 0;
    sp.n = cell_polygon_emit(G, tj, [&](int t, int x, int y) { pk_put(sp, t, x, y); });
}

// The cut polygon written straight into 9 parked words (rows[0..3] the x
// bytes, rows[4..7] the y bytes, rows[8] the count: park_polygon's layout),
// one byte store per coordinate.
template <typename GraphAt, typename TJ>
__device__ __forceinline__ void cell_polygon_parked(GraphAt G, TJ tj, uint32_t* rows)
{
#pragma unroll
    for (int r = 0; r < 8; r++) rows[r] = 0u;
    uint8_t* xb = reinterpret_cast<uint8_t*>(rows);
    uint8_t* yb = xb + 16;
    rows[8] = (uint32_t)cell_polygon_emit(G, tj, [&](int t, int x, int y) {
        xb[t] = (uint8_t)x;
        yb[t] = (uint8_t)y;
    });
}

// Coverage rows of a cut polygon and its spill bits (0 when the ear clip
// gives up, as the reference then draws nothing for the cell).
__device__ __forceinline__ unsigned polygon_mask(const Packed& sp, const MaskGeom& Gm, uint32_t* rows, int rstride)
{
    for (int r = 0; r < Gm.F; r++) rows[r * rstride] = 0;
    const int u = 4 * Gm.s;
    int mnx, mny, mxx, mxy;
    // a star-shaped polygon is simple: the reference's ear clip would tile it
    // exactly, so its crossing-number mask is the coverage
    if (!star_crossing_mask(sp, u, Gm.mlo, Gm.F, rows, rstride, mnx, mny, mxx, mxy)) {
        for (int r = 0; r < Gm.F; r++) rows[r * rstride] = 0;
        if (ear_clip_mask(sp, u, Gm.mlo, Gm.F, rows, rstride) == 0) return 0;
    }
    return spill_bits(mnx, mny, mxx, mxy);
}

// A cut polygon parked in its own cell's mask rows until the mask is made
// (rows[0..3] the x bytes, rows[4..7] the y bytes, rows[8] the count, as
// cell_polygon_parked writes it), and a 64-bit mix of it for the tile's table
// of distinct polygons.
__device__ __forceinline__ void unpark_polygon(const uint32_t* rows, Packed& sp)
{
    sp.x0 = rows[0] | (uint64_t)rows[1] << 32;
    sp.x1 = rows[2] | (uint64_t)rows[3] << 32;
    sp.y0 = rows[4] | (uint64_t)rows[5] << 32;
    sp.y1 = rows[6] | (uint64_t)rows[7] << 32;
    sp.n = (int)rows[8];
}

__device__ __forceinline__ uint64_t polygon_hash(const Packed& sp)
{
    uint64_t h = sp.x0 ^ (sp.x1 * 0x9E3779B97F4A7C15ull) ^ ((sp.y0 << 1 | sp.y0 >> 63) * 0xC2B2AE3D27D4EB4Full) ^
                 ((sp.y1 << 7 | sp.y1 >> 57) * 0x165667B19E3779F9ull) ^ (uint64_t)sp.n;
    h ^= h >> 33;
    h *= 0xFF51AFD7ED558CCDull;
    h ^= h >> 33;
    h *= 0xC4CEB9FE1A85EC53ull;
    h ^= h >> 33;
    return h;
}

template <int LAYOUT, int S, int TW, int TH, bool TMA = false>
__device__ void mask_raster_tile(MaskTile<TW, TH>& M, uint32_t* masks, const uint8_t* img, int ws, const uint8_t* g,
                                 uint8_t* out, int w, int h, int scale, bool subdivide, const uint32_t* lut, int x0,
                                 int y0, const CUtensorMap* pix_map = nullptr, int frame = 0,
                                 const CUtensorMap* graph_map = nullptr)
{
    using T = MaskTile<TW, TH>;
    const int s = S > 0 ? S : scale;
    const MaskGeom G = mask_geom(s);
    const int F = G.F;
    // ---- phase A
    if constexpr (TMA) {
        // the pixel window (x0 - 4 .. x0 + TW + 4) x (y0 - 2 .. y0 + TH + 2)
        // and, with a graph map, the graph window (x0 - 16 .. x0 + TW + 16) x
        // (y0 - 3 .. y0 + TH + 3) by TMA tile loads on one barrier
        if (threadIdx.x == 0) {
            mbar_init(&M.bar, 1);
            mbar_expect_tx(&M.bar, (uint32_t)(sizeof(M.pix) + (graph_map ? sizeof(M.graph) : 0)));
            tma_load_3d(&M.pix[0][0], pix_map, x0 - 4, y0 - 2, frame, &M.bar);
            if (graph_map) tma_load_3d(&M.graph[0][0], graph_map, x0 - T::kGOff - 3, y0 - 3, frame, &M.bar);
        }
    }
    if (threadIdx.x == 0) {
        M.count = 0;
        M.slow = 0;
        M.nreps = 0;
        M.nmakers = 0;
    }
    for (int k = threadIdx.x; k < kPolyTable; k += blockDim.x) M.table[k] = 0ull;
    if (!(TMA && graph_map)) {
        for (int k = threadIdx.x; k < T::BW * T::BH; k += blockDim.x) {
            int gx = x0 - 3 + k % T::BW, gy = y0 - 3 + k / T::BW;
            unsigned v = 0;
            if (gx >= 0 && gy >= 0 && gx < w && gy < h) v = __ldg(g + (size_t)gy * w + gx) & inside_mask(gx, gy, w, h);
            M.graph[k / T::BW][k % T::BW + T::kGOff] = (uint8_t)v;
        }
    }
    if constexpr (TMA) {
        // the box holds RGBA words; the tile works on the reference's byte
        // order (b0, b1, b2) = (B, G, R), as load_bgr gives it
        if (threadIdx.x == 0) {
            M.tma_ok = tma_wait_or_flag(&M.bar, &g_raster_fault) ? 1 : 0;
        }
        __syncthreads();
        if (!M.tma_ok) return;
        for (int k = threadIdx.x; k < T::CH * (T::CW + 4); k += blockDim.x) {
            uint32_t& v = M.pix[k / (T::CW + 4)][k % (T::CW + 4)];
            v = ((v >> 16) & 0xFFu) | (v & 0xFF00u) | ((v & 0xFFu) << 16);
        }
        // graph bytes on the image's edge lose their bits toward outside (the
        // box reads zero beyond the image); only tiles that reach an edge
        if (graph_map && (x0 < 3 || y0 < 3 || x0 + TW + 3 > w || y0 + TH + 3 > h)) {
            for (int k = threadIdx.x; k < T::BW * T::BH; k += blockDim.x) {
                const int gx = x0 - 3 + k % T::BW, gy = y0 - 3 + k / T::BW;
                if (gx >= 0 && gy >= 0 && gx < w && gy < h)
                    M.graph[k / T::BW][k % T::BW + T::kGOff] &= (uint8_t)inside_mask(gx, gy, w, h);
            }
        }
    } else {
        for (int k = threadIdx.x; k < T::CW * T::CH; k += blockDim.x) {
            int gx = x0 - 2 + k % T::CW, gy = y0 - 2 + k / T::CW;
            uint32_t v = 0;
            if (gx >= 0 && gy >= 0 && gx < w && gy < h) v = load_bgr(img, ws, LAYOUT, gx, gy);
            M.pix[k / T::CW][k % T::CW + 2] = v;
        }
    }
    __syncthreads();

    // ---- phase B: plain cells from the table, subdivided cells to the list
    for (int k = threadIdx.x; k < T::GN; k += blockDim.x) {
        int lx = k % T::GW, ly = k / T::GW;
        int ci = x0 - 1 + lx, cj = y0 - 1 + ly;
        uint32_t* rows = masks + (size_t)k * F;
        bool live = ci >= 0 && cj >= 0 && ci < w && cj < h;
        M.live[k] = live;
        M.spill[k] = 0;
        if (!live) {
            for (int r = 0; r < F; r++) rows[r] = 0;
            continue;
        }
        const int bx = lx + 2, by = ly + 2;
        unsigned node = M.graph[by][bx + T::kGOff];
        if (subdivide && node != 90) {
            int slot = atomicAdd(&M.count, 1);
            M.list[slot] = (uint16_t)k;
            continue;
        }
        int pat = cell_pattern(node, M.graph[by][bx - 1 + T::kGOff], M.graph[by][bx + 1 + T::kGOff]);
        const int dr = G.hlo - G.mlo; // hull window row/column offset inside the footprint
        const uint32_t* src = lut + (size_t)pat * G.HF;
        for (int r = 0; r < F; r++) {
            int q = r - dr;
            rows[r] = (q >= 0 && q < G.HF) ? (__ldg(src + q) << dr) : 0u;
        }
        M.spill[k] = __ldg(&g_spill_lut[pat]);
    }
    __syncthreads();

    // ---- phase B2: subdivided cells
    // A cut polygon is a function of the 5x3 graph bytes around its cell and
    // of the corner tests (tj) at the four cell corners, and its mask is a
    // function of the polygon. So (B2a) each cell keys itself by those inputs
    // and one cell per distinct key builds the polygon (B2b), one builder per
    // distinct polygon makes the mask (B2c), and the others copy (B2d). Cells
    // whose corner test goes through the reference's bounds test or linear
    // addressing (image edges) build on their own.
    const int nlist = M.count;
    auto cell_at = [&](int k, int& lx, int& ly, int& ci, int& cj, bool& border) {
        lx = k % T::GW;
        ly = k / T::GW;
        ci = x0 - 1 + lx;
        cj = y0 - 1 + ly;
        const long long st = LAYOUT == DEPIX_LAYOUT_BGR ? ws : ((3 * w + 3) & ~3);
        const long long index = (long long)cj * st + (long long)ci * 3;
        border = (index - st - 1) < 0 || (index + w + 1) > ((long long)h * st - 1) || ci == 0 || ci == w - 1 ||
                 cj >= h - 1;
    };
    // corner test at vertex (px, py) of the cell at tile position (lx, ly)
    auto tj_of = [&](int lx, int ly, int ci, int cj, bool border, int px, int py) -> bool {
        if (border) {
            const long long st = LAYOUT == DEPIX_LAYOUT_BGR ? ws : ((3 * w + 3) & ~3);
            const long long index = (long long)cj * st + (long long)ci * 3;
            if ((index - st - 1) < 0 || (index + w + 1) > ((long long)h * st - 1)) return true;
            return t_junction_global(img, w, h, ws, LAYOUT, ci, cj, px, py);
        }
        const int qx = lx + 1, qy = ly + 1;
        auto C = [&](int dx, int dy) { return M.pix[qy + dy][qx + dx + 2]; };
        if (px == 0 && py == 0) return C(-1, 0) != C(-1, -1) || C(-1, -1) != C(0, -1);
        if (px == kUnit && py == 0) return C(1, 0) != C(1, -1) || C(1, -1) != C(0, -1);
        if (px == kUnit && py == kUnit) return C(0, 1) != C(1, 1) || C(1, 1) != C(1, 0);
        if (px == 0 && py == kUnit) return C(-1, 1) != C(0, 1) || C(0, 1) != C(-1, 0);
        return false;
    };
    // insert-or-find in one half of the table: the list entry whose parked
    // words equal this entry's (same(rq)), or q when q took a free slot or
    // the probes ran out
    auto dedupe = [&](uint64_t hs, int half, int q, auto same) -> int {
        const unsigned long long tag = hs & ~0xFFFFull;
        constexpr int kHalf = kPolyTable / 2;
        int slot = (int)(hs >> 16) & (kHalf - 1);
        for (int probe = 0; probe < kPolyProbes; probe++, slot = (slot + 1) & (kHalf - 1)) {
            unsigned long long* e = &M.table[half * kHalf + slot];
            unsigned long long cur = *e;
            if (cur == 0ull) {
                cur = atomicCAS(e, 0ull, tag | (unsigned long long)(q + 1));
                if (cur == 0ull) return q;
            }
            if ((cur & ~0xFFFFull) == tag) {
                const int rq = (int)(cur & 0xFFFFull) - 1;
                if (same(rq)) return rq;
            }
        }
        return q;
    };
    // B2a
    for (int q = threadIdx.x; q < nlist; q += blockDim.x) {
        const int k = M.list[q];
        int lx, ly, ci, cj;
        bool border;
        cell_at(k, lx, ly, ci, cj, border);
        const int bx = lx + 2, by = ly + 2;
        uint32_t* rows = masks + (size_t)k * F;
        if (F < 10) { // no room to park keys or polygons: every cell makes its mask
            auto Gs = [&](int dx, int dy) -> unsigned { return M.graph[by + dy][bx + dx + T::kGOff]; };
            auto tj = [&](int px, int py) -> bool { return tj_of(lx, ly, ci, cj, border, px, py); };
            Packed sp;
            cell_polygon(Gs, tj, sp);
            M.spill[k] = (uint8_t)polygon_mask(sp, G, rows, 1);
            continue;
        }
        int rep = q;
        if (!border) {
            auto B = [&](int dx, int dy) -> uint32_t { return M.graph[by + dy][bx + dx + T::kGOff]; };
            const uint32_t corners = (uint32_t)tj_of(lx, ly, ci, cj, false, 0, 0) |
                                     (uint32_t)tj_of(lx, ly, ci, cj, false, kUnit, 0) << 1 |
                                     (uint32_t)tj_of(lx, ly, ci, cj, false, kUnit, kUnit) << 2 |
                                     (uint32_t)tj_of(lx, ly, ci, cj, false, 0, kUnit) << 3;
            const uint32_t w0 = B(-2, -1) | B(-1, -1) << 8 | B(0, -1) << 16 | B(1, -1) << 24;
            const uint32_t w1 = B(2, -1) | B(-2, 0) << 8 | B(-1, 0) << 16 | B(0, 0) << 24;
            const uint32_t w2 = B(1, 0) | B(2, 0) << 8 | B(-2, 1) << 16 | B(-1, 1) << 24;
            const uint32_t w3 = B(0, 1) | B(1, 1) << 8 | B(2, 1) << 16 | corners << 24;
            rows[0] = w0;
            rows[1] = w1;
            rows[2] = w2;
            rows[3] = w3;
            __threadfence_block();
            Packed kp;
            kp.x0 = w0 | (uint64_t)w1 << 32;
            kp.x1 = w2 | (uint64_t)w3 << 32;
            kp.y0 = kp.y1 = 0;
            kp.n = 0;
            rep = dedupe(polygon_hash(kp), 0, q, [&](int rq) {
                const uint32_t* o = masks + (size_t)M.list[rq] * F;
                return o[0] == w0 && o[1] == w1 && o[2] == w2 && o[3] == w3;
            });
        }
        M.rep[q] = (uint16_t)rep;
        if (rep == q) M.reps[atomicAdd(&M.nreps, 1)] = (uint16_t)q;
    }
    __syncthreads();
    if (F >= 10) {
        // B2b: one polygon per distinct key, parked in its cell's rows; the
        // builder's rep becomes the builder whose polygon (and mask) it shares
        const int nb = M.nreps;
        uint16_t* makers = reinterpret_cast<uint16_t*>(M.table); // the key half, free now
        for (int i = threadIdx.x; i < nb; i += blockDim.x) {
            const int q = M.reps[i], k = M.list[q];
            int lx, ly, ci, cj;
            bool border;
            cell_at(k, lx, ly, ci, cj, border);
            const int bx = lx + 2, by = ly + 2;
            auto Gs = [&](int dx, int dy) -> unsigned { return M.graph[by + dy][bx + dx + T::kGOff]; };
            auto tj = [&](int px, int py) -> bool { return tj_of(lx, ly, ci, cj, border, px, py); };
            cell_polygon_parked(Gs, tj, masks + (size_t)k * F);
            Packed sp;
            unpark_polygon(masks + (size_t)k * F, sp);
            __threadfence_block();
            const int rp = dedupe(polygon_hash(sp), 1, q, [&](int rq) {
                Packed o;
                unpark_polygon(masks + (size_t)M.list[rq] * F, o);
                return o.n == sp.n && o.x0 == sp.x0 && o.x1 == sp.x1 && o.y0 == sp.y0 && o.y1 == sp.y1;
            });
            M.rep[q] = (uint16_t)rp;
            if (rp == q) makers[atomicAdd(&M.nmakers, 1)] = (uint16_t)q;
        }
        __syncthreads();
        // B2c: the masks
        const int nm = M.nmakers;
        for (int i = threadIdx.x; i < nm; i += blockDim.x) {
            const int k = M.list[makers[i]];
            uint32_t* rows = masks + (size_t)k * F;
            Packed sp;
            unpark_polygon(rows, sp);
            M.spill[k] = (uint8_t)polygon_mask(sp, G, rows, 1);
        }
        __syncthreads();
        // B2d: copies (key rep -> its polygon's mask maker)
        for (int q = threadIdx.x; q < nlist; q += blockDim.x) {
            const int rq = M.rep[M.rep[q]];
            if (rq == q) continue;
            const int k = M.list[q], rk = M.list[rq];
            const uint32_t* src = masks + (size_t)rk * F;
            uint32_t* dst = masks + (size_t)k * F;
            for (int r = 0; r < F; r++) dst[r] = src[r];
            M.spill[k] = M.spill[rk];
        }
        __syncthreads();
    }

    // ---- phase C: one output block per tile cell
    const int ow = w * s;
    const bool vec = ((S == 4 || S == 8) && (ow % 4) == 0 && ((reinterpret_cast<uintptr_t>(out) & 15) == 0));
    const uint32_t blockbits = (s >= 32) ? 0xFFFFFFFFu : ((1u << s) - 1u);
    for (int q = threadIdx.x; q < TW * TH; q += blockDim.x) {
        int tx = q % TW, ty = q / TW;
        int ci = x0 + tx, cj = y0 + ty;
        if (ci >= w || cj >= h) continue;
        const int k0 = (ty + 1) * T::GW + (tx + 1);
        unsigned intr = 0;
#pragma unroll
        for (int e = 0; e < 8; e++) {
            int kn = k0 + dir_dj(e) * T::GW + dir_di(e);
            intr |= (unsigned)bitof(M.spill[kn], 7 - e);
        }
        const uint32_t* own = masks + (size_t)k0 * F;
        bool full = true;
        for (int r = 0; r < s; r++) full &= ((own[r - G.mlo] >> (-G.mlo)) & blockbits) == blockbits;
        if (!full || intr) {
            // owner resolution after the barrier, over a compacted list, so
            // that warps do not run it beside blocks that need none
            M.list[atomicAdd(&M.slow, 1)] = (uint16_t)q;
            continue;
        }
        const uint32_t own_col = rgba_of(M.pix[ty + 2][tx + 4]);
        uint8_t* orow = out + ((size_t)cj * s * ow + (size_t)ci * s) * 4;
        for (int r = 0; r < s; r++) {
            uint32_t* o = reinterpret_cast<uint32_t*>(orow + (size_t)r * ow * 4);
            if (vec) {
                for (int c4 = 0; c4 < s; c4 += 4)
                    __stcs(reinterpret_cast<uint4*>(o + c4), make_uint4(own_col, own_col, own_col, own_col));
            } else {
                for (int c = 0; c < s; c++) o[c] = own_col;
            }
        }
    }
    __syncthreads();
    const int nslow = M.slow;
    for (int qs = threadIdx.x; qs < nslow; qs += blockDim.x) {
        const int q = M.list[qs];
        const int tx = q % TW, ty = q / TW;
        const int ci = x0 + tx, cj = y0 + ty;
        const int k0 = (ty + 1) * T::GW + (tx + 1);
        uint8_t* orow = out + ((size_t)cj * s * ow + (size_t)ci * s) * 4;
        // the nine candidates' colours, in priority order
        uint32_t cand_col[9];
#pragma unroll
        for (int z = 0; z < 9; z++) cand_col[z] = rgba_of(M.pix[ty + 2 + 1 - z / 3][tx + 4 + 1 - z % 3]);
        for (int r = 0; r < s; r++) {
            // per candidate (priority order q = 0..8: rows above first, then
            // right to left) the samples of this row it covers and no
            // earlier candidate does; candidates are one cell apart so the
            // nine masks are disjoint and each sample has at most one owner
            uint32_t claimed = 0;
            uint32_t take[9];
            int qq = 0;
#pragma unroll
            for (int dj = 1; dj >= -1; dj--) {
                const int rr = r - s * dj - G.mlo;
#pragma unroll
                for (int di = 1; di >= -1; di--, qq++) {
                    take[qq] = 0;
                    if (rr < 0 || rr >= F) continue;
                    const int kn = k0 + dj * T::GW + di; // cells outside the image have zero rows
                    const uint64_t wbits = masks[(size_t)kn * F + rr];
                    const int sh = s * di + G.mlo; // block column c = footprint column + sh
                    const uint32_t bits =
                        (uint32_t)((sh >= 0 ? (wbits << sh) : (wbits >> (-sh))) & blockbits) & ~claimed;
                    claimed |= bits;
                    take[qq] = bits;
                }
            }
            uint32_t* o = reinterpret_cast<uint32_t*>(orow + (size_t)r * ow * 4);
            auto owner_colour = [&](int c) -> uint32_t {
                uint32_t col = 0xFF000000u; // no owner: the clear colour
#pragma unroll
                for (int q = 0; q < 9; q++)
                    if ((take[q] >> c) & 1u) col = cand_col[q];
                return col;
            };
            if (vec) {
#pragma unroll
                for (int c4 = 0; c4 < (S > 0 ? S : 16); c4 += 4)
                    if (c4 < s)
                        __stcs(reinterpret_cast<uint4*>(o + c4), make_uint4(owner_colour(c4), owner_colour(c4 + 1),
                                                                            owner_colour(c4 + 2), owner_colour(c4 + 3)));
            } else {
                for (int c = 0; c < s; c++) o[c] = owner_colour(c);
            }
        }
    }
}

template <int LAYOUT, int S, int TH>
__global__ void __launch_bounds__(256) k_mask_raster(RasterBatch b, const uint32_t* lut)
{
    __shared__ MaskTile<32, TH> M;
    extern __shared__ uint32_t masks[];
    size_t z = blockIdx.z;
    mask_raster_tile<LAYOUT, S, 32, TH>(M, masks, b.img + b.img_stride * z, b.ws, b.graph + b.graph_stride * z,
                                        b.out + b.out_stride * z, b.w, b.h, b.scale, b.subdivide != 0, lut,
                                        blockIdx.x * 32, blockIdx.y * TH);
}

// The equal-size batch raster with its pixel windows loaded by TMA (RGBA
// frames whose base, rows and frame stride are 16-byte aligned).
template <int S, int TH>
__global__ void __launch_bounds__(256, 3) k_mask_raster_tma(RasterBatch b, const uint32_t* lut,
                                                         const __grid_constant__ CUtensorMap pix_map,
                                                         const __grid_constant__ CUtensorMap graph_map, int with_graph)
{
    __shared__ MaskTile<32, TH> M;
    extern __shared__ uint32_t masks[];
    size_t z = blockIdx.z;
    mask_raster_tile<DEPIX_LAYOUT_RGBA, S, 32, TH, true>(M, masks, b.img + b.img_stride * z, b.ws,
                                                         b.graph + b.graph_stride * z, b.out + b.out_stride * z, b.w,
                                                         b.h, b.scale, b.subdivide != 0, lut, blockIdx.x * 32,
                                                         blockIdx.y * TH, &pix_map, (int)z,
                                                         with_graph ? &graph_map : nullptr);
}

bool rgba_tensor_map(const uint8_t* img, int w, int h, int ws, size_t frame_stride, int nframes, int box_w, int box_h,
                     CUtensorMap* map);

using TensorMapEncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                          const cuuint64_t*, const cuuint32_t*, const cuuint32_t*,
                                          CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                          CUtensorMapFloatOOBfill);

static TensorMapEncodeTiled tensor_map_encoder();

// A tensor map of RGBA frames as words, (w, h, frames), box (box_w, box_h, 1).
// False when the frames do not meet TMA's rules (16-byte aligned base, row
// and frame strides) or no encoder is available.
bool rgba_tensor_map(const uint8_t* img, int w, int h, int ws, size_t frame_stride, int nframes, int box_w, int box_h,
                     CUtensorMap* map)
{
    if ((reinterpret_cast<uintptr_t>(img) & 15) || (ws & 15) || w < 1 || h < 1) return false;
    const uint64_t fstride = nframes > 1 ? (uint64_t)frame_stride : ((uint64_t)ws * h + 15) & ~15ull;
    if (fstride & 15) return false;
    const TensorMapEncodeTiled enc = tensor_map_encoder();
    if (!enc) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)nframes};
    const cuuint64_t strides[2] = {(cuuint64_t)ws, (cuuint64_t)fstride};
    const cuuint32_t box[3] = {(cuuint32_t)box_w, (cuuint32_t)box_h, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, const_cast<uint8_t*>(img), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// A tensor map of 8-bit frames (graph bytes), (w, h, frames), box (box_w,
// box_h, 1); false when the buffers do not meet TMA's rules.
bool u8_tensor_map(const uint8_t* base, int w, int h, size_t frame_stride, int nframes, int box_w, int box_h,
                   CUtensorMap* map)
{
    if ((reinterpret_cast<uintptr_t>(base) & 15) || (w & 15) || w < 1 || h < 1) return false;
    const uint64_t fstride = nframes > 1 ? (uint64_t)frame_stride : ((uint64_t)w * h + 15) & ~15ull;
    if (fstride & 15) return false;
    const TensorMapEncodeTiled enc = tensor_map_encoder();
    if (!enc) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)nframes};
    const cuuint64_t strides[2] = {(cuuint64_t)w, (cuuint64_t)fstride};
    const cuuint32_t box[3] = {(cuuint32_t)box_w, (cuuint32_t)box_h, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 3, const_cast<uint8_t*>(base), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

static TensorMapEncodeTiled tensor_map_encoder()
{
    static TensorMapEncodeTiled fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<TensorMapEncodeTiled>(p);
    }();
    return fn;
}

static bool pixel_tensor_map(const RasterBatch& b, int nframes, int TH, CUtensorMap* map)
{
    if (b.layout != DEPIX_LAYOUT_RGBA) return false;
    return rgba_tensor_map(b.img, b.w, b.h, b.ws, b.img_stride, nframes, 32 + 8, TH + 4, map);
}

template <int LAYOUT, int S, int TH>
static cudaError_t launch_mask_raster_t(const RasterBatch& b, int nframes, const uint32_t* lut, cudaStream_t s)
{
    if constexpr (LAYOUT == DEPIX_LAYOUT_RGBA) {
        CUtensorMap map;
        if (pixel_tensor_map(b, nframes, TH, &map)) {
            MaskGeom g = mask_geom(b.scale);
            size_t smem = (size_t)MaskTile<32, TH>::GN * g.F * sizeof(uint32_t);
            if (smem + sizeof(MaskTile<32, TH>) > 48 * 1024) {
                cudaError_t e = cudaFuncSetAttribute(k_mask_raster_tma<S, TH>,
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                if (e != cudaSuccess) return e;
            }
            // the graph window too, when the graph's width and frame stride allow it
            CUtensorMap gmap;
            const bool with_graph = u8_tensor_map(b.graph, b.w, b.h, b.graph_stride, nframes, 32 + 32, TH + 6, &gmap);
            if (!with_graph) gmap = map; // unused
            dim3 grid((b.w + 32 - 1) / 32, (b.h + TH - 1) / TH, nframes);
            k_mask_raster_tma<S, TH><<<grid, 256, smem, s>>>(b, lut, map, gmap, with_graph ? 1 : 0);
            return cudaGetLastError();
        }
    }
    MaskGeom g = mask_geom(b.scale);
    size_t smem = (size_t)MaskTile<32, TH>::GN * g.F * sizeof(uint32_t);
    if (smem + sizeof(MaskTile<32, TH>) > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_mask_raster<LAYOUT, S, TH>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    dim3 grid((b.w + 32 - 1) / 32, (b.h + TH - 1) / TH, nframes);
    k_mask_raster<LAYOUT, S, TH><<<grid, 256, smem, s>>>(b, lut);
    return cudaGetLastError();
}

// ---- uneven batches: the raster as a persistent kernel over a tile queue

// three blocks per SM: the persistent loop would otherwise hold the kernel at
// 116 registers and two blocks (12 % slower on 4096 sprites at x4)
template <int S, int TW, int TH>
__global__ void __launch_bounds__(256, 3) k_raster_queue(QueueBatch q)
{
    __shared__ MaskTile<TW, TH> M;
    extern __shared__ uint32_t masks[];
    const QueueHeader* H = q.hdr;
    const int n = H->n;
    constexpr int SH = raster_shape_index(TW, TH);
    const int P = q.rbase + SH;
    queue_loop(q.counters + QC_RASTER + SH, (int)H->total[P], q.gran[QS_RASTER], [&](int t) {
        const uint32_t* base = H->base + P * (n + 1);
        const int f = queue_frame(base, n, (uint32_t)t);
        const QueueFrame fr = H->frames[f];
        const int lt = t - (int)base[f], tx = (fr.w + TW - 1) / TW;
        mask_raster_tile<DEPIX_LAYOUT_RGBA, S, TW, TH>(M, masks, H->img + fr.in_off, 4 * fr.w, q.graph_b + fr.px_off,
                                                       H->out + fr.out_off, fr.w, fr.h, q.scale, H->subdivide != 0,
                                                       q.lut, (lt % tx) * TW, (lt / tx) * TH);
    });
}

template <int S, int TW, int TH>
static size_t raster_queue_smem(int scale)
{
    return (size_t)MaskTile<TW, TH>::GN * mask_geom(scale).F * sizeof(uint32_t);
}

template <int S, int TW, int TH>
static cudaError_t queue_raster_t(const QueueBatch& q, int blocks, cudaStream_t s)
{
    // the shared-memory opt-in is made by raster_queue_occupancy, which the
    // host calls on each device before any launch or stream capture
    const size_t smem = raster_queue_smem<S, TW, TH>(q.scale);
    k_raster_queue<S, TW, TH><<<blocks, 256, smem, s>>>(q);
    return cudaGetLastError();
}

template <int S, int TW, int TH>
static int raster_queue_occupancy(int scale)
{
    int nb = 0;
    const size_t smem = raster_queue_smem<S, TW, TH>(scale);
    if (smem + sizeof(MaskTile<TW, TH>) > 48 * 1024 &&
        cudaFuncSetAttribute(k_raster_queue<S, TW, TH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
        return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_raster_queue<S, TW, TH>, 256, smem) != cudaSuccess)
        return 0;
    return nb;
}

// raster tile variants of the queue path: 32x32, 32x16, 16x16 cells
#define DEPIX_RQ_DISPATCH(FN, ...)                                                                      \
    do {                                                                                                \
        const int sc = q.scale == 4 ? 4 : (q.scale == 8 ? 8 : 0);                                       \
        if (q.rtw == 32 && q.rth == 32) {                                                               \
            if (sc == 4) return FN<4, 32, 32>(__VA_ARGS__);                                             \
            if (sc == 8) return FN<8, 32, 32>(__VA_ARGS__);                                             \
            return FN<0, 32, 32>(__VA_ARGS__);                                                          \
        }                                                                                               \
        if (q.rtw == 32) {                                                                              \
            if (sc == 4) return FN<4, 32, 16>(__VA_ARGS__);                                             \
            if (sc == 8) return FN<8, 32, 16>(__VA_ARGS__);                                             \
            return FN<0, 32, 16>(__VA_ARGS__);                                                          \
        }                                                                                               \
        if (sc == 4) return FN<4, 16, 16>(__VA_ARGS__);                                                 \
        if (sc == 8) return FN<8, 16, 16>(__VA_ARGS__);                                                 \
        return FN<0, 16, 16>(__VA_ARGS__);                                                              \
    } while (0)

cudaError_t queue_raster(const QueueBatch& q, int blocks, cudaStream_t s)
{
    DEPIX_RQ_DISPATCH(queue_raster_t, q, blocks, s);
}

int queue_raster_blocks_per_sm(const QueueBatch& q) { DEPIX_RQ_DISPATCH(raster_queue_occupancy, q.scale); }

// 32x32-cell tiles up to scale 4 (more subdivided cells per block to share
// the work), 32x16 above (the footprint masks grow with the scale)
// A single frame fills a fraction of the SMs, so it takes tiles half as high
// at x4 (twice the blocks, each half as long); batches keep the 32-row tiles.
cudaError_t launch_mask_raster(const RasterBatch& b, int nframes, const uint32_t* lut, cudaStream_t s)
{
    if (b.layout == DEPIX_LAYOUT_RGBA) {
        if (b.scale == 4)
            return nframes == 1 ? launch_mask_raster_t<DEPIX_LAYOUT_RGBA, 4, 16>(b, nframes, lut, s)
                                : launch_mask_raster_t<DEPIX_LAYOUT_RGBA, 4, 32>(b, nframes, lut, s);
        if (b.scale == 8) return launch_mask_raster_t<DEPIX_LAYOUT_RGBA, 8, 16>(b, nframes, lut, s);
        if (b.scale < 4) return launch_mask_raster_t<DEPIX_LAYOUT_RGBA, 0, 32>(b, nframes, lut, s);
        return launch_mask_raster_t<DEPIX_LAYOUT_RGBA, 0, 16>(b, nframes, lut, s);
    }
    if (b.scale == 4)
        return nframes == 1 ? launch_mask_raster_t<DEPIX_LAYOUT_BGR, 4, 16>(b, nframes, lut, s)
                            : launch_mask_raster_t<DEPIX_LAYOUT_BGR, 4, 32>(b, nframes, lut, s);
    if (b.scale == 8) return launch_mask_raster_t<DEPIX_LAYOUT_BGR, 8, 16>(b, nframes, lut, s);
    if (b.scale < 4) return launch_mask_raster_t<DEPIX_LAYOUT_BGR, 0, 32>(b, nframes, lut, s);
    return launch_mask_raster_t<DEPIX_LAYOUT_BGR, 0, 16>(b, nframes, lut, s);
}

cudaError_t take_raster_fault(int* out)
{
    int zero = 0;
    cudaError_t e = cudaMemcpyFromSymbol(out, g_raster_fault, sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_raster_fault, &zero, sizeof(int));
    return e;
}

size_t scale_mask_words(int s) { return (size_t)4096 * mask_geom(s).HF; }

}  // namespace depix
