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
}

cudaError_t init_tables(cudaStream_t s)
{
    k_init_tables<<<16, 256, 0, s>>>();
    return cudaGetLastError();
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
        p.x[t] = __float2int_rn(v.x * (float)kUnit);
        p.y[t] = __float2int_rn(v.y * (float)kUnit);
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
            S.vx[k][t] = (int8_t)c.x[t];
            S.vy[k][t] = (int8_t)c.y[t];
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

}  // namespace depix
