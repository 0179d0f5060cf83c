// depix_graph.cu -- similarity graph, crossing resolution and component
// labelling kernels.
//
// Frames are addressed through FrameRef so the same tile functions serve a
// single frame (grid.z = 1) and a batch of equal-size frames (grid.z = frame).
#include "depix_internal.h"

namespace depix {

// ------------------------------------------------------------ graph stage

// Pair bits of one pixel p inside the tile region: similarity with the
// right (bit 0), upper (bit 1), upper-right (bit 2) pixel, and of the pair
// (right, upper) (bit 3), each only when both pixels are in the image.
// set when a bounded wait for a TMA tile load gave up (that tile of the
// graph was left unwritten); read and cleared by depix_take_device_faults
__device__ int g_graph_fault;
__device__ int g_heur_fault; // the same for the heuristics stage
// Test switch (depix_debug_tma_timeout): the TMA graph kernel issues no tile
// load and its wait gives up after kTestPolls polls, with nothing in flight.
__device__ int g_graph_tma_timeout_test;
constexpr int kTestPolls = 16;

constexpr int kGTW = 64;  // graph tile width (pixels)
constexpr int kGTH = 16;  // graph tile height

// the pixel window of a graph tile as one TMA box: RGBA words from x0 - 4
// (16-byte aligned), y0 - 1, (kGTW + 8) x (kGTH + 2)
constexpr int kGBoxW = kGTW + 8, kGBoxH = kGTH + 2;

template <int LAYOUT, bool TMA = false>
__device__ __forceinline__ void graph_tile(const FrameRef f, int x0, int y0, uint32_t thr, bool fuse_trivial,
                                           const CUtensorMap* pix_map = nullptr, int frame = 0)
{
    constexpr int RW = kGTW + 2, RH = kGTH + 2;
    __shared__ uint32_t words[RH][RW];
    __shared__ uint8_t pairs[RH][RW];
    const int w = f.w, h = f.h;
    if constexpr (TMA) {
        __shared__ __align__(128) uint32_t box[kGBoxH][kGBoxW];
        __shared__ uint64_t bar;
        __shared__ int ok;
        if (threadIdx.x == 0) {
            const bool test_timeout = *(volatile int*)&g_graph_tma_timeout_test != 0;
            mbar_init(&bar, 1);
            mbar_expect_tx(&bar, (uint32_t)sizeof(box));
            if (!test_timeout) tma_load_3d(&box[0][0], pix_map, x0 - 4, y0 - 1, frame, &bar);
            ok = tma_wait_or_flag(&bar, &g_graph_fault, test_timeout ? kTestPolls : kTmaPolls) ? 1 : 0;
        }
        __syncthreads();
        if (!ok) return;
        for (int k = threadIdx.x; k < RW * RH; k += blockDim.x) {
            const int rx = k % RW, ry = k / RW;
            const uint32_t p = box[ry][rx + 3]; // window column rx is image column x0 - 1 + rx
            // RGBA -> the reference's byte order (b0, b1, b2) = (B, G, R); zero outside the image
            const uint32_t c = ((p >> 16) & 0xFFu) | (p & 0xFF00u) | ((p & 0xFFu) << 16);
            const int gx = x0 - 1 + rx, gy = y0 - 1 + ry;
            words[ry][rx] = (gx >= 0 && gy >= 0 && gx < w && gy < h) ? word_of_bgr(c, thr) : 0u;
        }
    } else {
        for (int k = threadIdx.x; k < RW * RH; k += blockDim.x) {
            int rx = k % RW, ry = k / RW;
            int gx = x0 - 1 + rx, gy = y0 - 1 + ry;
            uint32_t wd = 0;
            if (gx >= 0 && gy >= 0 && gx < w && gy < h) wd = word_of_bgr(load_bgr(f.img, f.ws, LAYOUT, gx, gy), thr);
            words[ry][rx] = wd;
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < RW * RH; k += blockDim.x) {
        int rx = k % RW, ry = k / RW;
        int gx = x0 - 1 + rx, gy = y0 - 1 + ry;
        unsigned pb = 0;
        bool in = gx >= 0 && gy >= 0 && gx < w && gy < h;
        bool rin = rx + 1 < RW && gx + 1 < w && gx + 1 >= 0 && in;
        bool uin = ry + 1 < RH && gy + 1 < h && gy + 1 >= 0 && in;
        if (rin && similar(words[ry][rx], words[ry][rx + 1], thr)) pb |= 1u;
        if (uin && similar(words[ry][rx], words[ry + 1][rx], thr)) pb |= 2u;
        if (rin && uin) {
            if (similar(words[ry][rx], words[ry + 1][rx + 1], thr)) pb |= 4u;
            if (similar(words[ry][rx + 1], words[ry + 1][rx], thr)) pb |= 8u;
        }
        pairs[ry][rx] = (uint8_t)pb;
    }
    __syncthreads();
    // fused trivial removal (crossCheck_4): a diagonal goes when the 2x2 block
    // it crosses has all four sides similar; each block decided once (bit 4
    // of the pairs byte of its lower-left node)
    if (fuse_trivial) {
        for (int k = threadIdx.x; k < (kGTW + 1) * (kGTH + 1); k += blockDim.x) {
            const int bx = k % (kGTW + 1), by = k / (kGTW + 1);
            const unsigned full = pairs[by][bx] & pairs[by + 1][bx] & (pairs[by][bx] >> 1) & (pairs[by][bx + 1] >> 1) & 1u;
            pairs[by][bx] |= (uint8_t)(full << 4);
        }
        __syncthreads();
    }
    // node bits (graph_Kernel)
    for (int k = threadIdx.x; k < kGTW * kGTH; k += blockDim.x) {
        int tx = k % kGTW, ty = k / kGTW;
        int gx = x0 + tx, gy = y0 + ty;
        if (gx >= w || gy >= h) continue;
        int rx = tx + 1, ry = ty + 1;
        unsigned c = pairs[ry][rx], l = pairs[ry][rx - 1], d = pairs[ry - 1][rx], dl = pairs[ry - 1][rx - 1];
        unsigned node = 0;
        node |= (unsigned)bitof(c, 1) << 1;   // up
        node |= (unsigned)bitof(d, 1) << 6;   // down
        node |= (unsigned)bitof(c, 0) << 4;   // right
        node |= (unsigned)bitof(l, 0) << 3;   // left
        node |= (unsigned)bitof(c, 2) << 2;   // up-right
        node |= (unsigned)bitof(l, 3) << 0;   // up-left: pair (right of l = c, up of l)
        node |= (unsigned)bitof(dl, 2) << 5;  // down-left
        node |= (unsigned)bitof(d, 3) << 7;   // down-right: pair (right of d, up of d = c)
        if (fuse_trivial) {
            // blocks with lower-left (rx, ry), (rx-1, ry), (rx-1, ry-1), (rx, ry-1)
            if (bitof(c, 4)) node &= ~4u;
            if (bitof(l, 4)) node &= ~1u;
            if (bitof(dl, 4)) node &= ~32u;
            if (bitof(d, 4)) node &= ~128u;
        }
        f.graph[(size_t)gy * w + gx] = (uint8_t)node;
    }
}

template <int LAYOUT>
__global__ void __launch_bounds__(256) k_graph(FrameBatch b, uint32_t thr, int fuse_trivial)
{
    FrameRef f = b.frame(blockIdx.z);
    graph_tile<LAYOUT>(f, blockIdx.x * kGTW, blockIdx.y * kGTH, thr, fuse_trivial != 0);
}

// RGBA frames whose base, rows and frame stride are 16-byte aligned: the
// pixel windows come by TMA
__global__ void __launch_bounds__(256) k_graph_tma(FrameBatch b, uint32_t thr, int fuse_trivial,
                                                   const __grid_constant__ CUtensorMap pix_map)
{
    FrameRef f = b.frame(blockIdx.z);
    graph_tile<DEPIX_LAYOUT_RGBA, true>(f, blockIdx.x * kGTW, blockIdx.y * kGTH, thr, fuse_trivial != 0, &pix_map,
                                        (int)blockIdx.z);
}

// Trivial removal on a graph in place (crossCheck_4, graph_functions.cu:1211-1274).
// Only orthogonal bits are read and only diagonal bits written: race-free.
__global__ void k_trivial(uint8_t* g, int w, int h)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= w || j >= h) return;
    auto at = [&](int x, int y) -> unsigned {
        return (x < 0 || y < 0 || x >= w || y >= h) ? 0u : (unsigned)g[(size_t)y * w + x];
    };
    unsigned c = at(i, j), l = at(i - 1, j), r = at(i + 1, j), u = at(i, j + 1), d = at(i, j - 1);
    unsigned ul = at(i - 1, j + 1), ur = at(i + 1, j + 1), dl = at(i - 1, j - 1), dr = at(i + 1, j - 1);
    unsigned out = c;
    if (bitof(l, 1) && bitof(l, 4) && bitof(ul, 6) && bitof(ul, 4) && bitof(c, 3) && bitof(c, 1) && bitof(u, 6) &&
        bitof(u, 3))
        out &= ~1u;
    if (bitof(c, 1) && bitof(c, 4) && bitof(u, 6) && bitof(u, 4) && bitof(r, 3) && bitof(r, 1) && bitof(ur, 6) &&
        bitof(ur, 3))
        out &= ~4u;
    if (bitof(dl, 1) && bitof(dl, 4) && bitof(l, 6) && bitof(l, 4) && bitof(d, 3) && bitof(d, 1) && bitof(c, 6) &&
        bitof(c, 3))
        out &= ~32u;
    if (bitof(d, 1) && bitof(d, 4) && bitof(c, 6) && bitof(c, 4) && bitof(dr, 3) && bitof(dr, 1) && bitof(r, 6) &&
        bitof(r, 3))
        out &= ~128u;
    if (out != c) g[(size_t)j * w + i] = (uint8_t)out;
}

// ------------------------------------------------------- heuristics stage

constexpr int kHTW = 64, kHTH = 16;
constexpr int kHalo = 32; // a curve-length walk moves at most 31 steps from a block node
constexpr int kHRW = kHTW + 2 * kHalo, kHRH = kHTH + 2 * kHalo;

struct SnapTile {
    const uint8_t (*s)[kHRW];
    int ox, oy; // image coordinates of s[0][0]
    __device__ __forceinline__ unsigned at(int x, int y) const { return s[y - oy][x - ox]; }
};

// set bits of node other than bit e; last = the highest such bit in the
// scan order e+1 .. e+7 (mod 8)
__device__ __forceinline__ int others(unsigned node, int e, int& last)
{
    unsigned rest = (node & 0xFFu) & ~(1u << e);
    int s = __popc(rest);
    if (s) {
        // scan order e+1, ..., 7, 0, ..., e-1: the last in that order is the
        // highest set bit below e if any, else the highest set bit overall
        unsigned below = rest & ((1u << e) - 1u);
        last = below ? 31 - __clz(below) : 31 - __clz(rest);
    }
    return s;
}

// curve-length walk (calcVal2PathSize, graph_functions.cu:541-573)
__device__ __forceinline__ void walk_len(const SnapTile& t, int i, int j, int e, int& result)
{
    for (;;) {
        int k_n = 0;
        int s = others(t.at(i, j), e, k_n);
        if (result > 30) return;
        if (s != 1) return;
        result++;
        i += dir_di(k_n);
        j += dir_dj(k_n);
        e = 7 - k_n;
    }
}

// block decision (processHeuristics2, graph_functions.cu:761-849): true
// removes "/" (bits 2/5), false removes "\" (bits 0/7)
__device__ bool block_decision(const SnapTile& t, int i, int j)
{
    unsigned n1 = t.at(i, j), n2 = t.at(i, j + 1), n3 = t.at(i + 1, j), n4 = t.at(i + 1, j + 1);
    int dummy;
    int o1 = others(n1, 2, dummy), o4 = others(n4, 5, dummy), o3 = others(n3, 0, dummy), o2 = others(n2, 7, dummy);
    if (o1 == 1 && o4 == 1) return false;      // curve through "/"
    if (o3 == 1 && o2 == 1) return true;       // curve through "\"
    bool v1 = o1 == 0, v4 = o4 == 0, v3 = o3 == 0, v2 = o2 == 0;
    if ((v1 || v4) && !v3 && !v2) return false; // island
    if (v3 || (v2 && !v1 && !v4)) return true;  // island, reference precedence (graph_functions.cu:805)
    int seg = 0, seg2 = 0;
    walk_len(t, i, j, 2, seg);
    walk_len(t, i + 1, j + 1, 5, seg);
    walk_len(t, i + 1, j, 0, seg2);
    walk_len(t, i, j + 1, 7, seg2);
    return !(seg2 < seg);
}

// Block decision codes: bit 0 a crossing, bit 1 remove "/" (bits 2/5),
// bit 2 remove "\" (bits 0/7).
constexpr unsigned kDecCross = 1, kDecSlash = 2, kDecBack = 4;

// Size of the component of `seed` in an 8x8 window whose bit r*8+c is the
// pixel in window row r, column c; m[e] holds the pixels with edge e. The
// fill follows the edges inside the window only (a move off the window's
// columns is masked, one off its rows shifts out).
__device__ __forceinline__ int window_component(const uint64_t (&m)[8], uint64_t seed)
{
    constexpr uint64_t kCol0 = 0x0101010101010101ull, kCol7 = 0x8080808080808080ull;
    uint64_t c = seed, prev;
    do {
        prev = c;
        c |= ((prev & m[0]) << 7) & ~kCol7; // (-1, +1)
        c |= (prev & m[1]) << 8;            // ( 0, +1)
        c |= ((prev & m[2]) << 9) & ~kCol0; // (+1, +1)
        c |= ((prev & m[3]) >> 1) & ~kCol7; // (-1,  0)
        c |= ((prev & m[4]) << 1) & ~kCol0; // (+1,  0)
        c |= ((prev & m[5]) >> 9) & ~kCol7; // (-1, -1)
        c |= (prev & m[6]) >> 8;            // ( 0, -1)
        c |= ((prev & m[7]) >> 7) & ~kCol0; // (+1, -1)
    } while (c != prev);
    return __popcll(c);
}

// Weighted vote of the three heuristics of Kopf and Lischinski,
// "Depixelizing Pixel Art" (SIGGRAPH 2011), section 3.2, for the block whose
// lower-left node is (i, j); not in the reference, which decides by the
// ordered tests of block_decision. Each heuristic votes for the diagonal to
// keep: curves by the difference of the two curve lengths (the same walks as
// block_decision), sparse pixels by the difference of the sizes of the two
// diagonals' components inside the 8x8 window centred on the block (the
// sparser one is kept), islands with weight 5 for a diagonal whose removal
// would leave one of its ends without edges. The diagonal with fewer votes
// is removed; a tie removes both.
__device__ unsigned vote_decision(const uint8_t (*s)[kHRW], int ox, int oy, int i, int j)
{
    const SnapTile t{s, ox, oy};
    unsigned n1 = t.at(i, j), n2 = t.at(i, j + 1), n3 = t.at(i + 1, j), n4 = t.at(i + 1, j + 1);
    int dummy;
    int o1 = others(n1, 2, dummy), o4 = others(n4, 5, dummy), o3 = others(n3, 0, dummy), o2 = others(n2, 7, dummy);
    int keep_slash = 0, keep_back = 0;
    int seg = 0, seg2 = 0;
    walk_len(t, i, j, 2, seg);
    walk_len(t, i + 1, j + 1, 5, seg);
    walk_len(t, i + 1, j, 0, seg2);
    walk_len(t, i, j + 1, 7, seg2);
    if (seg > seg2) keep_slash += seg - seg2;
    else keep_back += seg2 - seg;
    if (o1 == 0 || o4 == 0) keep_slash += 5;
    if (o3 == 0 || o2 == 0) keep_back += 5;
    // window columns i-3 .. i+4, rows j-3 .. j+4 (inside the snapshot halo)
    uint64_t m[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int r = 0; r < 8; r++) {
        const uint8_t* row = &s[j - 3 + r - oy][i - 3 - ox];
        for (int c = 0; c < 8; c++) {
            const unsigned nd = row[c];
            const uint64_t bit = 1ull << (r * 8 + c);
#pragma unroll
            for (int e = 0; e < 8; e++)
                if (nd >> e & 1u) m[e] |= bit;
        }
    }
    // i1 = (i, j) is window bit 27 (with i4 on "/"), i2 = (i, j + 1) bit 35
    const int size_slash = window_component(m, 1ull << 27), size_back = window_component(m, 1ull << 35);
    if (size_slash < size_back) keep_slash += size_back - size_slash;
    else keep_back += size_slash - size_back;
    if (keep_slash > keep_back) return kDecCross | kDecBack;
    if (keep_back > keep_slash) return kDecCross | kDecSlash;
    return kDecCross | kDecSlash | kDecBack;
}

template <int TW, int TH>
__device__ void cc_local_core(const uint8_t* sg, int* sl, uint16_t* run, int32_t* L, int w, int h, int x0, int y0);
template <int TW, int TH>
__device__ void cc_sym_unions(const uint8_t* sg, int* sl);
template <int TW, int TH>
__device__ void cc_sym_store(const uint8_t* sg, int* sl, int32_t* L, int w, int h, int x0, int y0);

// Heuristic resolution of one 64x16 tile; with L set, the tile's local
// component labels too (union-find over the resolved bytes, still in shared
// memory), which leaves the label stage only the merge across tile borders
// and the flattening.
template <bool TMA = false, bool VOTE = false>
__device__ __forceinline__ void heuristics_tile(const uint8_t* snap, uint8_t* out, int w, int h, int x0, int y0,
                                                int32_t* L = nullptr, const CUtensorMap* map = nullptr,
                                                int frame = 0)
{
    __shared__ __align__(128) uint8_t s[kHRH][kHRW];
    const int ox = x0 - kHalo, oy = y0 - kHalo;
    if constexpr (TMA) {
        // the window as one TMA box (x0 - 32 is a multiple of 16 bytes);
        // bytes outside the image read as zero
        __shared__ uint64_t bar;
        __shared__ int ok;
        if (threadIdx.x == 0) {
            mbar_init(&bar, 1);
            mbar_expect_tx(&bar, (uint32_t)sizeof(s));
            tma_load_3d(&s[0][0], map, ox, oy, frame, &bar);
            ok = tma_wait_or_flag(&bar, &g_heur_fault) ? 1 : 0;
        }
        __syncthreads();
        if (!ok) return;
    } else
    // 4-byte loads where a row is word aligned in memory, else bytes
    for (int k = threadIdx.x; k < kHRH * (kHRW / 4); k += blockDim.x) {
        int ry = k / (kHRW / 4), rx = 4 * (k % (kHRW / 4));
        int gy = oy + ry, gx = ox + rx;
        uint32_t v = 0;
        if (gy >= 0 && gy < h) {
            const uint8_t* row = snap + (size_t)gy * w;
            if (gx >= 0 && gx + 3 < w && ((reinterpret_cast<uintptr_t>(row + gx) & 3) == 0)) {
                v = __ldg(reinterpret_cast<const uint32_t*>(row + gx));
            } else {
                for (int q = 0; q < 4; q++)
                    if (gx + q >= 0 && gx + q < w) v |= (uint32_t)__ldg(row + gx + q) << (8 * q);
            }
        }
        *reinterpret_cast<uint32_t*>(&s[ry][rx]) = v;
    }
    SnapTile t{s, ox, oy};
    // each 2x2 block touching the tile decided once (the four corner nodes
    // each clear their own bit of it), as a kDec* code; blocks reaching
    // outside the image read the zero halo and are never crossings
    __shared__ uint8_t dec[kHTH + 1][kHTW + 1];
    __syncthreads();
    for (int k = threadIdx.x; k < (kHTW + 1) * (kHTH + 1); k += blockDim.x) {
        const int bx = k % (kHTW + 1), by = k / (kHTW + 1);
        const int bi = x0 - 1 + bx, bj = y0 - 1 + by;
        unsigned d = 0;
        if (bitof(t.at(bi, bj), 2) && bitof(t.at(bi, bj + 1), 7) && bitof(t.at(bi + 1, bj), 0) &&
            bitof(t.at(bi + 1, bj + 1), 5))
        {
            if constexpr (VOTE) d = vote_decision(s, ox, oy, bi, bj);
            else d = kDecCross | (block_decision(t, bi, bj) ? kDecSlash : kDecBack);
        }
        dec[by][bx] = (uint8_t)d;
    }
    __syncthreads();
    // With L, each pixel's union-find parent starts at the leftmost pixel of
    // its horizontal run, from one ballot of the warp that resolves the
    // pixel's 32-pixel row segment (a warp's 32 values of k are one segment:
    // blockDim.x is a multiple of 32 and a row is two segments); a run that
    // comes into the second segment from the first hangs from the first
    // segment's last pixel.
    __shared__ uint8_t res[kHTW * kHTH];
    __shared__ int sl[kHTW * kHTH];
    for (int k = threadIdx.x; k < kHTW * kHTH; k += blockDim.x) {
        const int tx = k % kHTW, ty = k / kHTW;
        const int i = x0 + tx, j = y0 + ty;
        unsigned v = 0;
        if (i < w && j < h) {
            unsigned o = t.at(i, j);
            // the node is the lower-right corner of block (i-1, j), the upper-right
            // of (i-1, j-1), the upper-left of (i, j-1), the lower-left of (i, j)
            const unsigned a = dec[ty + 1][tx], b = dec[ty][tx], c = dec[ty][tx + 1], d = dec[ty + 1][tx + 1];
            if (a & kDecBack) o &= ~1u;
            if (b & kDecSlash) o &= ~32u;
            if (c & kDecBack) o &= ~128u;
            if (d & kDecSlash) o &= ~4u;
            out[(size_t)j * w + i] = (uint8_t)o;
            v = o & inside_mask(i, j, w, h);
        }
        res[k] = (uint8_t)v;
        if (L) {
            const int lane = tx & 31;
            const unsigned starts = __ballot_sync(0xFFFFFFFFu, tx == 0 || !bitof(v, 3));
            const unsigned upto = starts & (0xFFFFFFFFu >> (31 - lane));
            sl[k] = upto ? (k - lane) + 31 - __clz(upto) : k - lane - 1;
        }
    }
    if (L) {
        __syncthreads();
        cc_sym_unions<kHTW, kHTH>(res, sl);
        __syncthreads();
        cc_sym_store<kHTW, kHTH>(res, sl, L, w, h, x0, y0);
    }
}

// VOTE: the weighted vote instead of the reference's ordered tests
template <bool VOTE>
__global__ void __launch_bounds__(256) k_heuristics(GraphBatch b)
{
    const uint8_t* snap = b.snap + b.frame_stride * blockIdx.z;
    uint8_t* out = b.out + b.frame_stride * blockIdx.z;
    heuristics_tile<false, VOTE>(snap, out, b.w, b.h, blockIdx.x * kHTW, blockIdx.y * kHTH);
}

template <bool VOTE>
__global__ void __launch_bounds__(256) k_heuristics_labels(GraphBatch b, int32_t* L)
{
    const uint8_t* snap = b.snap + b.frame_stride * blockIdx.z;
    uint8_t* out = b.out + b.frame_stride * blockIdx.z;
    heuristics_tile<false, VOTE>(snap, out, b.w, b.h, blockIdx.x * kHTW, blockIdx.y * kHTH,
                                 L + b.frame_stride * blockIdx.z);
}

// the same with the graph windows by TMA (width and frame stride multiples of
// 16 bytes, 16-byte aligned base); L may be NULL
template <bool VOTE>
__global__ void __launch_bounds__(256) k_heuristics_tma(GraphBatch b, int32_t* L, const __grid_constant__ CUtensorMap map)
{
    const uint8_t* snap = b.snap + b.frame_stride * blockIdx.z;
    uint8_t* out = b.out + b.frame_stride * blockIdx.z;
    heuristics_tile<true, VOTE>(snap, out, b.w, b.h, blockIdx.x * kHTW, blockIdx.y * kHTH,
                                L ? L + b.frame_stride * blockIdx.z : nullptr, &map, (int)blockIdx.z);
}

// -------------------------------------------------- component labelling

__device__ __forceinline__ int uf_find(int32_t* L, int x)
{
    int p = L[x];
    while (p != x) {
        x = p;
        p = L[x];
    }
    return x;
}

// lock-free union with the smaller root winning: the final root of every
// component is its minimum index
__device__ __forceinline__ void uf_unite(int32_t* L, int a, int b)
{
    for (;;) {
        a = uf_find(L, a);
        b = uf_find(L, b);
        if (a == b) return;
        if (a > b) {
            int t = a;
            a = b;
            b = t;
        }
        int old = atomicMin(&L[b], a);
        if (old == b) return;
        b = old;
    }
}

// Component labels in three passes: union-find inside tiles in shared memory
// (local roots are the tile-local minima, which are also the minima in global
// index order), then unions across tile borders on the global label array,
// then one flattening pass. The frame and batch paths make the tile-local
// labels inside the 64x16 heuristics tiles (cc_sym_unions, cc_sym_store) and
// merge with merge_tile_borders; the stage API (depix_label_components) runs
// its own 32x32 tiles over a graph in global memory (cc_local_core: a warp
// owns a row, horizontal runs from one ballot, one union per pair of touching
// runs).
constexpr int kLT = 32;

// find with path compression, for the passes that follow the unions (no
// union in flight: every parent lowered is lowered to its final root)
__device__ __forceinline__ int s_find(int* L, int x)
{
    int r = x;
    while (L[r] != r) r = L[r];
    while (L[x] > r) {
        int nx = L[x];
        atomicMin(&L[x], r);
        x = nx;
    }
    return r;
}

// root without compression, for the unions themselves
__device__ __forceinline__ int s_root(const int* L, int x)
{
    while (L[x] != x) x = L[x];
    return x;
}

// Lock-free union, the smaller root winning. Its finds do not compress:
// with compression interleaved with the unions of other threads, joins
// were lost on the GPU (tile-local labels of 4096-sprite batches wrong in
// about one tile in 10^5, one in 10^4 with volatile loads; none in 560
// batches, 6.2 million tiles, without it).
__device__ __forceinline__ void s_unite(int* L, int a, int b)
{
    for (;;) {
        a = s_root(L, a);
        b = s_root(L, b);
        if (a == b) return;
        if (a > b) {
            int t = a;
            a = b;
            b = t;
        }
        int old = atomicMin(&L[b], a);
        if (old == b) return;
        b = old;
    }
}

// position of the set bit of rank j (from 0, counted from bit 0) of m;
// j < popcount(m)
__device__ __forceinline__ int nth_set_bit64(uint64_t m, int j)
{
    const unsigned lo = (unsigned)m;
    const int nlo = __popc(lo);
    return j < nlo ? (int)__fns(lo, 0, j + 1) : 32 + (int)__fns((unsigned)(m >> 32), 0, j - nlo + 1);
}

// 64-bit row mask from the ballots of a warp's two 32-pixel segments
__device__ __forceinline__ uint64_t ballot64(bool lo, bool hi)
{
    return (uint64_t)__ballot_sync(0xFFFFFFFFu, lo) | (uint64_t)__ballot_sync(0xFFFFFFFFu, hi) << 32;
}

// the run start at or before position c of a line whose run starts are S
__device__ __forceinline__ int run_start(uint64_t S, int c) { return 63 - __clzll(S & (~0ull >> (63 - c))); }

// Which edges between two lines of at most 64 pixels, r and q, need a union
// when the pixels joined along each line are already one set. Edge e at
// position c joins r[c] and q[c + e - 1]; Sr and Sq mark where the lines'
// runs start; q_end marks positions past the end of q (another tile, so
// another set). An edge is skipped where another edge joins the same two
// runs: an e = 1 edge defers to the e = 1 edge one position before it, an
// e = 0 edge to the e = 0 or e = 1 edge one position before it, an e = 2
// edge to the e = 2 edge one position before it or the e = 1 edge one
// position after it, each when both runs are the same there. Every chain of
// deferrals ends at an edge that is kept (e = 0 and e = 1 edges defer only
// to lower positions, and an e = 2 edge to a lower position or to an e = 1
// edge), so the kept edges join the same sets as all of them.
__device__ __forceinline__ void join_masks(uint64_t Sr, uint64_t Sq, uint64_t E0, uint64_t E1, uint64_t E2,
                                           uint64_t q_end, uint64_t (&need)[3])
{
    const uint64_t nSr = ~Sr, nSq = ~Sq;
    need[0] = E0 & ~(nSr & (((E0 & nSq) << 1) | (E1 << 1)));
    need[1] = E1 & ~((E1 << 1) & nSr & nSq);
    need[2] = E2 & ~(((E2 << 1) & nSr & ~((Sq >> 1) | q_end)) | ((E1 & nSr) >> 1));
}

// fn(e, c) for every set bit c of need[e], spread over the warp's lanes
// (one union per lane in turn)
template <typename Fn>
__device__ __forceinline__ void for_each_join(const uint64_t (&need)[3], Fn fn)
{
    const int lane = threadIdx.x & 31;
    const int n0 = __popcll(need[0]), n01 = n0 + __popcll(need[1]), n = n01 + __popcll(need[2]);
    for (int i = lane; i < n; i += 32) {
        const int e = i < n0 ? 0 : i < n01 ? 1 : 2;
        const uint64_t m = e == 0 ? need[0] : e == 1 ? need[1] : need[2];
        fn(e, nth_set_bit64(m, i - (e == 0 ? 0 : e == 1 ? n0 : n01)));
    }
}

// Joins of a 64-pixel-wide tile of a symmetric graph (each edge held by
// both of its nodes, as in the resolved graph) whose parents start at the
// run roots (a run's leftmost pixel, see heuristics_tile). Warp w owns the
// row pairs (r, r + 1) for r = w and w + 8 (edges up-left, up, up-right as
// e = 0, 1, 2): it parks each pair's run starts and the edges join_masks
// keeps, then spreads the unions of both pairs over its lanes at once (one
// round of unions for up to 32 of them, not one per pair). Blocks of 256
// threads (8 warps).
template <int TW, int TH>
__device__ void cc_sym_unions(const uint8_t* sg, int* sl)
{
    static_assert(TW == 64 && TH <= 17, "two 32-pixel segments per row, at most two row pairs per warp");
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    __shared__ uint64_t pm[8][2][5]; // per warp and pair: Sr, Sq, kept edges e = 0, 1, 2
    __shared__ int pcnt[8][7];       // per warp: prefix of the kept-edge counts
    int npairs = 0;
    for (int r = warp; r < TH - 1; r += nwarp, npairs++) {
        const int p0 = r * TW + lane;
        const unsigned a0 = sg[p0], a1 = sg[p0 + 32], b0 = sg[p0 + TW], b1 = sg[p0 + TW + 32];
        const uint64_t Sr = ballot64(lane == 0 || !bitof(a0, 3), !bitof(a1, 3));
        const uint64_t Sq = ballot64(lane == 0 || !bitof(b0, 3), !bitof(b1, 3));
        uint64_t need[3];
        join_masks(Sr, Sq, ballot64(bitof(a0, 0), bitof(a1, 0)) & ~1ull, ballot64(bitof(a0, 1), bitof(a1, 1)),
                   ballot64(bitof(a0, 2), bitof(a1, 2)) & ~(1ull << 63), 1ull << 63, need);
        if (lane == 0) {
            pm[warp][npairs][0] = Sr;
            pm[warp][npairs][1] = Sq;
            pm[warp][npairs][2] = need[0];
            pm[warp][npairs][3] = need[1];
            pm[warp][npairs][4] = need[2];
        }
    }
    __syncwarp();
    if (lane == 0) {
        int t = 0;
        for (int k = 0; k < 6; k++) {
            pcnt[warp][k] = t;
            t += k / 3 < npairs ? __popcll(pm[warp][k / 3][2 + k % 3]) : 0;
        }
        pcnt[warp][6] = t;
    }
    __syncwarp();
    const int n = pcnt[warp][6];
    for (int i = lane; i < n; i += 32) {
        int k = 0;
        while (k < 5 && pcnt[warp][k + 1] <= i) k++;
        const int pr = k / 3, e = k % 3, r = warp + pr * nwarp;
        const uint64_t* m = pm[warp][pr];
        const int c = nth_set_bit64(m[2 + e], i - pcnt[warp][k]);
        s_unite(sl, r * TW + run_start(m[0], c), (r + 1) * TW + run_start(m[1], c + e - 1));
    }
}

// Labels of a tile after cc_sym_unions: one find per run (at its leftmost
// pixel), shuffled to the run's other pixels (a run that comes into the
// second segment takes the first segment's last label), stored as global
// indices of the tile-local roots.
template <int TW, int TH>
__device__ void cc_sym_store(const uint8_t* sg, int* sl, int32_t* L, int w, int h, int x0, int y0)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    for (int r = warp; r < TH; r += nwarp) {
        int carry = 0;
#pragma unroll
        for (int sgm = 0; sgm < TW / 32; sgm++) {
            const int c = sgm * 32 + lane, p = r * TW + c;
            const unsigned starts = __ballot_sync(0xFFFFFFFFu, c == 0 || !bitof(sg[p], 3));
            const unsigned upto = starts & (0xFFFFFFFFu >> (31 - lane));
            const int src = upto ? 31 - __clz(upto) : 0;
            int g = 0;
            if (upto && src == lane) {
                const int root = s_find(sl, p);
                g = (y0 + root / TW) * w + (x0 + root % TW);
            }
            g = __shfl_sync(0xFFFFFFFFu, g, src);
            if (!upto) g = carry;
            carry = __shfl_sync(0xFFFFFFFFu, g, 31);
            const int x = x0 + c, y = y0 + r;
            if (x < w && y < h) L[(size_t)y * w + x] = g;
        }
    }
}

// Union-find over a TW x TH tile whose graph bytes are in shared memory (sg,
// row-major, 0 outside the image): local roots as global indices. A warp
// owns a row and walks its 32-pixel segments left to right: horizontal runs
// from one ballot per segment (a run's root is its leftmost pixel, carried
// across segments), rows joined with one union per pair of touching runs.
template <int TW, int TH>
__device__ void cc_local_core(const uint8_t* sg, int* sl, uint16_t* run, int32_t* L, int w, int h, int x0, int y0)
{
    static_assert(TW % 32 == 0 && TW * TH <= 65536, "tile shape");
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    for (int r = warp; r < TH; r += nwarp) {
        int carry = r * TW;
#pragma unroll
        for (int sgm = 0; sgm < TW / 32; sgm++) {
            const int c = sgm * 32 + lane, p = r * TW + c;
            const bool link = c > 0 && (bitof(sg[p], 3) || bitof(sg[p - 1], 4));
            const unsigned starts = __ballot_sync(0xFFFFFFFFu, !link);
            const unsigned upto = lane == 31 ? starts : (starts & ((2u << lane) - 1u));
            const int root = upto ? r * TW + sgm * 32 + (31 - __clz(upto)) : carry;
            run[p] = (uint16_t)root;
            sl[p] = root;
            carry = __shfl_sync(0xFFFFFFFFu, root, 31);
        }
    }
    __syncthreads();
    for (int r = warp; r < TH - 1; r += nwarp) {
#pragma unroll
        for (int sgm = 0; sgm < TW / 32; sgm++) {
            const int c = sgm * 32 + lane, p = r * TW + c;
            const unsigned node = sg[p];
#pragma unroll
            for (int e = 0; e <= 2; e++) { // up-left, up, up-right
                const int nc = c + dir_di(e);
                if (nc < 0 || nc >= TW) continue;
                const int q = p + TW + dir_di(e);
                if (!(bitof(node, e) || bitof(sg[q], 7 - e))) continue;
                // the pixel to the left already joins the same two runs
                if (c > 0 && nc > 0 && run[p - 1] == run[p] && run[q - 1] == run[q] &&
                    (bitof(sg[p - 1], e) || bitof(sg[q - 1], 7 - e)))
                    continue;
                s_unite(sl, run[p], run[q]);
            }
        }
    }
    __syncthreads();
    for (int p = threadIdx.x; p < TW * TH; p += blockDim.x) {
        const int x = x0 + p % TW, y = y0 + p / TW;
        if (x >= w || y >= h) continue;
        const int r = s_find(sl, p);
        L[(size_t)y * w + x] = (y0 + r / TW) * w + (x0 + r % TW);
    }
}

// union-find inside one 32x32 tile (x0, y0) of a graph in global memory
__device__ void cc_local_tile(const uint8_t* g, int32_t* L, int w, int h, int x0, int y0)
{
    __shared__ int sl[kLT * kLT];
    __shared__ uint16_t run[kLT * kLT];
    __shared__ uint8_t sg[kLT * kLT];
    for (int p = threadIdx.x; p < kLT * kLT; p += blockDim.x) {
        int x = x0 + p % kLT, y = y0 + p / kLT;
        sg[p] = (x < w && y < h) ? g[(size_t)y * w + x] & inside_mask(x, y, w, h) : 0;
    }
    __syncthreads();
    cc_local_core<kLT, kLT>(sg, sl, run, L, w, h, x0, y0);
}

__global__ void __launch_bounds__(256) k_cc_local(const uint8_t* g, int32_t* L, int w, int h, size_t frame_stride)
{
    cc_local_tile(g + frame_stride * blockIdx.z, L + frame_stride * blockIdx.z, w, h, blockIdx.x * kLT,
                  blockIdx.y * kLT);
}

// unions across tile borders: every set bit whose neighbour lies in another
// tile (each symmetric pair is seen from both ends; uniting twice is
// harmless). One thread per border pixel of a tile (4 * 32 - 4 of them).
constexpr int kLBorder = 4 * kLT - 4;

// unions of border pixel q (of 4 kLT - 4) of tile `tile` in the kLT x kLT
// tiling with neighbours in other tiles
__device__ __forceinline__ void cc_merge_border(const uint8_t* g, int32_t* L, int w, int h, int tile, int q)
{
    constexpr int TW = kLT, TH = kLT;
    const int tiles_x = (w + TW - 1) / TW;
    // border position q: bottom row, top row, then left and right columns
    int lx, ly;
    if (q < TW) { lx = q; ly = 0; }
    else if (q < 2 * TW) { lx = q - TW; ly = TH - 1; }
    else if (q < 2 * TW + TH - 2) { lx = 0; ly = q - 2 * TW + 1; }
    else { lx = TW - 1; ly = q - (2 * TW + TH - 2) + 1; }
    const int i = (tile % tiles_x) * TW + lx, j = (tile / tiles_x) * TH + ly;
    if (i >= w || j >= h) return;
    const int k = j * w + i;
    unsigned node = g[k];
#pragma unroll
    for (int e = 0; e < 8; e++) {
        if (!bitof(node, e)) continue;
        int ni = i + dir_di(e), nj = j + dir_dj(e);
        if (ni < 0 || nj < 0 || ni >= w || nj >= h) continue;
        if (ni / TW == i / TW && nj / TH == j / TH) continue;
        uf_unite(L, k, nj * w + ni);
    }
}

// Unions across two borders of the 64x16 tile (tx, ty) of a symmetric
// graph, by one warp. Rows y0 + 15 and y0 + 16: the edges from row y0 + 15
// to (x - 1, y + 1), (x, y + 1), (x + 1, y + 1), the first reaching from
// column x0 into the tile at (tx - 1, ty + 1) and the last from column
// x0 + 63 into (tx + 1, ty + 1). Columns x0 + 63 and x0 + 64 over rows
// y0 .. y0 + 15 (runs along the columns: the pixels joined by their (x, y + 1)
// edge): the edges (x + 1, y) of every row, (x + 1, y + 1) of rows y0 ..
// y0 + 14 and, from column x0 + 64, (x - 1, y + 1) of those rows; the two
// diagonals from row y0 + 15 belong to the row pairs of this tile and of
// tile (tx + 1, ty). Every cross-tile pair is joined by exactly one tile, and
// of the edges between the same two runs only one (join_masks).
// unite(a, b) joins the sets of pixels a and b (frame indices).
template <typename Unite>
__device__ void merge_tile_borders(const uint8_t* g, int w, int h, int tx, int ty, Unite unite)
{
    const int lane = threadIdx.x & 31;
    const int x0 = tx * kHTW, y0 = ty * kHTH;
    const int yr = y0 + kHTH - 1, yq = yr + 1;
    if (yq < h) {
        unsigned a[2], b[2];
#pragma unroll
        for (int sgm = 0; sgm < 2; sgm++) {
            const int x = x0 + 32 * sgm + lane;
            a[sgm] = x < w ? g[(size_t)yr * w + x] & inside_mask(x, yr, w, h) : 0u;
            b[sgm] = x < w ? g[(size_t)yq * w + x] & inside_mask(x, yq, w, h) : 0u;
        }
        const uint64_t Sr = ballot64(lane == 0 || !bitof(a[0], 3), !bitof(a[1], 3));
        const uint64_t Sq = ballot64(lane == 0 || !bitof(b[0], 3), !bitof(b[1], 3));
        uint64_t need[3];
        join_masks(Sr, Sq, ballot64(bitof(a[0], 0), bitof(a[1], 0)), ballot64(bitof(a[0], 1), bitof(a[1], 1)),
                   ballot64(bitof(a[0], 2), bitof(a[1], 2)), 1ull << 63, need);
        for_each_join(need, [&](int e, int c) {
            const int nc = c + e - 1, qc = nc < 0 || nc >= kHTW ? nc : run_start(Sq, nc);
            unite(yr * w + x0 + run_start(Sr, c), yq * w + x0 + qc);
        });
    }
    const int xr = x0 + kHTW - 1, xq = xr + 1;
    if (xq < w) {
        const int y = y0 + lane;
        unsigned a = 0, b = 0;
        if (lane < kHTH && y < h) {
            a = g[(size_t)y * w + xr] & inside_mask(xr, y, w, h);
            b = g[(size_t)y * w + xq] & inside_mask(xq, y, w, h);
        }
        // runs along the columns: row y starts one unless row y - 1 links up
        const uint64_t Sr = ~((uint64_t)__ballot_sync(0xFFFFFFFFu, bitof(a, 1)) << 1);
        const uint64_t Sq = ~((uint64_t)__ballot_sync(0xFFFFFFFFu, bitof(b, 1)) << 1);
        const uint64_t E1 = __ballot_sync(0xFFFFFFFFu, bitof(a, 4));
        const uint64_t E2 = __ballot_sync(0xFFFFFFFFu, bitof(a, 2)) & 0x7FFFu;
        const uint64_t E0 = (uint64_t)(__ballot_sync(0xFFFFFFFFu, bitof(b, 0)) & 0x7FFFu) << 1;
        uint64_t need[3];
        join_masks(Sr, Sq, E0, E1, E2, 1ull << 63, need);
        for_each_join(need, [&](int e, int c) {
            unite((y0 + run_start(Sr, c)) * w + xr, (y0 + run_start(Sq, c + e - 1)) * w + xq);
        });
    }
}

// the same on the global labels
__device__ __forceinline__ void cc_merge_tile_warp(const uint8_t* g, int32_t* L, int w, int h, int tx, int ty)
{
    merge_tile_borders(g, w, h, tx, ty, [&](int a, int b) { uf_unite(L, a, b); });
}

// one warp per 64x16 tile
__global__ void __launch_bounds__(128) k_cc_merge_tiles(const uint8_t* g, int32_t* L, int w, int h, size_t frame_stride)
{
    const int tiles_x = (w + kHTW - 1) / kHTW, tiles = tiles_x * ((h + kHTH - 1) / kHTH);
    const int t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (t >= tiles) return;
    cc_merge_tile_warp(g + frame_stride * blockIdx.z, L + frame_stride * blockIdx.z, w, h, t % tiles_x,
                       t / tiles_x);
}

__global__ void k_cc_merge(const uint8_t* g, int32_t* L, int w, int h, size_t frame_stride)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int tiles = ((w + kLT - 1) / kLT) * ((h + kLT - 1) / kLT);
    if (t / kLBorder >= tiles) return;
    cc_merge_border(g + frame_stride * blockIdx.z, L + frame_stride * blockIdx.z, w, h, t / kLBorder, t % kLBorder);
}

// Four consecutive pixels per thread, their labels in one 16-byte load where
// aligned and their four finds interleaved, so that each thread keeps four
// independent loads in flight (one find per pixel is bound by load latency).
__global__ void k_cc_flatten(int32_t* L, int n, size_t frame_stride)
{
    const int k = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
    if (k >= n) return;
    L += frame_stride * blockIdx.z;
    int32_t* q = L + k;
    int p[4], x[4];
    if (k + 3 < n && (reinterpret_cast<uintptr_t>(q) & 15) == 0) {
        const int4 v = *reinterpret_cast<const int4*>(q);
        p[0] = v.x;
        p[1] = v.y;
        p[2] = v.z;
        p[3] = v.w;
    } else {
#pragma unroll
        for (int i = 0; i < 4; i++) p[i] = k + i < n ? q[i] : k + i;
    }
    int first[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        x[i] = k + i;
        first[i] = p[i];
    }
    for (;;) {
        bool more = false;
#pragma unroll
        for (int i = 0; i < 4; i++)
            if (p[i] != x[i]) {
                x[i] = p[i];
                p[i] = L[x[i]];
                more = true;
            }
        if (!more) break;
    }
#pragma unroll
    for (int i = 0; i < 4; i++)
        if (k + i < n && first[i] != x[i]) q[i] = x[i];
}

// ------------------------------------------------ uneven batches (queue)

__global__ void __launch_bounds__(256) k_graph_queue(QueueBatch q)
{
    const QueueHeader* H = q.hdr;
    const int n = H->n;
    queue_loop(q.counters + QC_GRAPH, (int)H->total[QS_GRAPH], q.gran[QS_GRAPH], [&](int t) {
        const uint32_t* base = H->base + QS_GRAPH * (n + 1);
        const int f = queue_frame(base, n, (uint32_t)t);
        const QueueFrame fr = H->frames[f];
        const int lt = t - (int)base[f], tx = (fr.w + kGTW - 1) / kGTW;
        FrameRef ref{H->img + fr.in_off, fr.w, fr.h, 4 * fr.w, q.graph_a + fr.px_off};
        graph_tile<DEPIX_LAYOUT_RGBA>(ref, (lt % tx) * kGTW, (lt / tx) * kGTH, H->thr, true);
    });
}

template <bool VOTE>
__global__ void __launch_bounds__(256) k_heur_queue(QueueBatch q)
{
    const QueueHeader* H = q.hdr;
    const int n = H->n;
    queue_loop(q.counters + QC_HEUR, (int)H->total[QS_HEUR], q.gran[QS_HEUR], [&](int t) {
        const uint32_t* base = H->base + QS_HEUR * (n + 1);
        const int f = queue_frame(base, n, (uint32_t)t);
        const QueueFrame fr = H->frames[f];
        const int lt = t - (int)base[f], tx = (fr.w + kHTW - 1) / kHTW;
        heuristics_tile<false, VOTE>(q.graph_a + fr.px_off, q.graph_b + fr.px_off, fr.w, fr.h, (lt % tx) * kHTW,
                                     (lt / tx) * kHTH, H->labels ? H->labels + fr.px_off : nullptr);
    });
}


__global__ void __launch_bounds__(128) k_label_merge_queue(QueueBatch q)
{
    // the local labels came with the heuristics stage: its tiles, its prefix
    const QueueHeader* H = q.hdr;
    const int n = H->n;
    warp_queue_loop(q.counters + QC_MERGE, (int)H->total[QS_HEUR], q.gran[QS_LABEL], [&](int t) {
        const uint32_t* base = H->base + QS_HEUR * (n + 1);
        const int f = queue_frame(base, n, (uint32_t)t);
        const QueueFrame fr = H->frames[f];
        const int lt = t - (int)base[f], tx = (fr.w + kHTW - 1) / kHTW;
        cc_merge_tile_warp(q.graph_b + fr.px_off, H->labels + fr.px_off, fr.w, fr.h, lt % tx, lt / tx);
    });
}

__global__ void __launch_bounds__(256) k_label_flatten_queue(QueueBatch q)
{
    const QueueHeader* H = q.hdr;
    const int n = H->n;
    queue_loop(q.counters + QC_FLATTEN, (int)H->total[QS_LABEL], q.gran[QS_LABEL], [&](int t) {
        const uint32_t* base = H->base + QS_LABEL * (n + 1);
        const int f = queue_frame(base, n, (uint32_t)t);
        const QueueFrame fr = H->frames[f];
        const int lt = t - (int)base[f], tx = (fr.w + kLT - 1) / kLT;
        const int x0 = (lt % tx) * kLT, y0 = (lt / tx) * kLT;
        int32_t* L = H->labels + fr.px_off;
        for (int p = threadIdx.x; p < kLT * kLT; p += blockDim.x) {
            const int x = x0 + p % kLT, y = y0 + p / kLT;
            if (x < fr.w && y < fr.h) L[y * fr.w + x] = uf_find(L, y * fr.w + x);
        }
    });
}

cudaError_t queue_graph(const QueueBatch& q, int blocks, cudaStream_t s)
{
    k_graph_queue<<<blocks, 256, 0, s>>>(q);
    return cudaGetLastError();
}

cudaError_t queue_heuristics(const QueueBatch& q, int blocks, cudaStream_t s)
{
    if (q.vote) k_heur_queue<true><<<blocks, 256, 0, s>>>(q);
    else k_heur_queue<false><<<blocks, 256, 0, s>>>(q);
    return cudaGetLastError();
}

cudaError_t queue_labels(const QueueBatch& q, int blocks, cudaStream_t s)
{
    // local labels were made by the heuristics stage
    k_label_merge_queue<<<blocks, 128, 0, s>>>(q);
    k_label_flatten_queue<<<blocks, 256, 0, s>>>(q);
    return cudaGetLastError();
}

static_assert(kQGraphTW == kGTW && kQGraphTH == kGTH, "graph queue tile");
static_assert(kQHeurTW == kHTW && kQHeurTH == kHTH, "heuristics queue tile");
static_assert(kQLabelT == kLT, "label queue tile");

template <typename K>
static int occupancy(K kernel, int threads)
{
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, threads, 0) != cudaSuccess) return 0;
    return nb;
}

int queue_blocks_per_sm(int stage, const QueueBatch& q)
{
    switch (stage) {
    case QS_GRAPH: return occupancy(k_graph_queue, 256);
    case QS_HEUR: return q.vote ? occupancy(k_heur_queue<true>, 256) : occupancy(k_heur_queue<false>, 256);
    case QS_LABEL: return occupancy(k_label_flatten_queue, 256);
    default: return queue_raster_blocks_per_sm(q);
    }
}

__global__ void k_yuv_words(const uint8_t* px3, size_t n, int mode, uint32_t* out)
{
    size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    out[k] = yuv_word(px3[3 * k], px3[3 * k + 1], px3[3 * k + 2], mode);
}

// ----------------------------------------------------------------- launch

cudaError_t launch_yuv_words(const uint8_t* px3, size_t n, int mode, uint32_t* out, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    k_yuv_words<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(px3, n, mode, out);
    return cudaGetLastError();
}

cudaError_t set_graph_tma_timeout_test(int on)
{
    int v = on ? 1 : 0;
    return cudaMemcpyToSymbol(g_graph_tma_timeout_test, &v, sizeof(int));
}

cudaError_t take_graph_fault(int* out)
{
    int zero = 0;
    cudaError_t e = cudaMemcpyFromSymbol(out, g_graph_fault, sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_graph_fault, &zero, sizeof(int));
    return e;
}

cudaError_t launch_graph(const FrameBatch& b, int nframes, uint32_t thr, bool fuse_trivial, cudaStream_t s)
{
    dim3 grid((b.w + kGTW - 1) / kGTW, (b.h + kGTH - 1) / kGTH, nframes);
    CUtensorMap map;
    if (b.layout == DEPIX_LAYOUT_RGBA &&
        rgba_tensor_map(b.img, b.w, b.h, b.ws, b.img_stride, nframes, kGBoxW, kGBoxH, &map))
        k_graph_tma<<<grid, 256, 0, s>>>(b, thr, fuse_trivial ? 1 : 0, map);
    else if (b.layout == DEPIX_LAYOUT_RGBA)
        k_graph<DEPIX_LAYOUT_RGBA><<<grid, 256, 0, s>>>(b, thr, fuse_trivial ? 1 : 0);
    else
        k_graph<DEPIX_LAYOUT_BGR><<<grid, 256, 0, s>>>(b, thr, fuse_trivial ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_trivial(uint8_t* g, int w, int h, cudaStream_t s)
{
    dim3 blk(32, 8), grid((w + 31) / 32, (h + 7) / 8);
    k_trivial<<<grid, blk, 0, s>>>(g, w, h);
    return cudaGetLastError();
}

cudaError_t launch_heuristics(const GraphBatch& b, int nframes, cudaStream_t s)
{
    dim3 grid((b.w + kHTW - 1) / kHTW, (b.h + kHTH - 1) / kHTH, nframes);
    CUtensorMap map;
    const bool tma = u8_tensor_map(b.snap, b.w, b.h, b.frame_stride, nframes, kHRW, kHRH, &map);
    if (tma && b.vote) k_heuristics_tma<true><<<grid, 256, 0, s>>>(b, nullptr, map);
    else if (tma) k_heuristics_tma<false><<<grid, 256, 0, s>>>(b, nullptr, map);
    else if (b.vote) k_heuristics<true><<<grid, 256, 0, s>>>(b);
    else k_heuristics<false><<<grid, 256, 0, s>>>(b);
    return cudaGetLastError();
}

cudaError_t launch_heuristics_labels(const GraphBatch& b, int nframes, int32_t* labels, cudaStream_t s)
{
    dim3 grid((b.w + kHTW - 1) / kHTW, (b.h + kHTH - 1) / kHTH, nframes);
    CUtensorMap map;
    const bool tma = u8_tensor_map(b.snap, b.w, b.h, b.frame_stride, nframes, kHRW, kHRH, &map);
    if (tma && b.vote) k_heuristics_tma<true><<<grid, 256, 0, s>>>(b, labels, map);
    else if (tma) k_heuristics_tma<false><<<grid, 256, 0, s>>>(b, labels, map);
    else if (b.vote) k_heuristics_labels<true><<<grid, 256, 0, s>>>(b, labels);
    else k_heuristics_labels<false><<<grid, 256, 0, s>>>(b, labels);
    return cudaGetLastError();
}

cudaError_t take_heuristics_fault(int* out)
{
    int zero = 0;
    cudaError_t e = cudaMemcpyFromSymbol(out, g_heur_fault, sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_heur_fault, &zero, sizeof(int));
    return e;
}

cudaError_t launch_labels_after_heuristics(const uint8_t* g, int32_t* labels, int w, int h, int nframes,
                                          size_t frame_stride, cudaStream_t s)
{
    const int n = w * h;
    const int tiles = ((w + kHTW - 1) / kHTW) * ((h + kHTH - 1) / kHTH);
    k_cc_merge_tiles<<<dim3((tiles + 3) / 4, 1, nframes), 128, 0, s>>>(g, labels, w, h, frame_stride);
    k_cc_flatten<<<dim3((n + 1023) / 1024, 1, nframes), 256, 0, s>>>(labels, n, frame_stride);
    return cudaGetLastError();
}

cudaError_t launch_labels(const uint8_t* g, int32_t* labels, int w, int h, int nframes, size_t frame_stride,
                          cudaStream_t s)
{
    int n = w * h;
    dim3 tiles((w + kLT - 1) / kLT, (h + kLT - 1) / kLT, nframes);
    k_cc_local<<<tiles, 256, 0, s>>>(g, labels, w, h, frame_stride);
    const int borders = tiles.x * tiles.y * kLBorder;
    k_cc_merge<<<dim3((borders + 127) / 128, 1, nframes), 128, 0, s>>>(g, labels, w, h, frame_stride);
    dim3 grid((n + 1023) / 1024, 1, nframes);
    k_cc_flatten<<<grid, 256, 0, s>>>(labels, n, frame_stride);
    return cudaGetLastError();
}

}  // namespace depix
