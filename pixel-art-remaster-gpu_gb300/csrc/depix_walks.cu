// depix_walks.cu -- border walks of the resolved graph's components, the
// input of the reference's spline export (extractBorderPoints,
// cc_functions.cu:348-503; recorded output alex_png.txt).
//
// The walks of one frame depend on each other in scan order (a node listed
// by one walk starts none; a walk that runs into a listed or discarded node
// is dropped and discards a node), so a frame is one thread's sequential
// loop. Lanes of one warp would run their frames' walks in lockstep, each
// waiting for the longest, so a batch runs one frame per warp: the lanes
// find the walks' start nodes by ballot and lane 0 walks. A frame that fits
// keeps its graph and node state (bit 0 listed, bit 1 discarded; two bits a
// node) in shared memory; larger frames read the graph from global memory
// and keep a state byte per node in a caller-provided scratch.
#include "depix_internal.h"

namespace depix {

// The reference enumerates a node's links clockwise from up-left (clock
// positions 0..7) and maps them to node bits and back (getRealLinkIndex /
// getClockLinkIndex, cc_functions.cu:48-100, 127-183), packed as nibbles.
__device__ __forceinline__ int real_of_clock(int c) { return (int)((0x35674210u >> (4 * (c & 7))) & 0xFu); }
__device__ __forceinline__ int clock_of_real(int r) { return (int)((0x45637210u >> (4 * r)) & 0xFu); }

// getFirstLink (cc_functions.cu:107-119)
__device__ __forceinline__ int walk_first_link(unsigned v)
{
    for (int c = 0; c < 8; c++)
        if ((v >> real_of_clock(c)) & 1u) return real_of_clock(c);
    return -1;
}

// nextEdgeCounterClockwise (cc_functions.cu:265-287)
__device__ __forceinline__ int walk_next_ccw(unsigned v, int e)
{
    if (__popc(v) == 1) return e;
    const int c = clock_of_real(e);
    for (int k = c + 7; k >= c + 1; k--)
        if ((v >> real_of_clock(k)) & 1u) return real_of_clock(k);
    return e;
}

// the link a walk leaves a node of links v by after arriving along e
// (nextNodeClockwise, cc_functions.cu:296-318); the link back on a valence-1
// node, and (not in the reference) on a node without links
__device__ __forceinline__ int walk_next_cw(unsigned v, int e)
{
    const int back = 7 - e;
    if (__popc(v) == 1) return back;
    const int c = clock_of_real(back);
    for (int k = c + 1; k <= c + 7; k++)
        if ((v >> real_of_clock(k)) & 1u) return real_of_clock(k);
    return back;
}

// Walk k of frame f: nodes[f * max_nodes + offsets[k] .. + offsets[k + 1]),
// offsets at offsets + f * (max_walks + 1); counts[3 f ..]: walks, nodes, 1
// when a capacity ran out (outputs up to the last complete walk). The rules
// are those of orc_border_walks in the oracle: scan order, internal (90) and
// listed nodes start none, a node without links is a walk of its own, a walk
// is dropped when it enters an internal, listed or discarded node (its last
// node discarded, its start unlisted) or passes 8 w h + 8 steps.
// Node state of one frame: bit 0 listed, bit 1 discarded.
struct ByteState { // a byte per node (global scratch)
    uint8_t* s;
    __device__ __forceinline__ unsigned get(int p) const { return s[p]; }
    __device__ __forceinline__ void set(int p, unsigned b) const { s[p] |= (uint8_t)b; }
    __device__ __forceinline__ void clear(int p, unsigned b) const { s[p] &= (uint8_t)~b; }
};
struct PackedState { // two bits per node (shared memory)
    uint8_t* s;
    __device__ __forceinline__ unsigned get(int p) const { return (s[p >> 2] >> (2 * (p & 3))) & 3u; }
    __device__ __forceinline__ void set(int p, unsigned b) const { s[p >> 2] |= (uint8_t)(b << (2 * (p & 3))); }
    __device__ __forceinline__ void clear(int p, unsigned b) const { s[p >> 2] &= (uint8_t)~(b << (2 * (p & 3))); }
};

// walk_next_cw for every node byte v and arrival link e, at [v * 8 + e]
__device__ __forceinline__ void build_cw_table(uint8_t* cw, int tid, int nthreads)
{
    for (int i = tid; i < 256 * 8; i += nthreads) cw[i] = (uint8_t)walk_next_cw((unsigned)(i >> 3), i & 7);
}

// The walks of one frame, by one warp: the lanes find the nodes that can
// start a walk (not internal) 32 at a time by ballot, lane 0 walks from each
// in scan order (re-checking the state, which its walks change). cw: the
// walk_next_cw table.
template <typename State>
__device__ void walk_frame(const uint8_t* g, int w, int h, State fl, const uint8_t* cw, int32_t* on, int8_t* oe,
                           int32_t* oo, int max_nodes, int max_walks, int32_t* cnt)
{
    const int lane = threadIdx.x & 31;
    const long long limit = 8LL * (long long)w * h + 8;
    auto node = [&](int x, int y) -> unsigned { return g[(size_t)y * w + x] & inside_mask(x, y, w, h); };
    int nw = 0, pos = 0, trunc = 0; // lane 0's
    if (lane == 0) oo[0] = 0;
    for (int y = 0; y < h && !trunc; y++)
        for (int x0 = 0; x0 < w && !trunc; x0 += 32) {
            const int xl = x0 + lane;
            unsigned cand = __ballot_sync(0xFFFFFFFFu, xl < w && node(xl, y) != 90);
            if (lane == 0) {
                while (cand) {
                    const int x = x0 + __ffs(cand) - 1;
                    cand &= cand - 1;
                    const int p = y * w + x;
                    const unsigned v0 = node(x, y);
                    if (fl.get(p) & 1u) continue;
                    if (v0 == 0) {
                        if (nw >= max_walks || pos >= max_nodes) {
                            trunc = 1;
                            break;
                        }
                        on[pos] = p;
                        oe[pos++] = -1;
                        fl.set(p, 1u);
                        oo[++nw] = pos;
                        continue;
                    }
                    fl.set(p, 1u);
                    int e = walk_first_link(v0);
                    const int arr = walk_next_ccw(v0, e);
                    const int start = pos;
                    int over = 0, last = p; // over: a node did not fit (the walk is then not recorded)
                    if (pos < max_nodes) {
                        on[pos] = p;
                        oe[pos++] = (int8_t)e;
                    } else {
                        over = 1;
                    }
                    int cx = x, cy = y, ok = 1;
                    long long steps = 0;
                    while (!(cx + dir_di(e) == x && cy + dir_dj(e) == y && 7 - e == arr)) {
                        cx += dir_di(e);
                        cy += dir_dj(e);
                        const int cp = cy * w + cx;
                        const unsigned v = node(cx, cy);
                        e = cw[v * 8 + e];
                        if (v == 90 || fl.get(cp) || ++steps > limit) {
                            fl.set(last, 2u);
                            fl.clear(p, 1u);
                            pos = start;
                            ok = 0;
                            break;
                        }
                        last = cp;
                        if (pos < max_nodes) {
                            on[pos] = cp;
                            oe[pos++] = (int8_t)e;
                        } else {
                            over = 1;
                        }
                    }
                    if (ok) {
                        if (over || nw >= max_walks) {
                            pos = start;
                            trunc = 1;
                            break;
                        }
                        for (int q = start; q < pos; q++) fl.set(on[q], 1u);
                        oo[++nw] = pos;
                    }
                }
            }
            trunc = __shfl_sync(0xFFFFFFFFu, trunc, 0);
        }
    if (lane == 0) {
        cnt[0] = nw;
        cnt[1] = pos;
        cnt[2] = trunc;
    }
}

// frames whose graph (w h bytes) and packed state (w h / 4 bytes) fit in
// shared memory: one warp per frame loads both and walks
__global__ void __launch_bounds__(32) k_border_walks_smem(const uint8_t* graph, int w, int h, int32_t* nodes,
                                                          int8_t* edges, int32_t* offsets, int max_nodes, int max_walks,
                                                          int32_t* counts)
{
    extern __shared__ __align__(16) uint8_t sm[];
    __shared__ uint8_t cw[256 * 8];
    const size_t n = (size_t)w * h, f = blockIdx.x;
    const size_t gbytes = (n + 15) & ~(size_t)15, sbytes = (n + 3) / 4;
    const uint8_t* g = graph + n * f;
    for (size_t i = threadIdx.x; i < n; i += 32) sm[i] = __ldg(g + i);
    for (size_t i = threadIdx.x; i < sbytes; i += 32) sm[gbytes + i] = 0;
    build_cw_table(cw, threadIdx.x, 32);
    __syncwarp();
    walk_frame(sm, w, h, PackedState{sm + gbytes}, cw, nodes + (size_t)max_nodes * f, edges + (size_t)max_nodes * f,
               offsets + (size_t)(max_walks + 1) * f, max_nodes, max_walks, counts + 3 * f);
}

// larger frames: the graph from global memory, the state in the scratch; a
// warp per frame, four per block
__global__ void __launch_bounds__(128) k_border_walks(const uint8_t* graph, int w, int h, int nframes, uint8_t* flags,
                                                      int32_t* nodes, int8_t* edges, int32_t* offsets, int max_nodes,
                                                      int max_walks, int32_t* counts)
{
    __shared__ uint8_t cw[256 * 8];
    build_cw_table(cw, threadIdx.x, blockDim.x);
    __syncthreads();
    const int f = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (f >= nframes) return; // whole warps
    const size_t n = (size_t)w * h;
    walk_frame(graph + n * f, w, h, ByteState{flags + n * f}, cw, nodes + (size_t)max_nodes * f,
               edges + (size_t)max_nodes * f, offsets + (size_t)(max_walks + 1) * f, max_nodes, max_walks,
               counts + 3 * f);
}

constexpr size_t kWalkSmemMax = 200 * 1024;

cudaError_t launch_border_walks(const uint8_t* graph, int w, int h, int nframes, uint8_t* flags, int32_t* nodes,
                                int8_t* edges, int32_t* offsets, int max_nodes, int max_walks, int32_t* counts,
                                cudaStream_t s)
{
    const size_t n = (size_t)w * h, smem = ((n + 15) & ~(size_t)15) + (n + 3) / 4;
    if (smem <= kWalkSmemMax) {
        cudaError_t e = cudaFuncSetAttribute(k_border_walks_smem, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kWalkSmemMax);
        if (e != cudaSuccess) return e;
        k_border_walks_smem<<<nframes, 32, smem, s>>>(graph, w, h, nodes, edges, offsets, max_nodes, max_walks,
                                                      counts);
        return cudaGetLastError();
    }
    cudaError_t e = cudaMemsetAsync(flags, 0, n * nframes, s);
    if (e != cudaSuccess) return e;
    k_border_walks<<<(nframes + 3) / 4, 128, 0, s>>>(graph, w, h, nframes, flags, nodes, edges, offsets, max_nodes,
                                                      max_walks, counts);
    return cudaGetLastError();
}

}  // namespace depix
