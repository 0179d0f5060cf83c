/*
 * depix_oracle.c -- CPU restatement of the reference depixelization frame
 * path. TEST INFRASTRUCTURE ONLY: it is the checker for the CUDA library, is
 * loaded only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg, and is never linked into the product.
 *
 * Every stage cites the reference function it restates (file:line in the
 * reference project). Out-of-image reads follow the parity contract: bytes
 * outside the image buffers read as 0, in-buffer reads keep the reference's
 * linear (row-wrapping) addressing where the result depends on it.
 *
 * Build: gcc -O2 -fPIC -shared -ffp-contract=off (no FMA contraction, IEEE
 * division and sqrt: the semantics of the reference stage bodies compiled
 * for the host, against which this file is pinned).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_CELL 45 /* slots per cell (kernel.cu:8) */

typedef struct { float x, y; } opt;

static inline int bit_of(unsigned v, int k) { return (int)((v >> k) & 1u); }

/* neighbour offsets of node bit e, j increasing upward (graph_functions.cu:162-235) */
static const int DI[8] = {-1, 0, 1, -1, 1, -1, 0, 1};
static const int DJ[8] = {1, 1, 1, 0, 0, -1, -1, -1};

/* ---------------------------------------------------------------- graph */

/* Luma arithmetic modes (the library's depix_yuv): the reference's CUDA
 * build contracts y's double sum into fused multiply-adds (nvcc's default,
 * depixel_gpu.pro:48); its host build rounds every product and sum. */
#define ORC_YUV_CUDA 0
#define ORC_YUV_HOST 1

/* Packed YUV word of one pixel given its three bytes in memory order.
 * Restates DATAtoINT + RGBtoYUV (graph_functions.cu:80-131): the first byte
 * plays "r", the third "b"; y in double (graph_functions.cu:90), u/v in
 * float, truncation toward zero, negative u/v borrow into the higher fields.
 * mode ORC_YUV_CUDA: y = fma(0.114, b, fma(0.299, r, 0.587 g)), the order
 * the CUDA build evaluates (all 2^24 words equal that build's, measured on
 * the GPU); ORC_YUV_HOST: (0.299 r + 0.587 g) + 0.114 b, each operation
 * rounded (this file is compiled with -ffp-contract=off). */
uint32_t orc_yuv_word(uint8_t b0, uint8_t b1, uint8_t b2, int mode)
{
    int r = b0, g = b1, b = b2;
    double R = (double)(float)r, G = (double)(float)g, B = (double)(float)b;
    double yd;
    if (mode == ORC_YUV_HOST) {
        yd = 0.299 * R + 0.587 * G;
        yd = yd + 0.114 * B;
    } else {
        yd = fma(0.114, B, fma(0.299, R, 0.587 * G));
    }
    int y = (int)yd;
    int u = (int)((float)(b - y) * 0.492f);
    int v = (int)((float)(r - y) * 0.877f);
    return (uint32_t)(y * 65536 + u * 256 + v);
}

/* Bulk form over n pixels of 3 bytes each. */
void orc_yuv_words(const uint8_t* px, long n, int mode, uint32_t* out)
{
    for (long k = 0; k < n; k++) out[k] = orc_yuv_word(px[3 * k], px[3 * k + 1], px[3 * k + 2], mode);
}

/* Similarity test of two words (graph_functions.cu:291-293): every masked
 * field differs by at most its threshold (thresholds in field units). */
static int similar_words(uint32_t a, uint32_t b, int tr_y, int tr_u, int tr_v)
{
    int dy = (int)((a >> 16) & 0xFF) - (int)((b >> 16) & 0xFF);
    int du = (int)((a >> 8) & 0xFF) - (int)((b >> 8) & 0xFF);
    int dv = (int)(a & 0xFF) - (int)(b & 0xFF);
    return abs(dy) <= tr_y && abs(du) <= tr_u && abs(dv) <= tr_v;
}

/* Similarity graph (graph_Kernel, kernel.cu:140-159 + diff,
 * graph_functions.cu:147-311): bit e set iff the neighbour in direction e
 * lies inside the image and is similar. */
void orc_graph(const uint8_t* bgr, int w, int h, int ws, int tr_y, int tr_u, int tr_v, int mode, uint8_t* graph)
{
    uint32_t* words = (uint32_t*)malloc((size_t)w * h * sizeof(uint32_t));
    for (int j = 0; j < h; j++)
        for (int i = 0; i < w; i++) {
            const uint8_t* p = bgr + (size_t)j * ws + 3 * i;
            words[j * w + i] = orc_yuv_word(p[0], p[1], p[2], mode);
        }
    for (int j = 0; j < h; j++)
        for (int i = 0; i < w; i++) {
            unsigned node = 0;
            for (int e = 0; e < 8; e++) {
                int ni = i + DI[e], nj = j + DJ[e];
                if (ni < 0 || nj < 0 || ni >= w || nj >= h) continue;
                if (similar_words(words[j * w + i], words[nj * w + ni], tr_y, tr_u, tr_v)) node |= 1u << e;
            }
            graph[j * w + i] = (uint8_t)node;
        }
    free(words);
}

static inline unsigned gat(const uint8_t* g, int w, int h, int i, int j)
{
    if (i < 0 || j < 0 || i >= w || j >= h) return 0;
    return g[j * w + i];
}

/* bits of a node whose neighbour lies inside the image */
static inline unsigned inside_bits(int x, int y, int w, int h)
{
    unsigned m = 0xFFu;
    if (x == 0) m &= ~0x29u;     /* 0, 3, 5 */
    if (x == w - 1) m &= ~0x94u; /* 2, 4, 7 */
    if (y == 0) m &= ~0xE0u;     /* 5, 6, 7 */
    if (y == h - 1) m &= ~0x07u; /* 0, 1, 2 */
    return m;
}

/* Trivial crossing removal (crossCheck_4, graph_functions.cu:1211-1274): a
 * node drops a diagonal when the 2x2 block that diagonal crosses is fully
 * 4-connected. Only orthogonal bits are read, so in-place update is exact. */
void orc_trivial(uint8_t* g, int w, int h)
{
    for (int j = 0; j < h; j++)
        for (int i = 0; i < w; i++) {
            unsigned c = gat(g, w, h, i, j);
            unsigned l = gat(g, w, h, i - 1, j), r = gat(g, w, h, i + 1, j);
            unsigned u = gat(g, w, h, i, j + 1), d = gat(g, w, h, i, j - 1);
            unsigned ul = gat(g, w, h, i - 1, j + 1), ur = gat(g, w, h, i + 1, j + 1);
            unsigned dl = gat(g, w, h, i - 1, j - 1), dr = gat(g, w, h, i + 1, j - 1);
            unsigned out = c;
            /* up-left block {l, ul, c, u} */
            if (bit_of(l, 1) && bit_of(l, 4) && bit_of(ul, 6) && bit_of(ul, 4) && bit_of(c, 3) && bit_of(c, 1) &&
                bit_of(u, 6) && bit_of(u, 3))
                out &= ~1u;
            /* up-right block {c, u, r, ur} */
            if (bit_of(c, 1) && bit_of(c, 4) && bit_of(u, 6) && bit_of(u, 4) && bit_of(r, 3) && bit_of(r, 1) &&
                bit_of(ur, 6) && bit_of(ur, 3))
                out &= ~4u;
            /* down-left block {dl, l, d, c} */
            if (bit_of(dl, 1) && bit_of(dl, 4) && bit_of(l, 6) && bit_of(l, 4) && bit_of(d, 3) && bit_of(d, 1) &&
                bit_of(c, 6) && bit_of(c, 3))
                out &= ~32u;
            /* down-right block {d, c, dr, r} */
            if (bit_of(d, 1) && bit_of(d, 4) && bit_of(c, 6) && bit_of(c, 4) && bit_of(dr, 3) && bit_of(dr, 1) &&
                bit_of(r, 6) && bit_of(r, 3))
                out &= ~128u;
            g[j * w + i] = (uint8_t)out;
        }
}

/* number of set bits of node other than bit e (the loops k = e+1 .. e+7 of
 * checkValence2Edge / checkValence2Vertex / calcVal2PathSize) */
static int others(unsigned node, int e, int* last)
{
    int s = 0;
    for (int k = e + 1; k < e + 8; k++)
        if (bit_of(node, k % 8)) {
            s++;
            if (last) *last = k % 8;
        }
    return s;
}

/* Curve-length walk (calcVal2PathSize, graph_functions.cu:541-573): follow
 * valence-2 nodes, adding one per step, until a node of other valence or
 * until the running count passes 30. The count accumulates across calls. */
static void walk_len(const uint8_t* g, int w, int h, int i, int j, int e, int* result)
{
    for (;;) {
        int k_n = 0;
        int s = others(gat(g, w, h, i, j), e, &k_n);
        if (*result > 30) return;
        if (s != 1) return;
        (*result)++;
        i += DI[k_n];
        j += DJ[k_n];
        e = 7 - k_n;
    }
}

/* Heuristic decision for the 2x2 block whose lower-left node is (i, j)
 * (processHeuristics2, graph_functions.cu:761-849). Returns 1 to remove the
 * "/" diagonal (bits 2/5), 0 to remove "\" (bits 0/7). */
static int block_decision(const uint8_t* g, int w, int h, int i, int j)
{
    unsigned n1 = gat(g, w, h, i, j), n2 = gat(g, w, h, i, j + 1);
    unsigned n3 = gat(g, w, h, i + 1, j), n4 = gat(g, w, h, i + 1, j + 1);
    /* curves: a diagonal whose two ends each have exactly one other edge */
    if (others(n1, 2, 0) == 1 && others(n4, 5, 0) == 1) return 0;
    if (others(n3, 0, 0) == 1 && others(n2, 7, 0) == 1) return 1;
    /* islands; the second test keeps the reference's operator precedence
     * (graph_functions.cu:805): A || (B && !C && !D) */
    int v1 = others(n1, 2, 0) == 0, v4 = others(n4, 5, 0) == 0;
    int v3 = others(n3, 0, 0) == 0, v2 = others(n2, 7, 0) == 0;
    if ((v1 || v4) && !v3 && !v2) return 0;
    if (v3 || (v2 && !v1 && !v4)) return 1;
    /* curve length; a tie removes "/" */
    int seg = 0, seg2 = 0;
    walk_len(g, w, h, i, j, 2, &seg);
    walk_len(g, w, h, i + 1, j + 1, 5, &seg);
    walk_len(g, w, h, i + 1, j, 0, &seg2);
    walk_len(g, w, h, i, j + 1, 7, &seg2);
    return seg2 < seg ? 0 : 1;
}

/* Pixels of the component of (si, sj) inside the 8x8 window whose lower-left
 * pixel is (wi, wj), following set edge bits between window pixels only
 * (breadth-first search). */
static int window_component(const uint8_t* g, int w, int h, int wi, int wj, int si, int sj)
{
    int seen[8][8] = {{0}};
    int qx[64], qy[64], head = 0, tail = 0;
    seen[sj - wj][si - wi] = 1;
    qx[tail] = si;
    qy[tail++] = sj;
    while (head < tail) {
        int x = qx[head], y = qy[head++];
        unsigned nd = gat(g, w, h, x, y);
        for (int e = 0; e < 8; e++) {
            if (!bit_of(nd, e)) continue;
            int nx = x + DI[e], ny = y + DJ[e];
            if (nx < wi || ny < wj || nx >= wi + 8 || ny >= wj + 8 || seen[ny - wj][nx - wi]) continue;
            seen[ny - wj][nx - wi] = 1;
            qx[tail] = nx;
            qy[tail++] = ny;
        }
    }
    return tail;
}

/* Not in the reference: the weighted vote of Kopf and Lischinski,
 * "Depixelizing Pixel Art" (SIGGRAPH 2011), section 3.2, for the block whose
 * lower-left node is (i, j). Votes go to the diagonal to keep: curves by the
 * difference of the curve lengths (the walks of block_decision), sparse
 * pixels by the difference of the two diagonals' component sizes inside the
 * 8x8 window centred on the block (the smaller component's diagonal is
 * kept), islands 5 for a diagonal with an end that has no other edge.
 * Returns bit 0 to remove "/" (bits 2/5), bit 1 to remove "\" (bits 0/7);
 * a tie removes both. */
static int vote_decision(const uint8_t* g, int w, int h, int i, int j)
{
    unsigned n1 = gat(g, w, h, i, j), n2 = gat(g, w, h, i, j + 1);
    unsigned n3 = gat(g, w, h, i + 1, j), n4 = gat(g, w, h, i + 1, j + 1);
    int keep_slash = 0, keep_back = 0;
    int seg = 0, seg2 = 0;
    walk_len(g, w, h, i, j, 2, &seg);
    walk_len(g, w, h, i + 1, j + 1, 5, &seg);
    walk_len(g, w, h, i + 1, j, 0, &seg2);
    walk_len(g, w, h, i, j + 1, 7, &seg2);
    if (seg > seg2) keep_slash += seg - seg2;
    else keep_back += seg2 - seg;
    if (others(n1, 2, 0) == 0 || others(n4, 5, 0) == 0) keep_slash += 5;
    if (others(n3, 0, 0) == 0 || others(n2, 7, 0) == 0) keep_back += 5;
    int a = window_component(g, w, h, i - 3, j - 3, i, j);
    int b = window_component(g, w, h, i - 3, j - 3, i, j + 1);
    if (a < b) keep_slash += b - a;
    else keep_back += a - b;
    if (keep_slash > keep_back) return 2;
    if (keep_back > keep_slash) return 1;
    return 3;
}

/* The heuristics pass with the vote: each node of a crossing block clears
 * its own bit of every diagonal the vote removes. */
void orc_heuristics_vote(const uint8_t* snap, int w, int h, uint8_t* out)
{
    for (int j = 0; j < h; j++)
        for (int i = 0; i < w; i++) {
            unsigned c = gat(snap, w, h, i, j);
            unsigned o = c;
            if (bit_of(gat(snap, w, h, i - 1, j), 2) && bit_of(gat(snap, w, h, i - 1, j + 1), 7) && bit_of(c, 0) &&
                bit_of(gat(snap, w, h, i, j + 1), 5))
                if (vote_decision(snap, w, h, i - 1, j) & 2) o &= ~1u;
            if (bit_of(gat(snap, w, h, i - 1, j - 1), 2) && bit_of(gat(snap, w, h, i - 1, j), 7) &&
                bit_of(gat(snap, w, h, i, j - 1), 0) && bit_of(c, 5))
                if (vote_decision(snap, w, h, i - 1, j - 1) & 1) o &= ~32u;
            if (bit_of(gat(snap, w, h, i, j - 1), 2) && bit_of(c, 7) && bit_of(gat(snap, w, h, i + 1, j - 1), 0) &&
                bit_of(gat(snap, w, h, i + 1, j), 5))
                if (vote_decision(snap, w, h, i, j - 1) & 2) o &= ~128u;
            if (bit_of(c, 2) && bit_of(gat(snap, w, h, i, j + 1), 7) && bit_of(gat(snap, w, h, i + 1, j), 0) &&
                bit_of(gat(snap, w, h, i + 1, j + 1), 5))
                if (vote_decision(snap, w, h, i, j) & 1) o &= ~4u;
            out[j * w + i] = (uint8_t)o;
        }
}

/* Heuristic crossing resolution (crossCheck_Heuristics,
 * graph_functions.cu:1433-1518): for each of the four 2x2 blocks around a
 * node in which both diagonals survive in the snapshot, the node clears its
 * own bit of the diagonal the block decision removes. */
void orc_heuristics(const uint8_t* snap, int w, int h, uint8_t* out)
{
    for (int j = 0; j < h; j++)
        for (int i = 0; i < w; i++) {
            unsigned c = gat(snap, w, h, i, j);
            unsigned o = c;
            /* block with lower-left (i-1, j): node is its lower-right */
            if (bit_of(gat(snap, w, h, i - 1, j), 2) && bit_of(gat(snap, w, h, i - 1, j + 1), 7) && bit_of(c, 0) &&
                bit_of(gat(snap, w, h, i, j + 1), 5))
                if (!block_decision(snap, w, h, i - 1, j)) o &= ~1u;
            /* block with lower-left (i-1, j-1): node is its upper-right */
            if (bit_of(gat(snap, w, h, i - 1, j - 1), 2) && bit_of(gat(snap, w, h, i - 1, j), 7) &&
                bit_of(gat(snap, w, h, i, j - 1), 0) && bit_of(c, 5))
                if (block_decision(snap, w, h, i - 1, j - 1)) o &= ~32u;
            /* block with lower-left (i, j-1): node is its upper-left */
            if (bit_of(gat(snap, w, h, i, j - 1), 2) && bit_of(c, 7) && bit_of(gat(snap, w, h, i + 1, j - 1), 0) &&
                bit_of(gat(snap, w, h, i + 1, j), 5))
                if (!block_decision(snap, w, h, i, j - 1)) o &= ~128u;
            /* block with lower-left (i, j): node is its lower-left */
            if (bit_of(c, 2) && bit_of(gat(snap, w, h, i, j + 1), 7) && bit_of(gat(snap, w, h, i + 1, j), 0) &&
                bit_of(gat(snap, w, h, i + 1, j + 1), 5))
                if (block_decision(snap, w, h, i, j)) o &= ~4u;
            out[j * w + i] = (uint8_t)o;
        }
}

/* ---------------------------------------------------------------- cells */

typedef struct { int x, y; } qpt; /* point in quarter units */

/* Cell points of a node in emission order (createCellFromPattern,
 * diagram_functions.cu:320-520). left/right are the row neighbours' bytes. */
static int cell_points(unsigned nd, unsigned left, unsigned right, qpt* p)
{
    int n = 0;
#define PUT(X, Y) (p[n].x = (X), p[n].y = (Y), n++)
    int b0 = bit_of(nd, 0), b1 = bit_of(nd, 1), b2 = bit_of(nd, 2), b3 = bit_of(nd, 3);
    int b4 = bit_of(nd, 4), b5 = bit_of(nd, 5), b6 = bit_of(nd, 6), b7 = bit_of(nd, 7);
    if (b0) {
        if (b1 && !b3) PUT(-1, 3);
        else if (b3 && !b1) PUT(1, 5);
        else { PUT(-1, 3); PUT(1, 5); }
    } else if (bit_of(left, 2)) PUT(1, 3);
    else PUT(0, 4);
    if (b1) { PUT(0, 4); PUT(4, 4); }
    else PUT(2, 3);
    if (b2) {
        if (b1 && !b4) PUT(5, 3);
        else if (b4 && !b1) PUT(3, 5);
        else { PUT(3, 5); PUT(5, 3); }
    } else if (bit_of(right, 0)) PUT(3, 3);
    else PUT(4, 4);
    if (b4) { PUT(4, 4); PUT(4, 0); }
    else PUT(3, 3);
    if (b7) {
        if (b4 && !b6) PUT(3, -1);
        else if (b6 && !b4) PUT(5, 1);
        else { PUT(5, 1); PUT(3, -1); }
    } else if (bit_of(right, 5)) PUT(3, 1);
    else PUT(4, 0);
    if (b6) { PUT(4, 0); PUT(0, 0); }
    else PUT(1, 3);
    if (b5) {
        if (b3 && !b6) PUT(1, -1);
        else if (b6 && !b3) PUT(-1, 1);
        else { PUT(1, -1); PUT(-1, 1); }
    } else if (bit_of(left, 7)) PUT(1, 1);
    else PUT(0, 0);
    if (b3) { PUT(0, 0); PUT(0, 4); }
    else PUT(1, 2);
#undef PUT
    return n;
}

static void qswap(qpt* a, qpt* b) { qpt t = *a; *a = *b; *b = t; }

/* Brings the minimum-y points of P[start..end] to the front of the range
 * (sort_y, diagram_functions.cu:37-80). */
static void front_min_y(qpt* P, int start, int end)
{
    int minor = 1 << 20, tie = 0, idx[ORC_CELL];
    for (int i = start; i <= end; i++) {
        if (P[i].y < minor) { minor = P[i].y; tie = 0; idx[0] = i; }
        else if (P[i].y == minor) idx[++tie] = i;
    }
    for (int t = 0; t <= tie; t++) qswap(&P[start + t], &P[idx[t]]);
}

/* The reference's lexicographic point sort with its tie handling
 * (sort, diagram_functions.cu:83-129): repeatedly gather every point with the
 * minimum remaining x to the front, then order that group by front_min_y. */
static void lex_sort(qpt* P, int n)
{
    int sorted = 0;
    while (sorted < n) {
        int minor = 1 << 20, tie = 0, idx[ORC_CELL];
        for (int i = sorted; i < n; i++) {
            if (P[i].x < minor) { minor = P[i].x; tie = 0; idx[0] = i; }
            else if (P[i].x == minor) idx[++tie] = i;
        }
        for (int t = 0; t <= tie; t++) qswap(&P[sorted + t], &P[idx[t]]);
        if (tie > 0) front_min_y(P, sorted, sorted + tie);
        sorted += tie + 1;
    }
}

static long qcross(qpt o, qpt a, qpt b) { return (long)(a.x - o.x) * (b.y - o.y) - (long)(a.y - o.y) * (b.x - o.x); }

/* Monotone-chain hull (convex_hull, diagram_functions.cu:239-316). The
 * reference's x100 integer cross product is exact on quarter-unit points, so
 * its sign equals qcross's. Returns the vertex count; H holds count+1 points
 * with H[count] == H[0]. */
static int hull(qpt* P, int n, qpt* H)
{
    lex_sort(P, n);
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

/* Reshaped cell polygon of one node, in local float coordinates. Writes n+1
 * points (closing duplicate included) and returns n. */
int orc_cell_polygon(unsigned node, unsigned left, unsigned right, float* xy)
{
    qpt P[ORC_CELL], H[ORC_CELL];
    int np = cell_points(node, left, right, P);
    int k = hull(P, np, H);
    for (int t = 0; t <= k; t++) {
        xy[2 * t] = (float)H[t].x * 0.25f;
        xy[2 * t + 1] = (float)H[t].y * 0.25f;
    }
    return k;
}

/* Cell stage (cells_Kernel, kernel.cu:192-213): row neighbours are read
 * linearly, so the first and last node see the zero guard. */
void orc_cells(const uint8_t* g, int w, int h, float* diagram, int* edge_count)
{
    int n = w * h;
    for (int idx = 0; idx < n; idx++) {
        unsigned left = idx > 0 ? g[idx - 1] : 0;
        unsigned right = idx + 1 < n ? g[idx + 1] : 0;
        float* cell = diagram + (size_t)idx * ORC_CELL * 2;
        memset(cell, 0, ORC_CELL * 2 * sizeof(float));
        edge_count[idx] = orc_cell_polygon(g[idx], left, right, cell);
    }
}

/* Hull table over the 12 pattern bits that decide a cell: node byte (bits
 * 0-7), left bit 2 (bit 8), left bit 7 (bit 9), right bit 0 (bit 10), right
 * bit 5 (bit 11). Each entry: count, then up to 16 points in quarter units. */
void orc_hull_table(int32_t* counts, int8_t* pts /* 4096*16*2 */)
{
    for (int pat = 0; pat < 4096; pat++) {
        unsigned node = pat & 0xFF;
        unsigned left = (bit_of(pat, 8) << 2) | (bit_of(pat, 9) << 7);
        unsigned right = (bit_of(pat, 10) << 0) | (bit_of(pat, 11) << 5);
        qpt P[ORC_CELL], H[ORC_CELL];
        int np = cell_points(node, left, right, P);
        int k = hull(P, np, H);
        counts[pat] = k;
        for (int t = 0; t < 16; t++) {
            pts[(pat * 16 + t) * 2] = (int8_t)(t < k ? H[t].x : 0);
            pts[(pat * 16 + t) * 2 + 1] = (int8_t)(t < k ? H[t].y : 0);
        }
    }
}

/* ----------------------------------------------------------- subdivision */

static inline int pmod(int i, int n) { return (n + (i % n)) % n; }

/* corner-cutting points on edge i -> i+1 (getQ_i / getR_i,
 * subdivision_functions.cu:42-122) */
static opt q_point(int i, const float* c, int n)
{
    int a = i % n;
    if (a < 0) a += n;
    int b = (i + 1) % n;
    float px = c[2 * a], py = c[2 * a + 1], nx = c[2 * b], ny = c[2 * b + 1];
    float len = sqrtf((nx - px) * (nx - px) + (ny - py) * (ny - py));
    opt q;
    if (len <= 1.0) {
        q.x = (float)(px / 2.0 + (px + nx) / 4.0);
        q.y = (float)(py / 2.0 + (py + ny) / 4.0);
    } else {
        q.x = (float)((7.0 * px) / 8.0 + nx / 8.0);
        q.y = (float)((7.0 * py) / 8.0 + ny / 8.0);
    }
    return q;
}

static opt r_point(int i, const float* c, int n)
{
    int a = i % n;
    if (a < 0) a += n;
    int b = (i + 1) % n;
    float px = c[2 * a], py = c[2 * a + 1], nx = c[2 * b], ny = c[2 * b + 1];
    float len = sqrtf((nx - px) * (nx - px) + (ny - py) * (ny - py));
    opt r;
    if (len <= 1.0) {
        r.x = (float)(nx / 2.0 + (px + nx) / 4.0);
        r.y = (float)(ny / 2.0 + (py + ny) / 4.0);
    } else {
        r.x = (float)((1.0 * px) / 8.0 + (7.0 * nx) / 8.0);
        r.y = (float)((1.0 * py) / 8.0 + (7.0 * ny) / 8.0);
    }
    return r;
}

/* Edge-link classification (isLinkedEdge, subdivision_functions.cu:245-424):
 * returns the neighbour direction an edge is shared with, or -1. */
static int edge_link(const float* c, unsigned node, int idx, int n)
{
    int nx = pmod(idx + 1, n);
    float ax = c[2 * idx], ay = c[2 * idx + 1], bx = c[2 * nx], by = c[2 * nx + 1];
    float slope = (by - ay) / (bx - ax);
    float mid_y = (float)((ay + by) / 2.0);
    if (ay == by && ay > 0.5 && bit_of(node, 1)) return 1;
    if (ax == bx && ax > 0.5 && bit_of(node, 4)) return 4;
    if (ay == by && ay < 0.5 && bit_of(node, 6)) return 6;
    if (ax == bx && ax < 0.5 && bit_of(node, 3)) return 3;
    if (slope == 1 && mid_y > 0.5 && bit_of(node, 0)) return 0;
    if (slope == -1 && mid_y > 0.5 && bit_of(node, 2)) return 2;
    if (slope == 1 && mid_y < 0.5 && bit_of(node, 7)) return 7;
    if (slope == -1 && mid_y < 0.5 && bit_of(node, 5)) return 5;
    return -1;
}

/* byte at linear offset off of the reference BGR image, zero outside */
static inline int img_byte(const uint8_t* bgr, long size, long off) { return (off < 0 || off >= size) ? 0 : bgr[off]; }

static int same_color(const uint8_t* bgr, long size, long a, long b)
{
    return img_byte(bgr, size, a) == img_byte(bgr, size, b) && img_byte(bgr, size, a + 1) == img_byte(bgr, size, b + 1) &&
           img_byte(bgr, size, a + 2) == img_byte(bgr, size, b + 2);
}

/* T-junction test at a cell corner (checkTJunction,
 * subdivision_functions.cu:170-242), including its bounds test written with
 * the image width in place of the stride. */
static int t_junction(const uint8_t* bgr, int w, int ws, int h, int i, int j, float px, float py)
{
    long index = (long)j * ws + (long)i * 3;
    long size = (long)h * ws;
    if ((index - ws - 1) < 0 || (index + w + 1) > ((long)h * ws - 1)) return 1;
    long c0 = index + ws - 3, c1 = index + ws, c2 = index + ws + 3, c3 = index - 3, c4 = index + 3;
    long c5 = index - ws - 3, c6 = index - ws, c7 = index - ws + 3;
    if (px == 0.0 && py == 0.0)
        if (!same_color(bgr, size, c3, c5) || !same_color(bgr, size, c5, c6)) return 1;
    if (px == 1.0 && py == 0.0)
        if (!same_color(bgr, size, c4, c7) || !same_color(bgr, size, c7, c6)) return 1;
    if (px == 1.0 && py == 1.0)
        if (!same_color(bgr, size, c1, c2) || !same_color(bgr, size, c2, c4)) return 1;
    if (px == 0.0 && py == 1.0)
        if (!same_color(bgr, size, c0, c1) || !same_color(bgr, size, c1, c3)) return 1;
    return 0;
}

/* the point of a linked neighbour cell matching local point (px,py), then the
 * Q or R point around it mapped back to this cell's coordinates
 * (get{Q,R}_i_from_linked_cell, getOppositePoint{,Coord}, getPointIndex:
 * subdivision_functions.cu:125-154, 427-538) */
static opt linked_point(const float* snap, const int* ec_snap, int w, int node_index, int link, float px, float py,
                        int want_r)
{
    int nb = node_index + DJ[link] * w + DI[link];
    const float* lc = snap + (size_t)nb * ORC_CELL * 2;
    int ln = ec_snap[nb];
    float ox = px - (float)DI[link], oy = py - (float)DJ[link];
    int op = 0;
    for (int t = 0; t < ln; t++)
        if (ox == lc[2 * t] && oy == lc[2 * t + 1]) { op = t; break; }
    opt p = want_r ? r_point(op - 1, lc, ln) : q_point(op, lc, ln);
    p.x = p.x + (float)DI[link];
    p.y = p.y + (float)DJ[link];
    return p;
}

static opt mid(opt a, opt b)
{
    opt m;
    m.x = (float)((a.x + b.x) / 2.0);
    m.y = (float)((a.y + b.y) / 2.0);
    return m;
}

/* One corner-cutting round of a cell (subdivision,
 * subdivision_functions.cu:564-669). Reads the hull snapshot, writes the new
 * polygon into out (up to 2n points) and returns its size. */
static int subdivide_cell(const uint8_t* bgr, int w, int ws, int h, int i, int j, unsigned node, const float* snap,
                          const int* ec_snap, float* out)
{
    int node_index = j * w + i;
    const float* c = snap + (size_t)node_index * ORC_CELL * 2;
    int n = ec_snap[node_index];
    int link[ORC_CELL];
    for (int e = 0; e < n; e++) link[e] = edge_link(c, node, e, n);
    int m = 0;
#define EMIT(P) (out[2 * m] = (P).x, out[2 * m + 1] = (P).y, m++)
    for (int v = 0; v < n; v++) {
        int cur = link[v] >= 0, prev = link[pmod(v - 1, n)] >= 0;
        float px = c[2 * v], py = c[2 * v + 1];
        if (!cur && !prev) {
            if (t_junction(bgr, w, ws, h, i, j, px, py)) {
                opt p = {px, py};
                EMIT(p);
            } else {
                opt q = q_point(v, c, n), r = r_point(v - 1, c, n);
                EMIT(r);
                EMIT(q);
            }
        } else if (!cur && prev) {
            opt q = q_point(v, c, n);
            opt ra = linked_point(snap, ec_snap, w, node_index, link[pmod(v - 1, n)], px, py, 1);
            opt mm = mid(q, ra);
            EMIT(mm);
            EMIT(q);
        } else if (cur && !prev) {
            opt qa = linked_point(snap, ec_snap, w, node_index, link[v], px, py, 0);
            opt r = r_point(v - 1, c, n);
            opt mm = mid(r, qa);
            EMIT(r);
            EMIT(mm);
        } else {
            opt p = {px, py};
            EMIT(p);
        }
    }
#undef EMIT
    return m;
}

/* Subdivision stage (subdivision_Kernel, kernel.cu:216-261): interior nodes
 * (byte 90: four orthogonal links, no diagonal) keep their hull. */
void orc_subdivide(const uint8_t* bgr, int w, int h, int ws, const uint8_t* g, const float* snap, const int* ec_snap,
                   float* diagram, int* edge_count)
{
    for (int j = 0; j < h; j++)
        for (int i = 0; i < w; i++) {
            int idx = j * w + i;
            if (g[idx] == 90) continue;
            float tmp[4 * ORC_CELL];
            int m = subdivide_cell(bgr, w, ws, h, i, j, g[idx], snap, ec_snap, tmp);
            if (m > ORC_CELL) m = ORC_CELL; /* the reference would overrun its cell here */
            memcpy(diagram + (size_t)idx * ORC_CELL * 2, tmp, (size_t)m * 2 * sizeof(float));
            edge_count[idx] = m;
        }
}

/* --------------------------------------------------------- triangulation */

/* signed area (area, triangulate_functions.cu:6-34) */
static float poly_area(const float* c, int n)
{
    float A = 0.0f;
    for (int p = n - 1, q = 0; q < n; p = q++) A += c[2 * p] * c[2 * q + 1] - c[2 * q] * c[2 * p + 1];
    return A * 0.5f;
}

static int inside_tri(float Ax, float Ay, float Bx, float By, float Cx, float Cy, float Px, float Py)
{
    float ax = Cx - Bx, ay = Cy - By, bx = Ax - Cx, by = Ay - Cy, cx = Bx - Ax, cy = By - Ay;
    float apx = Px - Ax, apy = Py - Ay, bpx = Px - Bx, bpy = Py - By, cpx = Px - Cx, cpy = Py - Cy;
    float a_bp = ax * bpy - ay * bpx, c_ap = cx * apy - cy * apx, b_cp = bx * cpy - by * cpx;
    return a_bp >= 0.0f && b_cp >= 0.0f && c_ap >= 0.0f;
}

/* ear test (snip, triangulate_functions.cu:70-105) */
static int is_ear(const float* c, int u, int v, int w, int n, const int* V)
{
    const float EPS = 0.0000000001f;
    float Ax = c[2 * V[u]], Ay = c[2 * V[u] + 1], Bx = c[2 * V[v]], By = c[2 * V[v] + 1];
    float Cx = c[2 * V[w]], Cy = c[2 * V[w] + 1];
    if (EPS > (((Bx - Ax) * (Cy - Ay)) - ((By - Ay) * (Cx - Ax)))) return 0;
    for (int p = 0; p < n; p++) {
        if (p == u || p == v || p == w) continue;
        if (inside_tri(Ax, Ay, Bx, By, Cx, Cy, c[2 * V[p]], c[2 * V[p] + 1])) return 0;
    }
    return 1;
}

/* Ear clipping (process, triangulate_functions.cu:108-217). Writes triangle
 * corner indices into tri (3 per triangle) and returns the triangle count;
 * *ok is 0 when the reference's loop guard gives up. */
int orc_ear_clip(const float* c, int n, int* tri, int* ok)
{
    *ok = 1;
    if (n < 3) { *ok = 0; return 0; }
    int V[ORC_CELL];
    if (0.0f < poly_area(c, n))
        for (int v = 0; v < n; v++) V[v] = v;
    else
        for (int v = 0; v < n; v++) V[v] = (n - 1) - v;
    int nv = n, nt = 0, count = 2 * nv;
    for (int v = nv - 1; nv > 2;) {
        if (0 >= (count--)) { *ok = 0; return nt; }
        int u = v;
        if (nv <= u) u = 0;
        v = u + 1;
        if (nv <= v) v = 0;
        int w = v + 1;
        if (nv <= w) w = 0;
        if (is_ear(c, u, v, w, nv, V)) {
            tri[3 * nt] = V[u];
            tri[3 * nt + 1] = V[v];
            tri[3 * nt + 2] = V[w];
            nt++;
            for (int s = v, t = v + 1; t < nv; s++, t++) V[s] = V[t];
            nv--;
            count = 2 * nv;
        }
    }
    return nt;
}

/* Triangulation + VBO fill (triangulate_polygon,
 * triangulate_functions.cu:220-276; position_kernel / color_kernel,
 * kernel.cu:67-137). pos gets each triangle corner plus the cell offset in
 * the first 3*(count-2) slots and (-100,-100) elsewhere; col gets the pixel's
 * bytes 2,1,0 and alpha 255 in all 45 slots. Slots a failed ear clip leaves
 * unwritten (undefined in the reference) are filled with (-100,-100) here.
 * Returns the number of cells whose ear clip failed. */
int orc_emit(const uint8_t* bgr, int w, int h, int ws, const float* diagram, const int* edge_count, float* pos,
             uint8_t* col)
{
    int fails = 0;
    for (int j = 0; j < h; j++)
        for (int i = 0; i < w; i++) {
            int idx = j * w + i;
            const float* c = diagram + (size_t)idx * ORC_CELL * 2;
            int n = edge_count[idx];
            int tri[3 * ORC_CELL], ok = 1;
            int nt = orc_ear_clip(c, n, tri, &ok);
            if (!ok) fails++;
            int lim = (n - 2) * 3;
            for (int t = 0; t < ORC_CELL; t++) {
                float x = -100.0f, y = -100.0f;
                if (t < lim && t < 3 * nt) {
                    x = c[2 * tri[t]] + (float)i;
                    y = c[2 * tri[t] + 1] + (float)j;
                }
                if (pos) {
                    pos[2 * ((size_t)idx * ORC_CELL + t)] = x;
                    pos[2 * ((size_t)idx * ORC_CELL + t) + 1] = y;
                }
                if (col) {
                    const uint8_t* px = bgr + (size_t)j * ws + 3 * i;
                    uint8_t* o = col + 4 * ((size_t)idx * ORC_CELL + t);
                    o[0] = px[2];
                    o[1] = px[1];
                    o[2] = px[0];
                    o[3] = 255;
                }
            }
        }
    return fails;
}

/* ---------------------------------------------------------------- raster */

/* Headless raster contract (stands in for glDrawArrays(GL_TRIANGLES) over
 * the VBO, simpleVBO.cpp:255-281, no depth test, main.cpp:261):
 *  - output (W*s) x (H*s) RGBA8, row 0 at the bottom (the input's y-up rows);
 *  - output pixel (X,Y) samples the point (X+0.5, Y+0.5) in output pixels;
 *  - vertices are scaled by s and snapped to 1/256 px (round half away from 0);
 *  - a triangle covers a sample when every edge function (CCW orientation)
 *    is > 0, or == 0 on a top or left edge; zero-area triangles cover nothing;
 *  - the covering triangle latest in VBO order wins (painter order);
 *  - uncovered samples are (0,0,0,255), the clear colour.
 * Written as the painter loop itself, triangle by triangle. */
static long snap256(float v, int s) { double d = (double)v * (double)s * 256.0; return (long)(d < 0 ? d - 0.5 : d + 0.5); }

void orc_raster(const float* pos, const uint8_t* col, int w, int h, int s, uint8_t* out)
{
    int ow = w * s, oh = h * s;
    for (long k = 0; k < (long)ow * oh; k++) {
        out[4 * k] = 0;
        out[4 * k + 1] = 0;
        out[4 * k + 2] = 0;
        out[4 * k + 3] = 255;
    }
    long ntri = (long)w * h * (ORC_CELL / 3);
    for (long t = 0; t < ntri; t++) {
        const float* v = pos + 6 * t;
        long ax = snap256(v[0], s), ay = snap256(v[1], s), bx = snap256(v[2], s), by = snap256(v[3], s);
        long cx = snap256(v[4], s), cy = snap256(v[5], s);
        long area = (bx - ax) * (cy - ay) - (by - ay) * (cx - ax);
        if (area == 0) continue;
        if (area < 0) {
            long tx = bx, ty = by;
            bx = cx; by = cy; cx = tx; cy = ty;
        }
        long minx = ax < bx ? ax : bx, maxx = ax > bx ? ax : bx, miny = ay < by ? ay : by, maxy = ay > by ? ay : by;
        if (cx < minx) minx = cx;
        if (cx > maxx) maxx = cx;
        if (cy < miny) miny = cy;
        if (cy > maxy) maxy = cy;
        /* samples at 256*X + 128 */
        long X0 = (minx - 128 + 255) / 256, X1 = (maxx - 128) / 256, Y0 = (miny - 128 + 255) / 256, Y1 = (maxy - 128) / 256;
        if (minx - 128 < 0) X0 = 0;
        if (miny - 128 < 0) Y0 = 0;
        if (X1 >= ow) X1 = ow - 1;
        if (Y1 >= oh) Y1 = oh - 1;
        long ex[3] = {bx - ax, cx - bx, ax - cx}, ey[3] = {by - ay, cy - by, ay - cy};
        long ox[3] = {ax, bx, cx}, oy[3] = {ay, by, cy};
        const uint8_t* cc = col + 12 * t; /* colour of the triangle's first corner */
        for (long Y = Y0; Y <= Y1; Y++)
            for (long X = X0; X <= X1; X++) {
                long sx = 256 * X + 128, sy = 256 * Y + 128;
                int in = 1;
                for (int e = 0; e < 3 && in; e++) {
                    long f = ex[e] * (sy - oy[e]) - ey[e] * (sx - ox[e]);
                    int tl = ey[e] < 0 || (ey[e] == 0 && ex[e] < 0);
                    if (!(f > 0 || (f == 0 && tl))) in = 0;
                }
                if (in) {
                    uint8_t* o = out + 4 * (Y * ow + X);
                    o[0] = cc[0];
                    o[1] = cc[1];
                    o[2] = cc[2];
                    o[3] = cc[3];
                }
            }
    }
}

/* ------------------------------------------------------ component labels */

static int uf_find(int* p, int x)
{
    while (p[x] != x) {
        p[x] = p[p[x]];
        x = p[x];
    }
    return x;
}

/* Connected components of the resolved graph over its set bits (8-way);
 * each node's label is the minimum linear index in its component. (The
 * reference has only a sequential border walk for this, cc_functions.cu:348-503,
 * outside its live build; the label definition is this project's.) */
void orc_label_cc(const uint8_t* g, int w, int h, int32_t* labels)
{
    int n = w * h;
    int* p = (int*)malloc((size_t)n * sizeof(int));
    for (int k = 0; k < n; k++) p[k] = k;
    for (int j = 0; j < h; j++)
        for (int i = 0; i < w; i++)
            for (int e = 0; e < 8; e++) {
                if (!bit_of(g[j * w + i], e)) continue;
                int ni = i + DI[e], nj = j + DJ[e];
                if (ni < 0 || nj < 0 || ni >= w || nj >= h) continue;
                int a = uf_find(p, j * w + i), b = uf_find(p, nj * w + ni);
                if (a < b) p[b] = a;
                else if (b < a) p[a] = b;
            }
    for (int k = 0; k < n; k++) labels[k] = uf_find(p, k);
    free(p);
}

/* ---------------------------------------------------------- border walks */

/* Link order of the border walk (cc_functions.cu:48-100, 127-183): the
 * reference enumerates a node's links clockwise from up-left as clock
 * positions 0..7 and maps them to node bits (getRealLinkIndex) and back
 * (getClockLinkIndex). */
static const int REAL_OF_CLOCK[8] = {0, 1, 2, 4, 7, 6, 5, 3};
static const int CLOCK_OF_REAL[8] = {0, 1, 2, 7, 3, 6, 5, 4};

static int popc8(unsigned v)
{
    int c = 0;
    for (int e = 0; e < 8; e++) c += bit_of(v, e);
    return c;
}

/* getFirstLink (cc_functions.cu:107-119) */
static int first_link(unsigned v)
{
    for (int c = 0; c < 8; c++)
        if (bit_of(v, REAL_OF_CLOCK[c])) return REAL_OF_CLOCK[c];
    return -1;
}

/* nextEdgeCounterClockwise (cc_functions.cu:265-287): the link met first
 * counter-clockwise from e, e itself on a valence-1 node */
static int next_ccw(unsigned v, int e)
{
    if (popc8(v) == 1) return e;
    int c = CLOCK_OF_REAL[e];
    for (int k = c + 7; k >= c + 1; k--)
        if (bit_of(v, REAL_OF_CLOCK[k % 8])) return REAL_OF_CLOCK[k % 8];
    return e;
}

/* the link a walk leaves a node of links v by after arriving along e
 * (nextNodeClockwise, cc_functions.cu:296-318): clockwise from the link back,
 * the link back itself on a valence-1 node (and, not in the reference, on a
 * node without links, which only a malformed graph leads to) */
static int next_cw(unsigned v, int e)
{
    int back = 7 - e;
    if (popc8(v) == 1) return back;
    int c = CLOCK_OF_REAL[back];
    for (int k = c + 1; k <= c + 7; k++)
        if (bit_of(v, REAL_OF_CLOCK[k % 8])) return REAL_OF_CLOCK[k % 8];
    return back;
}

/* Border walks of the graph's components in the form the reference's spline
 * export recorded them (extractBorderPoints, cc_functions.cu:348-503, and
 * its output alex_png.txt). Nodes are taken in scan order; a node that is
 * internal (byte 90) or already listed starts no walk. A walk leaves its
 * start by its first link and turns clockwise at every node until its next
 * move would enter the start again along the link the start's
 * counter-clockwise turn gives; it is recorded (every node listed) unless it
 * enters an internal, listed or discarded node first. A walk that stops
 * there marks its last recorded node discarded and leaves its start
 * unlisted: that is how the recorded file was made (all 21 walks of
 * alex_png.txt follow from it), where the checked-in loop keeps the start
 * listed and would drop walks 4 and 7 of that file. Not in the reference: a
 * node without links is a walk of its own (the reference reads past its
 * link table there), links toward outside the image are ignored, and a walk
 * longer than 8 w h + 8 steps stops as above.
 *
 * Writes walk k's nodes to nodes[offsets[k] .. offsets[k+1]) and the link
 * each leaves by to edges[] (-1 for a node without links); returns the walk
 * count, or -1 when max_nodes or max_walks would be exceeded (outputs up to
 * the last complete walk). *n_nodes gets the nodes written. */
int orc_border_walks(const uint8_t* g, int w, int h, int32_t* nodes, int8_t* edges, int32_t* offsets, int max_nodes,
                     int max_walks, int* n_nodes)
{
    const int n = w * h;
    uint8_t* fl = (uint8_t*)calloc((size_t)n + 1, 1); /* bit 0 listed, bit 1 discarded */
    int nw = 0, pos = 0, trunc = 0;
    const long long limit = 8LL * n + 8;
    offsets[0] = 0;
#define NODE(x, y) (gat(g, w, h, (x), (y)) & inside_bits((x), (y), w, h))
    for (int y = 0; y < h && !trunc; y++)
        for (int x = 0; x < w; x++) {
            const int p = y * w + x;
            const unsigned v0 = NODE(x, y);
            if (v0 == 90 || (fl[p] & 1)) continue;
            if (v0 == 0) {
                if (nw >= max_walks || pos >= max_nodes) {
                    trunc = 1;
                    break;
                }
                nodes[pos] = p;
                edges[pos++] = -1;
                fl[p] |= 1;
                offsets[++nw] = pos;
                continue;
            }
            fl[p] |= 1;
            int e = first_link(v0);
            const int arr = next_ccw(v0, e);
            const int start = pos;
            int over = 0, last = p; // over: a node did not fit (the walk is then not recorded)
            if (pos < max_nodes) {
                nodes[pos] = p;
                edges[pos++] = (int8_t)e;
            } else {
                over = 1;
            }
            int cx = x, cy = y, ok = 1;
            long long steps = 0;
            while (!(cx + DI[e] == x && cy + DJ[e] == y && 7 - e == arr)) {
                cx += DI[e];
                cy += DJ[e];
                const int cp = cy * w + cx;
                const unsigned v = NODE(cx, cy);
                e = next_cw(v, e);
                if (v == 90 || fl[cp] || ++steps > limit) {
                    fl[last] |= 2;
                    fl[p] &= (uint8_t)~1u;
                    pos = start;
                    ok = 0;
                    break;
                }
                last = cp;
                if (pos < max_nodes) {
                    nodes[pos] = cp;
                    edges[pos++] = (int8_t)e;
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
                for (int q = start; q < pos; q++) fl[nodes[q]] |= 1;
                offsets[++nw] = pos;
            }
        }
#undef NODE
    free(fl);
    *n_nodes = pos;
    return trunc ? -1 : nw;
}

/* ------------------------------------------------------------ whole frame */

/* Runs the whole path on one BGR frame with the same outputs as the
 * reference driver (kernel.cu:286-526). Any output may be NULL. Returns the
 * number of cells whose ear clip failed. */
int orc_frame(const uint8_t* bgr, int w, int h, int ws, int subdivide, int tr_y, int tr_u, int tr_v, int mode,
              const uint8_t* graph_in, uint8_t* graph_trivial_out, uint8_t* graph_resolved_out, int* ec_cells_out,
              float* diag_cells_out, int* ec_final_out, float* diag_final_out, float* pos_out, uint8_t* col_out)
{
    int n = w * h;
    uint8_t* g0 = (uint8_t*)malloc(n);
    uint8_t* g1 = (uint8_t*)malloc(n);
    if (graph_in) {
        memcpy(g0, graph_in, n);
        memcpy(g1, graph_in, n);
    } else {
        orc_graph(bgr, w, h, ws, tr_y, tr_u, tr_v, mode, g0);
        orc_trivial(g0, w, h);
        orc_heuristics(g0, w, h, g1);
    }
    if (graph_trivial_out) memcpy(graph_trivial_out, g0, n);
    if (graph_resolved_out) memcpy(graph_resolved_out, g1, n);
    float* diag = (float*)malloc((size_t)n * ORC_CELL * 2 * sizeof(float));
    int* ec = (int*)malloc((size_t)n * sizeof(int));
    orc_cells(g1, w, h, diag, ec);
    if (ec_cells_out) memcpy(ec_cells_out, ec, (size_t)n * sizeof(int));
    if (diag_cells_out) memcpy(diag_cells_out, diag, (size_t)n * ORC_CELL * 2 * sizeof(float));
    if (subdivide) {
        float* snap = (float*)malloc((size_t)n * ORC_CELL * 2 * sizeof(float));
        int* ec_snap = (int*)malloc((size_t)n * sizeof(int));
        memcpy(snap, diag, (size_t)n * ORC_CELL * 2 * sizeof(float));
        memcpy(ec_snap, ec, (size_t)n * sizeof(int));
        orc_subdivide(bgr, w, h, ws, g1, snap, ec_snap, diag, ec);
        free(snap);
        free(ec_snap);
    }
    if (ec_final_out) memcpy(ec_final_out, ec, (size_t)n * sizeof(int));
    if (diag_final_out) memcpy(diag_final_out, diag, (size_t)n * ORC_CELL * 2 * sizeof(float));
    int fails = orc_emit(bgr, w, h, ws, diag, ec, pos_out, col_out);
    free(diag);
    free(ec);
    free(g0);
    free(g1);
    return fails;
}
