"""The edge-deferral rule of the component labelling (csrc/depix_graph.cu,
join_masks) restated on the CPU and checked against brute-force components
on random symmetric graphs, crossing diagonals included:
  - inside a 64x16 tile: parents start at each pixel's run start, then one
    union per kept edge between rows r and r + 1 (cc_sym_unions);
  - across tiles: the kept edges between row y0 + 15 and y0 + 16 and between
    columns x0 + 63 and x0 + 64 of every tile (merge_tile_borders), on top of
    exact tile-local components.
Line masks are Python ints of 64 bits; edge e joins r[c] and q[c + e - 1]."""
import numpy as np
import pytest

DI = [-1, 0, 1, -1, 1, -1, 0, 1]  # neighbour x offset of edge bit e
DJ = [1, 1, 1, 0, 0, -1, -1, -1]  # neighbour y offset of edge bit e
TW, TH = 64, 16
M64 = (1 << 64) - 1


def join_masks(Sr, Sq, E0, E1, E2, q_end):
    nSr, nSq = ~Sr & M64, ~Sq & M64
    n0 = E0 & ~(nSr & ((((E0 & nSq) << 1) | (E1 << 1)) & M64)) & M64
    n1 = E1 & ~(((E1 << 1) & M64) & nSr & nSq) & M64
    n2 = E2 & ~((((E2 << 1) & M64) & nSr & (~((Sq >> 1) | q_end) & M64)) | ((E1 & nSr) >> 1)) & M64
    return n0, n1, n2


def run_start(S, c):
    return (S & ((1 << (c + 1)) - 1)).bit_length() - 1


class UF:
    def __init__(self, n):
        self.p = list(range(n))

    def find(self, x):
        while self.p[x] != x:
            self.p[x] = self.p[self.p[x]]
            x = self.p[x]
        return x

    def unite(self, a, b):
        a, b = self.find(a), self.find(b)
        if a != b:
            self.p[max(a, b)] = min(a, b)


def random_symmetric(rng, w, h, density):
    g = np.zeros((h, w), np.int64)
    for y in range(h):
        for x in range(w):
            for e in (0, 1, 2, 4):
                nx, ny = x + DI[e], y + DJ[e]
                if 0 <= nx < w and 0 <= ny < h and rng.random() < density:
                    g[y, x] |= 1 << e
                    g[ny, nx] |= 1 << (7 - e)
    return g


def brute(g, keep):
    """Components of the edges (x, y) -> neighbour for which keep(...) holds."""
    h, w = g.shape
    uf = UF(w * h)
    for y in range(h):
        for x in range(w):
            for e in range(8):
                nx, ny = x + DI[e], y + DJ[e]
                if g[y, x] >> e & 1 and 0 <= nx < w and 0 <= ny < h and keep(x, y, nx, ny):
                    uf.unite(y * w + x, ny * w + nx)
    return [uf.find(k) for k in range(w * h)]


def bits(line, f):
    return sum(1 << c for c in range(len(line)) if f(c, int(line[c])))


def tile_labels(t):
    """cc_sym_unions on one 64x16 tile t (rows as y)."""
    uf = UF(TW * TH)
    for r in range(TH):
        S = bits(t[r], lambda c, v: c == 0 or not v >> 3 & 1)
        for c in range(TW):
            uf.p[r * TW + c] = r * TW + run_start(S, c)
    unions = 0
    for r in range(TH - 1):
        a, b = t[r], t[r + 1]
        Sr = bits(a, lambda c, v: c == 0 or not v >> 3 & 1)
        Sq = bits(b, lambda c, v: c == 0 or not v >> 3 & 1)
        E = [bits(a, lambda c, v, e=e: v >> e & 1) for e in range(3)]
        need = join_masks(Sr, Sq, E[0] & ~1, E[1], E[2] & ~(1 << 63), 1 << 63)
        for e in range(3):
            for c in range(TW):
                if need[e] >> c & 1:
                    uf.unite(r * TW + run_start(Sr, c), (r + 1) * TW + run_start(Sq, c + e - 1))
                    unions += 1
    return [uf.find(k) for k in range(TW * TH)], unions


@pytest.mark.parametrize("density", [0.15, 0.4, 0.7, 0.95])
def test_tile_unions_give_the_tile_components(density):
    rng = np.random.default_rng(int(density * 100))
    for _ in range(3):
        t = random_symmetric(rng, TW, TH, density)
        got, unions = tile_labels(t)
        assert got == brute(t, lambda *_: True)
        edges = int(sum(bin(int(v)).count("1") for v in t.reshape(-1)))
        assert unions < edges  # the rule drops edges between runs already joined


def test_tile_unions_on_uniform_regions_are_one_per_row_pair():
    t = random_symmetric(np.random.default_rng(0), TW, TH, 1.0)
    got, unions = tile_labels(t)
    assert len(set(got)) == 1 and unions == TH - 1


def frame_labels(g):
    """Exact tile-local components, then merge_tile_borders on every tile."""
    h, w = g.shape
    same_tile = lambda x, y, nx, ny: x // TW == nx // TW and y // TH == ny // TH
    local = brute(g, same_tile)
    uf = UF(w * h)
    for k in range(w * h):
        uf.p[k] = local[k]
    at = lambda x, y: int(g[y, x]) if 0 <= x < w and 0 <= y < h else 0
    for ty in range((h + TH - 1) // TH):
        for tx in range((w + TW - 1) // TW):
            x0, y0 = tx * TW, ty * TH
            yr, yq = y0 + TH - 1, y0 + TH
            if yq < h:
                a = [at(x0 + c, yr) for c in range(TW)]
                b = [at(x0 + c, yq) for c in range(TW)]
                Sr = bits(a, lambda c, v: c == 0 or not v >> 3 & 1)
                Sq = bits(b, lambda c, v: c == 0 or not v >> 3 & 1)
                E = [bits(a, lambda c, v, e=e: v >> e & 1) for e in range(3)]
                need = join_masks(Sr, Sq, E[0], E[1], E[2], 1 << 63)
                for e in range(3):
                    for c in range(TW):
                        if need[e] >> c & 1:
                            nc = c + e - 1
                            qc = nc if nc < 0 or nc >= TW else run_start(Sq, nc)
                            uf.unite(yr * w + x0 + run_start(Sr, c), yq * w + x0 + qc)
            xr, xq = x0 + TW - 1, x0 + TW
            if xq < w:
                a = [at(xr, y0 + y) if y < TH else 0 for y in range(32)]
                b = [at(xq, y0 + y) if y < TH else 0 for y in range(32)]
                Sr = ~(bits(a, lambda y, v: v >> 1 & 1) << 1) & M64
                Sq = ~(bits(b, lambda y, v: v >> 1 & 1) << 1) & M64
                E1 = bits(a, lambda y, v: v >> 4 & 1)
                E2 = bits(a, lambda y, v: v >> 2 & 1) & 0x7FFF
                E0 = (bits(b, lambda y, v: v & 1) & 0x7FFF) << 1
                need = join_masks(Sr, Sq, E0, E1, E2, 1 << 63)
                for e in range(3):
                    for c in range(64):
                        if need[e] >> c & 1:
                            uf.unite((y0 + run_start(Sr, c)) * w + xr, (y0 + run_start(Sq, c + e - 1)) * w + xq)
    return [uf.find(k) for k in range(w * h)]


@pytest.mark.parametrize("w,h,density", [(130, 40, 0.3), (200, 35, 0.8), (70, 50, 0.95)])
def test_border_unions_give_the_frame_components(w, h, density):
    g = random_symmetric(np.random.default_rng(w + h), w, h, density)
    assert frame_labels(g) == brute(g, lambda *_: True)
