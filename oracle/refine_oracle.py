"""CPU specification of the spline refinement stage, in float64 numpy.
TEST INFRASTRUCTURE ONLY: imported by tests/ and by bench.py's CPU legs,
never by the product library.

The reference has no refinement stage (its frame path ends at the VBO fill,
kernel.cu:439-520), so nothing upstream pins this module: it is the
definition that the CUDA stage is checked against, and its gradient is
checked against float64 central differences of its own energy.

Topology (frozen for the whole optimisation):
  * the reshaped cells are the hulls of the resolved graph's cell patterns
    (createCellFromPattern + convex_hull, diagram_functions.cu:239-520; the
    oracle's pattern table); they tile the frame exactly once every hull
    edge is split at the hull vertices lying inside it;
  * a split edge is a curve edge when the cell on its other side is a
    dissimilar 8-neighbour (raw similarity bit clear); it is kept once, from
    the lower-indexed cell, oriented along that cell's counter-clockwise
    hull (its colour on the left, the other cell's on the right);
  * nodes are the vertices of curve edges, in global quarter-pixel units;
    a node is pinned when it is not of degree 2, when it lies on an edge
    without a twin (the frame), or when its two edges turn by 90 degrees or
    more (a corner);
  * one Chaikin round (points at 1/4 and 3/4 of each edge) gives the curve
    segments: the middle of every edge, the cut corner of every free node,
    and the piece from a pinned node to the first cut point of each of its
    edges;
  * every output sample (x s) within 1.5 output pixels of a segment at the
    start is assigned to the nearest one (exact integer distances, ties to
    the lower segment slot).

Energy of node positions P (source pixels), every term a mean:
  E = w_curv * C + w_dev * D + w_cov * V
  C = 1/F * sum_free 1/8 |P[a] - 2 P[p] + P[b]|^2
  D = 1/F * sum_free |P[p] - P0[p]|^2
  V = 1/(3 Ws Hs) * sum_samples sum_rgb ((r - t) / 255)^2
  F the number of free nodes, Ws x Hs the output raster; r = cR + (cL - cR) *
  Phi(d / sigma_src), d the signed distance of the sample from its segment's
  line (positive on the left), sigma_src = sigma / s; t the nearest-neighbour
  x s image under the same Gaussian coverage (each source pixel's square
  blurred by sigma_src), so that a boundary lying on a pixel edge costs
  nothing. Samples farther than 1.5 output pixels from every curve add a
  constant that does not depend on P and are left out. The curvature term is
  the sum of the squared second differences of the two Chaikin points next
  to a free node (both equal (P[a] - 2 P[p] + P[b]) / 4).
"""
from __future__ import annotations

from dataclasses import dataclass
from math import gcd

import numpy as np

import oracle as O

DI = [-1, 0, 1, -1, 1, -1, 0, 1]  # neighbour direction of graph bit e
DJ = [1, 1, 1, 0, 0, -1, -1, -1]
BAND = 48        # 1.5 output pixels in units of 1/(32 s) source pixel
# segment types
SEG_NONE, SEG_MID, SEG_PIN_U, SEG_PIN_V, SEG_CORNER = 0, 1, 2, 3, 4


@dataclass
class Topology:
    w: int
    h: int
    scale: int
    qx: np.ndarray       # nodes: global quarter-pixel coordinates
    qy: np.ndarray
    flags: np.ndarray    # bit 0 pinned, bit 1 frame, bit 2 corner; degree in bits 4-7
    nbr: np.ndarray      # (N, 2) neighbours of degree-2 nodes (ascending), -1 otherwise
    eu: np.ndarray       # edges: endpoints and the cells on their left / right
    ev: np.ndarray
    ecell: np.ndarray    # (E, 2)
    seg_type: np.ndarray  # slots 3e..3e+2 per edge, then 3E + node
    seg_nodes: np.ndarray  # (S, 3), -1 unused
    seg_a: np.ndarray    # (S, 3) weights x4 of A and B over seg_nodes
    seg_b: np.ndarray
    seg_col: np.ndarray  # (S, 2, 3) left / right RGB
    samp_idx: np.ndarray  # assigned output samples (linear, row 0 at the bottom)
    samp_seg: np.ndarray

    @property
    def free(self):
        return (self.flags & 1) == 0


def cell_hulls(graph, w, h):
    """Per cell: hull vertex count and local quarter-unit vertices (CCW)."""
    counts, pts = O.hull_table()
    g = graph.astype(np.int64)
    left = np.concatenate([[0], g[:-1]])
    right = np.concatenate([g[1:], [0]])
    pat = g | ((left >> 2) & 1) << 8 | ((left >> 7) & 1) << 9 | (right & 1) << 10 | ((right >> 5) & 1) << 11
    return counts[pat], pts[pat].astype(np.int64)


def topology(img, graph, raw_graph, scale=4) -> Topology:
    """img: (h, w, 4) RGBA8 (row 0 at the bottom); graph: resolved; raw_graph:
    the similarity graph before any resolution."""
    h, w = img.shape[:2]
    cnt, pts = cell_hulls(graph, w, h)
    n = w * h
    hull = []
    verts = set()
    for idx in range(n):
        i, j = idx % w, idx // w
        P = [(4 * i + int(pts[idx, t, 0]), 4 * j + int(pts[idx, t, 1])) for t in range(cnt[idx])]
        hull.append(P)
        verts.update(P)

    def sub_edges(a, b):
        dx, dy = b[0] - a[0], b[1] - a[1]
        g = gcd(abs(dx), abs(dy))
        out = [a]
        for t in range(1, g):
            p = (a[0] + dx * t // g, a[1] + dy * t // g)
            if p in verts:
                out.append(p)
        out.append(b)
        return list(zip(out[:-1], out[1:]))

    def on_edge(p, q, u, v):
        # v -> u lies on p -> q, same direction
        ex, ey = q[0] - p[0], q[1] - p[1]
        if ex * (v[1] - p[1]) - ey * (v[0] - p[0]) or ex * (u[1] - p[1]) - ey * (u[0] - p[0]):
            return False
        if ex * (u[0] - v[0]) + ey * (u[1] - v[1]) <= 0:
            return False
        L = ex * ex + ey * ey
        tv = ex * (v[0] - p[0]) + ey * (v[1] - p[1])
        tu = ex * (u[0] - p[0]) + ey * (u[1] - p[1])
        return 0 <= tv and tu <= L

    edges = []  # (u, v, A, B)
    frame_v = set()
    for idx in range(n):
        i, j = idx % w, idx // w
        P = hull[idx]
        k = len(P)
        for t in range(k):
            for u, v in sub_edges(P[t], P[(t + 1) % k]):
                owner = -1
                for e in range(8):
                    ni, nj = i + DI[e], j + DJ[e]
                    if not (0 <= ni < w and 0 <= nj < h):
                        continue
                    Q = hull[nj * w + ni]
                    if any(on_edge(Q[s], Q[(s + 1) % len(Q)], u, v) for s in range(len(Q))):
                        owner = e
                        break
                if owner < 0:
                    frame_v.add(u)
                    frame_v.add(v)
                    continue
                B = (j + DJ[owner]) * w + (i + DI[owner])
                if B > idx and not (int(raw_graph[idx]) >> owner) & 1:
                    edges.append((u, v, idx, B))

    W4 = 4 * w + 3
    key = lambda p: (p[1] + 1) * W4 + (p[0] + 1)
    nodes = sorted({p for e in edges for p in e[:2]}, key=key)
    nid = {p: k for k, p in enumerate(nodes)}
    N = len(nodes)
    adj = [[] for _ in range(N)]
    for u, v, _, _ in edges:
        adj[nid[u]].append(nid[v])
        adj[nid[v]].append(nid[u])
    qx = np.array([p[0] for p in nodes], np.int64)
    qy = np.array([p[1] for p in nodes], np.int64)
    flags = np.zeros(N, np.int64)
    nbr = -np.ones((N, 2), np.int64)
    for k in range(N):
        deg = len(adj[k])
        f = min(deg, 15) << 4
        if nodes[k] in frame_v:
            f |= 2
        if deg == 2:
            a, b = sorted(adj[k])
            nbr[k] = (a, b)
            if (qx[k] - qx[a]) * (qx[b] - qx[k]) + (qy[k] - qy[a]) * (qy[b] - qy[k]) <= 0:
                f |= 4
        if deg != 2 or f & 6:
            f |= 1
        flags[k] = f

    E = len(edges)
    eu = np.array([nid[e[0]] for e in edges], np.int64)
    ev = np.array([nid[e[1]] for e in edges], np.int64)
    ecell = np.array([(e[2], e[3]) for e in edges], np.int64).reshape(-1, 2)
    rgb = img[..., :3].reshape(-1, 3).astype(np.int64)
    S = 3 * E + N
    st = np.zeros(S, np.int64)
    sn = -np.ones((S, 3), np.int64)
    sa = np.zeros((S, 3), np.int64)
    sb = np.zeros((S, 3), np.int64)
    sc = np.zeros((S, 2, 3), np.int64)
    pinned = (flags & 1) == 1
    for e in range(E):
        u, v = eu[e], ev[e]
        col = (rgb[ecell[e, 0]], rgb[ecell[e, 1]])
        for slot, typ, wa, wb in ((0, SEG_PIN_U, (4, 0), (3, 1)), (1, SEG_MID, (3, 1), (1, 3)),
                                  (2, SEG_PIN_V, (1, 3), (0, 4))):
            if typ == SEG_PIN_U and not pinned[u] or typ == SEG_PIN_V and not pinned[v]:
                continue
            s = 3 * e + slot
            st[s], sn[s, :2], sa[s, :2], sb[s, :2] = typ, (u, v), wa, wb
            sc[s] = col
    edge_of = {}
    for e in range(E):
        edge_of[(eu[e], ev[e])] = (e, False)
        edge_of[(ev[e], eu[e])] = (e, True)
    for p in range(N):
        if pinned[p]:
            continue
        a, b = nbr[p]
        e, flip = edge_of[(a, p)]
        s = 3 * E + p
        st[s], sn[s], sa[s], sb[s] = SEG_CORNER, (a, p, b), (1, 3, 0), (0, 3, 1)
        cl, cr = rgb[ecell[e, 0]], rgb[ecell[e, 1]]
        sc[s] = (cr, cl) if flip else (cl, cr)

    samp_idx, samp_seg = assign_samples(w, h, scale, qx, qy, st, sn, sa, sb)
    return Topology(w, h, scale, qx, qy, flags, nbr, eu, ev, ecell, st, sn, sa, sb, sc, samp_idx, samp_seg)


def seg_ends_units(top_qx, top_qy, sn, sa, sb, scale):
    """Initial segment ends in units of 1/(32 s) source pixel (exact)."""
    nodes = np.where(sn < 0, 0, sn)
    qx, qy = top_qx[nodes], top_qy[nodes]
    k = 2 * scale  # quarter * 8 s = units; weights are x4
    ax = (sa * qx).sum(1) * k
    ay = (sa * qy).sum(1) * k
    bx = (sb * qx).sum(1) * k
    by = (sb * qy).sum(1) * k
    return ax, ay, bx, by


def assign_samples(w, h, scale, qx, qy, st, sn, sa, sb):
    """Nearest segment per output sample within BAND, exact integer squared
    distances divided once in float64; ties to the lower slot."""
    ax, ay, bx, by = seg_ends_units(qx, qy, sn, sa, sb, scale)
    ow, oh = w * scale, h * scale
    best = np.full(ow * oh, np.inf)
    bseg = np.full(ow * oh, -1, np.int64)
    for s in np.nonzero(st)[0]:
        lo_x = min(ax[s], bx[s]) - BAND
        hi_x = max(ax[s], bx[s]) + BAND
        lo_y = min(ay[s], by[s]) - BAND
        hi_y = max(ay[s], by[s]) + BAND
        # sample X at 16 (2 Xo + 1) units
        x0 = max(0, -(-(lo_x - 16) // 32))
        x1 = min(ow - 1, (hi_x - 16) // 32)
        y0 = max(0, -(-(lo_y - 16) // 32))
        y1 = min(oh - 1, (hi_y - 16) // 32)
        if x0 > x1 or y0 > y1:
            continue
        X = 16 * (2 * np.arange(x0, x1 + 1) + 1)
        Y = 16 * (2 * np.arange(y0, y1 + 1) + 1)
        XX, YY = np.meshgrid(X, Y)
        d2 = seg_dist2(ax[s], ay[s], bx[s], by[s], XX, YY)
        idx = (np.arange(y0, y1 + 1)[:, None] * ow + np.arange(x0, x1 + 1)[None, :])
        m = d2 <= BAND * BAND
        better = m & (d2 < best[idx])  # slots visited in ascending order: ties keep the lower
        best[idx[better]] = d2[better]
        bseg[idx[better]] = s
    sel = np.nonzero(bseg >= 0)[0]
    return sel, bseg[sel]


def seg_dist2(ax, ay, bx, by, X, Y):
    ex, ey = bx - ax, by - ay
    wx, wy = X - ax, Y - ay
    L = ex * ex + ey * ey
    dot = ex * wx + ey * wy
    cr = ex * wy - ey * wx
    with np.errstate(divide="ignore", invalid="ignore"):
        mid = (cr * cr).astype(np.float64) / np.float64(L)
    d_a = (wx * wx + wy * wy).astype(np.float64)
    d_b = ((X - bx) ** 2 + (Y - by) ** 2).astype(np.float64)
    return np.where(dot <= 0, d_a, np.where(dot >= L, d_b, mid))


# -------------------------------------------------------------- warm start

WARM_TILE = 16


def tile_signatures(img, graph):
    """FNV-1a (64-bit) per 16x16 tile over the resolved graph byte and the
    RGB of each pixel of the tile and its one-pixel ring, row-major, pixels
    outside the frame skipped."""
    h, w = img.shape[:2]
    tx, ty = -(-w // WARM_TILE), -(-h // WARM_TILE)
    g = graph.reshape(h, w)
    out = []
    for t in range(tx * ty):
        x0, y0 = (t % tx) * WARM_TILE - 1, (t // tx) * WARM_TILE - 1
        hsh = 0xCBF29CE484222325
        for y in range(max(y0, 0), min(y0 + WARM_TILE + 2, h)):
            for x in range(max(x0, 0), min(x0 + WARM_TILE + 2, w)):
                for byte in (int(g[y, x]), int(img[y, x, 0]), int(img[y, x, 1]), int(img[y, x, 2])):
                    hsh = ((hsh ^ byte) * 0x100000001B3) & 0xFFFFFFFFFFFFFFFF
        out.append(hsh)
    return out, tx


def warm_positions(top, sig, prev_top, prev_sig, prev_pos, tiles_x):
    """Start positions of `top` warm-started from the previous frame: a node
    in a tile whose signature is unchanged takes the previous position of the
    node at the same quarter coordinates, if there is one."""
    prev = {(int(x), int(y)): k for k, (x, y) in enumerate(zip(prev_top.qx, prev_top.qy))}
    P = initial_positions(top)
    for k, (x, y) in enumerate(zip(top.qx, top.qy)):
        px = min(max(int(x) >> 2, 0), top.w - 1)
        py = min(max(int(y) >> 2, 0), top.h - 1)
        t = (py // WARM_TILE) * tiles_x + px // WARM_TILE
        j = prev.get((int(x), int(y)))
        if sig[t] == prev_sig[t] and j is not None:
            P[k] = prev_pos[j]
    return P


# ------------------------------------------------------------------ energy


def initial_positions(top: Topology):
    return np.stack([top.qx, top.qy], 1).astype(np.float64) / 4.0


def _phi(z):
    from scipy.special import erf
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0)))


def energy_grad(top: Topology, P, P0, img, w_curv=1.0, w_dev=0.25, w_cov=1.0, sigma=0.5, want_grad=True):
    """(C, D, V) weighted, their total and dE/dP (float64)."""
    free = np.nonzero(top.free)[0]
    F = max(len(free), 1)
    G = np.zeros_like(P)
    a, b = top.nbr[free, 0], top.nbr[free, 1]
    t = P[a] - 2 * P[free] + P[b]
    e_curv = w_curv * 0.125 * float((t * t).sum()) / F
    dv = P[free] - P0[free]
    e_dev = w_dev * float((dv * dv).sum()) / F
    if want_grad:
        gt = (w_curv * 0.25 / F) * t  # dE/dt
        np.add.at(G, a, gt)
        np.add.at(G, b, gt)
        np.add.at(G, free, -2 * gt)
        G[free] += (2 * w_dev / F) * dv
    # coverage
    s = top.scale
    sig = sigma / s
    norm = w_cov / (3.0 * top.w * s * top.h * s)
    seg = top.samp_seg
    nodes = top.seg_nodes[seg]
    nz = np.where(nodes < 0, 0, nodes)
    wa = top.seg_a[seg] / 4.0
    wb = top.seg_b[seg] / 4.0
    A = (wa[..., None] * P[nz]).sum(1)
    B = (wb[..., None] * P[nz]).sum(1)
    ow = top.w * s
    Xo, Yo = top.samp_idx % ow, top.samp_idx // ow
    X = np.stack([(Xo + 0.5) / s, (Yo + 0.5) / s], 1)
    e = B - A
    wv = X - A
    L = np.sqrt((e * e).sum(1))
    cr = e[:, 0] * wv[:, 1] - e[:, 1] * wv[:, 0]
    d = cr / L
    z = d / sig
    Phi = _phi(z)
    cl = top.seg_col[seg, 0].astype(np.float64)
    crr = top.seg_col[seg, 1].astype(np.float64)
    tgt = soft_target(img, s, sig, Xo, Yo)
    r = crr + (cl - crr) * Phi[:, None]
    res = (r - tgt) / 255.0
    e_cov = norm * float((res * res).sum())
    if want_grad:
        dEdr = 2 * norm * res / 255.0
        phi = np.exp(-0.5 * z * z) / (sig * np.sqrt(2 * np.pi))
        dEdd = (dEdr * (cl - crr)).sum(1) * phi
        # d d / d e and d d / d w
        dde = np.stack([wv[:, 1], -wv[:, 0]], 1) / L[:, None] - (d / (L * L))[:, None] * e
        ddw = np.stack([-e[:, 1], e[:, 0]], 1) / L[:, None]
        gB = dEdd[:, None] * dde
        gA = dEdd[:, None] * (-dde - ddw)
        for k in range(3):
            m = nodes[:, k] >= 0
            contrib = wa[m, k][:, None] * gA[m] + wb[m, k][:, None] * gB[m]
            np.add.at(G, nodes[m, k], contrib)
        G[~top.free] = 0.0
    parts = (e_curv, e_dev, e_cov)
    return parts, sum(parts), (G if want_grad else None)


def soft_target(img, s, sig, Xo, Yo):
    """The nearest-neighbour x s image under the same Gaussian coverage: each
    source pixel's unit square blurred by sigma_src, sampled at the output
    sample (separable; pixels more than 1 away contribute < Phi(-8))."""
    h, w = img.shape[:2]
    rgb = img[..., :3].astype(np.float64)
    x = (Xo + 0.5) / s
    y = (Yo + 0.5) / s
    ix, iy = Xo // s, Yo // s
    out = np.zeros((len(Xo), 3))
    for dj in (-1, 0, 1):
        jj = iy + dj
        cy = _phi((y - jj) / sig) - _phi((y - jj - 1) / sig)
        for di in (-1, 0, 1):
            ii = ix + di
            cx = _phi((x - ii) / sig) - _phi((x - ii - 1) / sig)
            ok = (ii >= 0) & (ii < w) & (jj >= 0) & (jj < h)
            c = rgb[np.clip(jj, 0, h - 1), np.clip(ii, 0, w - 1)]
            out += np.where(ok, cx * cy, 0.0)[:, None] * c
    return out


def central_differences(top, P, P0, img, nodes, h=1e-4, **kw):
    """float64 central differences of the total energy at the given nodes."""
    out = np.zeros((len(nodes), 2))
    for k, p in enumerate(nodes):
        for c in range(2):
            Pp = P.copy()
            Pp[p, c] += h
            Pm = P.copy()
            Pm[p, c] -= h
            out[k, c] = (energy_grad(top, Pp, P0, img, want_grad=False, **kw)[1] -
                         energy_grad(top, Pm, P0, img, want_grad=False, **kw)[1]) / (2 * h)
    return out


def _local_energy(top, P, P0, img, curv_free, samples, dev_node, w_curv, w_dev, w_cov, sigma, tgt):
    """The energy terms of energy_grad restricted to the curvature terms of
    the free nodes curv_free, the deviation term of dev_node (or none) and the
    coverage terms of the given samples, with the same normalisations."""
    F = max(int(top.free.sum()), 1)
    a, b = top.nbr[curv_free, 0], top.nbr[curv_free, 1]
    t = P[a] - 2 * P[curv_free] + P[b]
    e = w_curv * 0.125 * float((t * t).sum()) / F
    if dev_node is not None:
        dv = P[dev_node] - P0[dev_node]
        e += w_dev * float((dv * dv).sum()) / F
    s = top.scale
    sig = sigma / s
    norm = w_cov / (3.0 * top.w * s * top.h * s)
    seg = top.samp_seg[samples]
    nodes = top.seg_nodes[seg]
    nz = np.where(nodes < 0, 0, nodes)
    A = ((top.seg_a[seg] / 4.0)[..., None] * P[nz]).sum(1)
    B = ((top.seg_b[seg] / 4.0)[..., None] * P[nz]).sum(1)
    ow = top.w * s
    Xo, Yo = top.samp_idx[samples] % ow, top.samp_idx[samples] // ow
    X = np.stack([(Xo + 0.5) / s, (Yo + 0.5) / s], 1)
    ed = B - A
    wv = X - A
    d = (ed[:, 0] * wv[:, 1] - ed[:, 1] * wv[:, 0]) / np.sqrt((ed * ed).sum(1))
    Phi = _phi(d / sig)
    cl = top.seg_col[seg, 0].astype(np.float64)
    cr = top.seg_col[seg, 1].astype(np.float64)
    res = (cr + (cl - cr) * Phi[:, None] - tgt) / 255.0
    return e + norm * float((res * res).sum())


def central_differences_local(top, P, P0, img, nodes, h=1e-4, w_curv=1.0, w_dev=0.25, w_cov=1.0, sigma=0.5):
    """float64 central differences of the total energy at the given nodes,
    each from only the energy terms that depend on the node: the curvature
    terms of the free nodes whose stencil holds it, its own deviation term
    and the coverage terms of the samples whose segment it shapes. Every
    other term of E(P + h) - E(P - h) is the same in both evaluations and
    cancels exactly, so this equals central_differences up to rounding, at
    a cost independent of the frame's size."""
    free = np.nonzero(top.free)[0]
    is_free = top.free.astype(bool)
    samp_nodes = top.seg_nodes[top.samp_seg]
    s = top.scale
    ow = top.w * s
    out = np.zeros((len(nodes), 2))
    kw = dict(w_curv=w_curv, w_dev=w_dev, w_cov=w_cov, sigma=sigma)
    for k, p in enumerate(nodes):
        curv = free[(free == p) | (top.nbr[free, 0] == p) | (top.nbr[free, 1] == p)]
        samples = np.nonzero((samp_nodes == p).any(1))[0]
        Xo, Yo = top.samp_idx[samples] % ow, top.samp_idx[samples] // ow
        tgt = soft_target(img, s, sigma / s, Xo, Yo)
        dev = p if is_free[p] else None
        for c in range(2):
            Pp = P.copy()
            Pp[p, c] += h
            Pm = P.copy()
            Pm[p, c] -= h
            out[k, c] = (_local_energy(top, Pp, P0, img, curv, samples, dev, tgt=tgt, **kw) -
                         _local_energy(top, Pm, P0, img, curv, samples, dev, tgt=tgt, **kw)) / (2 * h)
    return out


def adam(top, img, steps=200, lr=0.05, beta1=0.9, beta2=0.999, eps=1e-8, **kw):
    """Plain Adam over the free nodes; returns positions and energies before/after."""
    P0 = initial_positions(top)
    P = P0.copy()
    m = np.zeros_like(P)
    v = np.zeros_like(P)
    free = top.free
    e0 = energy_grad(top, P, P0, img, want_grad=False, **kw)
    for t in range(1, steps + 1):
        _, _, g = energy_grad(top, P, P0, img, **kw)
        m = beta1 * m + (1 - beta1) * g
        v = beta2 * v + (1 - beta2) * g * g
        mh = m / (1 - beta1 ** t)
        vh = v / (1 - beta2 ** t)
        P[free] -= lr * mh[free] / (np.sqrt(vh[free]) + eps)
    e1 = energy_grad(top, P, P0, img, want_grad=False, **kw)
    return P, e0, e1
