"""Seeded synthetic pixel-art inputs with the shapes of the benchmark workloads.

There is no public dataset for this path: every workload is generated here
from a fixed seed. Images are RGBA8 ``(H, W, 4)`` uint8 arrays whose row 0 is
the bottom row (the y-up order the reference's frame path works in after its
image loader flips rows, Image.cpp:21-38).

* ``frame``   -- one 256x224 frame: 16-colour palette, 40 rectangles and
                 30 ellipses of 4-48 px, dark 1-px outlines on half of the
                 shapes, checkerboard dithering over 5 % of the area.
* ``frame_large`` -- 640x480, 64 colours, 200 shapes, 10 % dithering and 2 %
                 isolated single-pixel noise.
* ``sprites`` -- a list of sprites with sides drawn from U[8, 64], 4-16
                 colours, 1-8 shapes; 30 % have a fully transparent background
                 and outlined shapes.
* ``stream``  -- frames of a 256x224 background (``frame``) with 24 sprites
                 moving at integer velocities of 0-3 px/frame, wrapping around.
"""
from __future__ import annotations

import numpy as np

__all__ = ["frame", "frame_large", "sprites", "stream", "draw_scene", "rgba_to_bgr"]


def _outline(img, mask, color):
    """Paint the 1-px inner border of ``mask`` with ``color``."""
    inner = mask.copy()
    inner[1:, :] &= mask[:-1, :]
    inner[:-1, :] &= mask[1:, :]
    inner[:, 1:] &= mask[:, :-1]
    inner[:, :-1] &= mask[:, 1:]
    border = mask & ~inner
    img[border, :3] = color


def draw_scene(rng, w, h, n_colors, n_rect, n_ell, size_lo=4, size_hi=48, outline_p=0.5, dither_frac=0.05,
               noise_frac=0.0, transparent_bg=False):
    palette = rng.integers(0, 256, size=(n_colors, 3), dtype=np.int64).astype(np.uint8)
    img = np.zeros((h, w, 4), np.uint8)
    if transparent_bg:
        img[..., 3] = 0
    else:
        img[..., :3] = palette[rng.integers(n_colors)]
        img[..., 3] = 255
    yy, xx = np.mgrid[0:h, 0:w]
    kinds = np.array([0] * n_rect + [1] * n_ell)
    rng.shuffle(kinds)
    for kind in kinds:
        sw = int(rng.integers(size_lo, size_hi + 1))
        sh = int(rng.integers(size_lo, size_hi + 1))
        x0 = int(rng.integers(-sw // 2, max(w - sw // 2, 1)))
        y0 = int(rng.integers(-sh // 2, max(h - sh // 2, 1)))
        if kind == 0:
            mask = (xx >= x0) & (xx < x0 + sw) & (yy >= y0) & (yy < y0 + sh)
        else:
            cx, cy = x0 + (sw - 1) / 2.0, y0 + (sh - 1) / 2.0
            rx, ry = max(sw / 2.0, 0.5), max(sh / 2.0, 0.5)
            mask = ((xx - cx) / rx) ** 2 + ((yy - cy) / ry) ** 2 <= 1.0
        color = palette[rng.integers(n_colors)]
        img[mask, :3] = color
        img[mask, 3] = 255
        if transparent_bg or rng.random() < outline_p:
            dark = (color.astype(np.int64) // 4).astype(np.uint8)
            _outline(img, mask, dark)
    # checkerboard dithering: random rectangles until the requested area is covered
    target = dither_frac * w * h
    covered = np.zeros((h, w), bool)
    tries = 0
    while covered.sum() < target and tries < 10000:
        tries += 1
        dw = int(rng.integers(4, 33))
        dh = int(rng.integers(4, 33))
        x0 = int(rng.integers(0, max(w - dw, 1)))
        y0 = int(rng.integers(0, max(h - dh, 1)))
        region = np.zeros((h, w), bool)
        region[y0:y0 + dh, x0:x0 + dw] = True
        checker = region & (((xx + yy) & 1) == 0)
        img[checker, :3] = palette[rng.integers(n_colors)]
        img[checker, 3] = 255
        covered |= region
    if noise_frac > 0:
        k = int(noise_frac * w * h)
        idx = rng.choice(w * h, size=k, replace=False)
        flat = img.reshape(-1, 4)
        flat[idx, :3] = palette[rng.integers(n_colors, size=k)]
        flat[idx, 3] = 255
    return img


def frame(seed: int = 0, w: int = 256, h: int = 224) -> np.ndarray:
    """The 256x224 benchmark frame (16 colours, 40 rects + 30 ellipses)."""
    rng = np.random.default_rng([0xDE91, 0, seed])
    return draw_scene(rng, w, h, 16, 40, 30, dither_frac=0.05)


def frame_large(seed: int = 0, w: int = 640, h: int = 480) -> np.ndarray:
    """The 640x480 frame (64 colours, 200 shapes, 10 % dither, 2 % noise)."""
    rng = np.random.default_rng([0xDE91, 1, seed])
    n_rect = 110
    return draw_scene(rng, w, h, 64, n_rect, 200 - n_rect, dither_frac=0.10, noise_frac=0.02)


def sprites(count: int = 4096, seed: int = 0, lo: int = 8, hi: int = 64):
    """``count`` sprites of uneven sizes (sides ~ U[lo, hi])."""
    rng = np.random.default_rng([0xDE91, 2, seed])
    out = []
    for _ in range(count):
        w = int(rng.integers(lo, hi + 1))
        h = int(rng.integers(lo, hi + 1))
        n_colors = int(rng.integers(4, 17))
        n_shapes = int(rng.integers(1, 9))
        n_rect = int(rng.integers(0, n_shapes + 1))
        transparent = bool(rng.random() < 0.3)
        out.append(draw_scene(rng, w, h, n_colors, n_rect, n_shapes - n_rect, size_lo=4,
                              size_hi=min(48, max(w, h)), dither_frac=0.05, transparent_bg=transparent))
    return out


def stream(n_frames: int, seed: int = 0, n_sprites: int = 24, w: int = 256, h: int = 224):
    """``n_frames`` frames: the background ``frame(seed)`` with ``n_sprites``
    sprites of the ``sprites`` generator on top, each moving by an integer
    velocity (vx, vy in 0..3 px/frame) and wrapping around the frame edges.
    Sprite pixels with alpha 0 show the background. Returns (n, h, w, 4)."""
    rng = np.random.default_rng([0xDE91, 3, seed])
    bg = frame(seed, w=w, h=h)
    sp = sprites(n_sprites, seed=seed + 1000)
    pos = [(int(rng.integers(0, w)), int(rng.integers(0, h))) for _ in sp]
    vel = [(int(rng.integers(0, 4)), int(rng.integers(0, 4))) for _ in sp]
    out = np.empty((n_frames, h, w, 4), np.uint8)
    for f in range(n_frames):
        img = bg.copy()
        for s_img, (x0, y0), (vx, vy) in zip(sp, pos, vel):
            sh, sw = s_img.shape[:2]
            ys = (y0 + vy * f + np.arange(sh)) % h
            xs = (x0 + vx * f + np.arange(sw)) % w
            opaque = s_img[..., 3] > 0
            region = img[np.ix_(ys, xs)]
            region[opaque] = s_img[opaque]
            img[np.ix_(ys, xs)] = region
        out[f] = img
    return out


def rgba_to_bgr(img: np.ndarray):
    """The reference's image layout for an RGBA8 image: 3 bytes per pixel in
    B,G,R order (the loader's BGR, Image.cpp:42-48), rows padded to a 4-byte
    stride with zero padding. Returns ``(buffer, widthstep)``."""
    h, w = img.shape[:2]
    ws = (3 * w + 3) & ~3
    buf = np.zeros((h, ws), np.uint8)
    px = buf[:, :3 * w].reshape(h, w, 3)
    px[..., 0] = img[..., 2]
    px[..., 1] = img[..., 1]
    px[..., 2] = img[..., 0]
    return buf.reshape(-1), ws
