"""Seeded synthetic images and covers for the benchmark workloads.

The workloads of this path are defined on generated images, not on a public
dataset: per channel a sum of four low-frequency sinusoids (period 32-256 px,
random orientation and phase), 1/f Gaussian noise of sigma 12 DN shaped in
the Fourier domain, and six axis-aligned hard-edged rectangles of uniform
random colour, clamped to [0, 255]; 16-bit images scale the same values by
257.  Everything derives from one numpy PCG64 seed.
"""
from __future__ import annotations

import numpy as np

from . import DCT8, DCT16, DCT32, ORIGIN, SHAPES


def synthetic_rgb(width: int, height: int, seed: int, bits: int = 8) -> np.ndarray:
    """Interleaved [H, W, 3] uint8 (bits 8) or uint16 (bits 16) image."""
    rng = np.random.Generator(np.random.PCG64(seed))
    yy, xx = np.mgrid[0:height, 0:width].astype(np.float32)
    out = np.empty((height, width, 3), np.float32)
    fy = np.fft.fftfreq(height)[:, None]
    fx = np.fft.rfftfreq(width)[None, :]
    radius = np.sqrt(fx * fx + fy * fy)
    radius[0, 0] = 1.0
    shaping = (1.0 / radius).astype(np.float32)
    shaping[0, 0] = 0.0
    for c in range(3):
        acc = np.full((height, width), 128.0, np.float32)
        for _ in range(4):
            period = rng.uniform(32.0, 256.0)
            theta = rng.uniform(0.0, np.pi)
            phase = rng.uniform(0.0, 2.0 * np.pi)
            amp = rng.uniform(15.0, 40.0)
            k = 2.0 * np.pi / period
            acc += amp * np.sin(k * (np.cos(theta) * xx + np.sin(theta) * yy) + phase)
        white = rng.standard_normal((height, width)).astype(np.float32)
        colored = np.fft.irfft2(np.fft.rfft2(white) * shaping, s=(height, width))
        std = float(colored.std()) or 1.0
        acc += (colored * (12.0 / std)).astype(np.float32)
        out[..., c] = acc
    for _ in range(6):
        rw = int(rng.integers(max(1, width // 16), max(2, width // 3)))
        rh = int(rng.integers(max(1, height // 16), max(2, height // 3)))
        x0 = int(rng.integers(0, max(1, width - rw)))
        y0 = int(rng.integers(0, max(1, height - rh)))
        colour = rng.uniform(0.0, 255.0, size=3).astype(np.float32)
        out[y0:y0 + rh, x0:x0 + rw, :] = colour
    img = np.clip(np.rint(out), 0, 255)
    if bits == 8:
        return img.astype(np.uint8)
    return (img.astype(np.uint32) * 257).astype(np.uint16)


def fixed_dct8_map(width: int, height: int) -> np.ndarray:
    """policy block.rs:39 fixed_dct8x8: every block its own DCT8 varblock."""
    bw, bh = (width + 7) // 8, (height + 7) // 8
    return np.full((bh, bw), DCT8 | ORIGIN, np.uint8)


def place(map_: np.ndarray, bx: int, by: int, sel: int) -> None:
    r, c = SHAPES[sel]
    map_[by:by + r, bx:bx + c] = sel
    map_[by, bx] = sel | ORIGIN


def activity_cover(rgb: np.ndarray, threshold16: float = 6.0, threshold32: float = 3.0) -> np.ndarray:
    """A square DCT8/16/32 cover chosen by local activity.

    Stand-in for the reference's rate-distortion cover (policy lib.rs:5260
    select_blocks), which is host policy outside this path: smooth aligned
    32x32 regions take DCT32, smooth 16x16 regions DCT16, the rest DCT8.
    """
    h, w = rgb.shape[:2]
    bw, bh = (w + 7) // 8, (h + 7) // 8
    luma = rgb.astype(np.float32).mean(axis=2)
    if rgb.dtype == np.uint16:
        luma /= 257.0
    pad = np.pad(luma, ((0, bh * 8 - h), (0, bw * 8 - w)), mode="edge")
    std8 = pad.reshape(bh, 8, bw, 8).std(axis=(1, 3))
    m = np.full((bh, bw), DCT8 | ORIGIN, np.uint8)
    done = np.zeros((bh, bw), bool)
    for by in range(0, bh - 3, 4):
        for bx in range(0, bw - 3, 4):
            if std8[by:by + 4, bx:bx + 4].max() < threshold32:
                place(m, bx, by, DCT32)
                done[by:by + 4, bx:bx + 4] = True
    for by in range(0, bh - 1, 2):
        for bx in range(0, bw - 1, 2):
            if not done[by:by + 2, bx:bx + 2].any() and std8[by:by + 2, bx:bx + 2].max() < threshold16:
                place(m, bx, by, DCT16)
                done[by:by + 2, bx:bx + 2] = True
    return m


def mixed_cover(width: int, height: int, seed: int, rectangles: bool = True) -> np.ndarray:
    """A seeded cover mixing all nine plain DCT shapes (for render parity)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    bw, bh = (width + 7) // 8, (height + 7) // 8
    m = np.full((bh, bw), DCT8 | ORIGIN, np.uint8)
    taken = np.zeros((bh, bw), bool)
    shapes = list(SHAPES) if rectangles else [DCT8, DCT16, DCT32]
    for by in range(bh):
        for bx in range(bw):
            if taken[by, bx]:
                continue
            order = rng.permutation(len(shapes))
            for i in order:
                sel = shapes[i]
                r, c = SHAPES[sel]
                if bx % c or by % r or bx + c > bw or by + r > bh:
                    continue
                if taken[by:by + r, bx:bx + c].any():
                    continue
                place(m, bx, by, sel)
                taken[by:by + r, bx:bx + c] = True
                break
    return m
