"""Seeded synthetic multi-shot stereo scenes.

Stand-in for libBICOS's real dataset (data/prepare.sh downloads it; it is
not available here).  A scene is a disparity field plus n left/right frame
pairs of a projected random pattern:

* disparity d(x, y) = 60 + 25 sin(2 pi x / 400) cos(2 pi y / 300), plus three
  random planar patches, clipped to [d_lo, d_hi];
* each left frame is i.i.d. Gaussian noise blurred with sigma (fixed, or
  drawn per frame), rescaled to 30..220 DN around 125 with a per-frame
  contrast factor;
* the right frame at column x samples the left frame at x + d(x, y) with
  linear interpolation (so the left pixel at column c matches the right
  pixel at c - d, the BICOS sign convention), plus Gaussian sensor noise;
* a random ~10% rectangle is flat 40 DN plus noise on both sides (no
  pattern), exercising the variance mask;
* 12-bit variants scale intensities by 16 (noise sigma 8 DN).

The generator is deterministic in ``seed`` (numpy PCG64).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Scene:
    left: np.ndarray       # (n, rows, cols) uint8 / uint16
    right: np.ndarray      # (n, rows, cols)
    disparity: np.ndarray  # (rows, cols) float32 ground truth at left pixels
    seed: int


def _blur(img: np.ndarray, sigma: float) -> np.ndarray:
    try:
        from scipy.ndimage import gaussian_filter
        return gaussian_filter(img, sigma, mode="reflect")
    except ImportError:  # separable fallback
        r = int(3 * sigma + 1)
        k = np.exp(-0.5 * (np.arange(-r, r + 1) / sigma) ** 2)
        k /= k.sum()
        tmp = np.apply_along_axis(lambda v: np.convolve(np.pad(v, r, mode="reflect"), k, "valid"), 1, img)
        return np.apply_along_axis(lambda v: np.convolve(np.pad(v, r, mode="reflect"), k, "valid"), 0, tmp)


def disparity_field(rows: int, cols: int, rng: np.random.Generator, d_lo: float, d_hi: float) -> np.ndarray:
    y, x = np.mgrid[0:rows, 0:cols].astype(np.float64)
    d = 60.0 + 25.0 * np.sin(2 * np.pi * x / 400.0) * np.cos(2 * np.pi * y / 300.0)
    for _ in range(3):
        h = int(rng.uniform(0.1, 0.3) * rows)
        w = int(rng.uniform(0.1, 0.3) * cols)
        y0 = int(rng.integers(0, max(1, rows - h)))
        x0 = int(rng.integers(0, max(1, cols - w)))
        base = rng.uniform(d_lo, d_hi)
        gx, gy = rng.uniform(-0.05, 0.05, size=2)
        yy, xx = y[y0:y0 + h, x0:x0 + w], x[y0:y0 + h, x0:x0 + w]
        d[y0:y0 + h, x0:x0 + w] = base + gx * (xx - x0) + gy * (yy - y0)
    return np.clip(d, d_lo, d_hi)


def make_scene(rows: int, cols: int, n: int, seed: int = 0, bits: int = 8, d_range=(20.0, 120.0),
               sigma=1.5, contrast=None, noise: float | None = None, flat_fraction: float = 0.10) -> Scene:
    """sigma: float, or (lo, hi) drawn per frame; contrast: None or (lo, hi)
    per frame; noise: sensor noise sigma in DN (default 2, x4 for 12 bit)."""
    rng = np.random.default_rng(seed)
    scale = 16.0 if bits == 12 else 1.0
    maxv = 4095 if bits == 12 else 255
    dtype = np.uint16 if bits > 8 else np.uint8
    noise = (8.0 if bits == 12 else 2.0) if noise is None else noise
    d = disparity_field(rows, cols, rng, *d_range)

    # flat region, same rectangle on both sides
    fh = int(rows * np.sqrt(flat_fraction))
    fw = int(cols * np.sqrt(flat_fraction))
    fy = int(rng.integers(0, max(1, rows - fh)))
    fx = int(rng.integers(0, max(1, cols - fw)))

    xs = np.arange(cols, dtype=np.float64)[None, :] + d  # right column x samples left at x + d
    x0 = np.floor(xs).astype(np.int64)
    fr = xs - x0
    x0c = np.clip(x0, 0, cols - 1)
    x1c = np.clip(x0 + 1, 0, cols - 1)
    ridx = np.arange(rows)[:, None]

    left = np.empty((n, rows, cols), dtype)
    right = np.empty((n, rows, cols), dtype)
    for t in range(n):
        s = rng.uniform(*sigma) if isinstance(sigma, (tuple, list)) else sigma
        c = rng.uniform(*contrast) if contrast is not None else 1.0
        pat = _blur(rng.standard_normal((rows, cols)), s)
        pat = (pat - pat.min()) / max(pat.max() - pat.min(), 1e-12)
        img = 125.0 + (pat * 190.0 - 95.0) * c  # 30..220 DN at full contrast
        r = img[ridx, x0c] * (1 - fr) + img[ridx, x1c] * fr
        r = r + rng.normal(0.0, noise / scale, size=r.shape)
        img[fy:fy + fh, fx:fx + fw] = 40.0 + rng.normal(0.0, noise / scale, size=(fh, fw))
        r[fy:fy + fh, fx:fx + fw] = 40.0 + rng.normal(0.0, noise / scale, size=(fh, fw))
        left[t] = np.clip(np.rint(img * scale), 0, maxv).astype(dtype)
        right[t] = np.clip(np.rint(r * scale), 0, maxv).astype(dtype)

    # ground truth at left pixels: the left column c matches right c - d(c - d)
    # (d is smooth, so a fixed-point step from d at c is enough)
    cgrid = np.arange(cols, dtype=np.float64)[None, :]
    gt = d.copy()
    for _ in range(3):
        xr = np.clip(cgrid - gt, 0, cols - 1)
        i0 = np.floor(xr).astype(np.int64)
        f = xr - i0
        i1 = np.clip(i0 + 1, 0, cols - 1)
        gt = d[ridx, i0] * (1 - f) + d[ridx, i1] * f
    return Scene(left, right, gt.astype(np.float32), seed)


# The workloads: (rows, cols, n, bits, mode, kwargs) of the seeded configs.
WORKLOADS = {
    "vga_n12": dict(rows=480, cols=640, n=12, bits=8, d_range=(20.0, 120.0), sigma=1.5),
    "mv1936_n33": dict(rows=1216, cols=1936, n=33, bits=8, d_range=(30.0, 250.0), sigma=(1.0, 2.0),
                       contrast=(0.5, 1.0)),
    "qxga12_n20": dict(rows=1536, cols=2048, n=20, bits=12, d_range=(20.0, 120.0), sigma=1.5),
}


def workload_scene(name: str, seed: int = 0, rows: int | None = None, cols: int | None = None) -> Scene:
    kw = dict(WORKLOADS[name])
    if rows is not None:
        kw["rows"] = rows
    if cols is not None:
        kw["cols"] = cols
    return make_scene(seed=seed, **kw)


def make_scene_device(rows: int, cols: int, n: int, seed: int = 0, bits: int = 8, d_range=(20.0, 120.0),
                      sigma=1.5, noise: float | None = None, flat_fraction: float = 0.10, device="cuda"):
    """The make_scene recipe on the GPU (torch, seeded Philox generator), for
    stacks too large to synthesise quickly on the host: returns (left, right)
    as (n, rows, cols) uint8 / uint16 CUDA tensors.  Blur is a separable
    Gaussian of radius 3 sigma with edge replication."""
    import torch
    g = torch.Generator(device=device).manual_seed(seed)
    rng = np.random.default_rng(seed)
    scale = 16.0 if bits == 12 else 1.0
    maxv = 4095 if bits == 12 else 255
    dtype = torch.int16 if bits > 8 else torch.uint8
    noise = (8.0 if bits == 12 else 2.0) if noise is None else noise
    d = torch.from_numpy(disparity_field(rows, cols, rng, *d_range)).to(device=device, dtype=torch.float32)
    fh, fw = int(rows * np.sqrt(flat_fraction)), int(cols * np.sqrt(flat_fraction))
    fy = int(rng.integers(0, max(1, rows - fh)))
    fx = int(rng.integers(0, max(1, cols - fw)))
    xs = torch.arange(cols, device=device, dtype=torch.float32)[None, :] + d
    x0 = torch.floor(xs)
    fr = xs - x0
    x0c = x0.long().clamp(0, cols - 1)
    x1c = (x0.long() + 1).clamp(0, cols - 1)
    r_ = int(3 * sigma + 1)
    k = torch.exp(-0.5 * (torch.arange(-r_, r_ + 1, device=device, dtype=torch.float32) / sigma) ** 2)
    k = (k / k.sum()).view(1, 1, -1)
    left = torch.empty((n, rows, cols), dtype=dtype, device=device)
    right = torch.empty((n, rows, cols), dtype=dtype, device=device)
    for t in range(n):
        z = torch.randn((1, rows, cols), generator=g, device=device)
        z = torch.nn.functional.conv1d(torch.nn.functional.pad(z.view(rows, 1, cols), (r_, r_), mode="replicate"), k)
        z = z.view(rows, cols).t().contiguous().view(cols, 1, rows)
        z = torch.nn.functional.conv1d(torch.nn.functional.pad(z, (r_, r_), mode="replicate"), k).view(cols, rows).t()
        pat = (z - z.min()) / (z.max() - z.min()).clamp_min(1e-12)
        img = 125.0 + (pat * 190.0 - 95.0)
        rimg = torch.gather(img, 1, x0c) * (1 - fr) + torch.gather(img, 1, x1c) * fr
        rimg = rimg + torch.randn((rows, cols), generator=g, device=device) * (noise / scale)
        img[fy:fy + fh, fx:fx + fw] = 40.0 + torch.randn((fh, fw), generator=g, device=device) * (noise / scale)
        rimg[fy:fy + fh, fx:fx + fw] = 40.0 + torch.randn((fh, fw), generator=g, device=device) * (noise / scale)
        left[t] = torch.round(img * scale).clamp(0, maxv).to(dtype)
        right[t] = torch.round(rimg * scale).clamp(0, maxv).to(dtype)
    if bits > 8:  # the matcher takes uint16: same bits
        left, right = left.view(torch.uint16), right.view(torch.uint16)
    return left, right


# Batching workload: 16 stacks of mixed size, depth, input type, mode and step.
BATCH_SIZES = [(480, 640), (1024, 1280), (1216, 1936), (2048, 2448)]
BATCH_DEPTHS = [8, 12, 20, 33, 40]


# FULL descriptors need n^2 - 2n + 3 bits: n <= 16 within libBICOS's 256,
# n <= 23 with the 512-bit extension; the deeper stacks of the draw (33, 40:
# 1026 and 1523 bits) are matched with limited descriptors.
BATCH_MAX_FULL_N = 23


def batch_specs(count: int = 16, seed: int = 0):
    """(rows, cols, n, bits, full, step) per stack, drawn from seed: FULL
    descriptors where the 512-bit extension allows them (n <= 23; match
    with max_bits=512), limited otherwise."""
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(count):
        rows, cols = BATCH_SIZES[int(rng.integers(len(BATCH_SIZES)))]
        n = int(rng.choice(BATCH_DEPTHS))
        bits = 12 if rng.random() < 0.5 else 8
        full = bool(n <= BATCH_MAX_FULL_N and rng.random() < 0.5)
        step = 0.1 if rng.random() < 0.5 else None
        specs.append((rows, cols, n, bits, full, step))
    return specs
