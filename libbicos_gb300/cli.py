"""Headless command-line front end: libBICOS's bicos-cli (src/cli.cpp)
on the GB300 matcher.

    python -m libbicos_gb300.cli folder0 [folder1] [options]

Options, defaults and behaviour follow src/cli.cpp:59-253:

* inputs: numbered images N.png in folder0 and folder1, or N_left.png /
  N_right.png in folder0 alone (PNG, TIFF or .npy; colour becomes grey);
  ``-n`` keeps the first n of each stack;
* ``-t`` threshold (default 0.75; <= 0 disables the NCC stage), ``-v``
  minimum variance (applied only when given, and > 0), ``-s`` subpixel
  step, ``--limited`` (the default transform is FULL), ``--double``,
  ``-m`` max left-right difference (Consistency), ``--no-dupes``,
  ``--corrmap`` (forces threshold -1 when none is set);
* outputs: ``<out>.tiff`` (the raw disparity, int16 or float32),
  ``<out>.png`` (the valid disparities scaled to 0..255, invalid = 0; the
  reference additionally applies OpenCV's TURBO colour map, which is not
  reproduced here), ``<out>-corrmap.*`` likewise, and with ``-q`` a
  point cloud ``<out>.xyz`` (cv::reprojectImageTo3D on the GPU, then the
  reference's filters: invalid disparity, non-finite points, Z < 0 unless
  ``--allow-negative-z``).  The reference reads that last flag under a
  different, undeclared name (src/cli.cpp:232), so there it never takes
  effect; here it does.
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np

from . import imageio, pointcloud, pybicos

BANNER = "libbicos_gb300: BICOS stereo matching on GB300 (bicos-cli front end)"


def parse_args(argv=None) -> argparse.Namespace:
    ap = argparse.ArgumentParser(prog="bicos-cli", description="cli to process images with BICOS")
    ap.add_argument("folder0", help="First folder containing input images with numbered names.")
    ap.add_argument("folder1", nargs="?", default=None,
                    help="Optional second folder with input images. If specified, file names need to be 0.png, "
                         "1.png... Else, folder0 needs to contain 0_left.png, 0_right.png, 1_left.png...")
    ap.add_argument("-t", "--threshold", type=float, default=0.75,
                    help="Minimum normalized cross corellation for a match to be accepted. Set to 0.0 to disable.")
    ap.add_argument("-v", "--variance", type=float, default=None,
                    help="Minimum intensity variance. Only active with --threshold.")
    ap.add_argument("-s", "--step", type=float, default=None,
                    help="Stepsize for subpixel interpolation. Only effective when threshold is set.")
    ap.add_argument("-o", "--out", default="bicosdisp.png", help="Output file for disparity image.")
    ap.add_argument("-n", "--stacksize", type=int, default=None,
                    help="Number of images to process. Defaults to all found in the input folders.")
    ap.add_argument("-q", "--qmatrix", default=None,
                    help='Path to cv::FileStorage with single matrix "Q" for reconstructing a pointcloud.')
    ap.add_argument("--allow-negative-z", action="store_true",
                    help="Allow for points with negative Z values in the pointcloud output.")
    ap.add_argument("-m", "--lr-maxdiff", type=int, default=None,
                    help="Maximum disparity difference between left and right image. Enabling this disables "
                         "duplicate filtering.")
    ap.add_argument("--double", action="store_true", help="Set double instead of single precision")
    ap.add_argument("--limited", action="store_true", help="Limit transformation mode. Allows for more images.")
    ap.add_argument("--corrmap", action="store_true", help="Output map of normalized cross correlation values.")
    ap.add_argument("--no-dupes", action="store_true",
                    help="Default BICOS variant when --lr-maxdiff is not specified. Can be set together with "
                         "--lr-maxdiff to activate both.")
    return ap.parse_args(argv)


def config_from_args(a: argparse.Namespace, err=sys.stderr):
    """(pybicos.Config, need_corrmap) as src/cli.cpp:136-171 builds them."""
    c = pybicos.Config()
    c.nxcorr_threshold = a.threshold if a.threshold > 0.0 else None
    c.mode = pybicos.Limited if a.limited else pybicos.Full
    need_corrmap = a.corrmap
    if need_corrmap and c.nxcorr_threshold is None:
        c.nxcorr_threshold = -1.0
        print(f"Computing with nxcorr-threshold of {c.nxcorr_threshold} because 'corrmap' is set", file=err)
    if a.step is not None:
        c.subpixel_step = a.step
    if a.variance is not None and a.variance > 0.0:
        c.min_variance = a.variance
    if a.double:
        c.precision = pybicos.Double
    if a.lr_maxdiff is not None:
        c.variant = pybicos.Variant.Consistency(int(a.lr_maxdiff), bool(a.no_dupes))
    return c, need_corrmap


def normalized_u8(img: np.ndarray) -> np.ndarray:
    """Valid values scaled linearly to 0..255 (min -> 0, max -> 255,
    rounded), invalid (INT16_MIN / NaN) -> 0."""
    valid = img != pointcloud.INVALID_I16 if img.dtype == np.int16 else ~np.isnan(img)
    out = np.zeros(img.shape, dtype=np.uint8)
    if valid.any():
        v = img[valid].astype(np.float64)
        lo, hi = v.min(), v.max()
        scale = 255.0 / (hi - lo) if hi > lo else 0.0
        out[valid] = np.clip(np.rint((v - lo) * scale), 0, 255).astype(np.uint8)
    return out


def save_image(img: np.ndarray, outfile: str, out=sys.stdout, err=sys.stderr) -> None:
    base = os.path.splitext(outfile)[0]
    imageio.write_png(base + ".png", normalized_u8(img))
    print(f"Saved normalized disparity to\t\t{base}.png", file=out)
    imageio.write_tiff(base + ".tiff", img)
    print(f"Saved floating-point disparity to\t{base}.tiff", file=err)


def main(argv=None, out=sys.stdout, err=sys.stderr) -> int:
    import torch

    import libbicos_gb300 as lbg

    a = parse_args(argv)
    print(BANNER, file=out)
    if a.no_dupes and a.lr_maxdiff is None:
        print("'no-dupes' is the default when 'lr-maxdiff' is not set.", file=err)
    if a.qmatrix is not None and not os.path.exists(a.qmatrix):
        raise ValueError(f"'{a.qmatrix}' does not exist")

    left, right = imageio.read_sequence(a.folder0, a.folder1)
    if a.stacksize is not None and a.stacksize < len(left):
        left, right = left[:a.stacksize], right[:a.stacksize]
    if len(left) != len(right):
        raise ValueError(f"Left stack: {len(left)}, right stack: {len(right)} images")
    if not left:
        raise ValueError("no input images")
    print(f"Loaded {2 * len(left)} {left[0].dtype.itemsize * 8}-bit images in total", file=out)

    cfg, need_corrmap = config_from_args(a, err)
    dev = torch.device("cuda")
    tick = time.perf_counter()
    l_gpu = torch.from_numpy(np.stack(left)).to(dev)
    r_gpu = torch.from_numpy(np.stack(right)).to(dev)
    torch.cuda.synchronize()
    t_up = (time.perf_counter() - tick) * 1e3
    print(f"Latency:\t {t_up:.3f}ms (upload)\t", end="", file=out)
    tick = time.perf_counter()
    disp_gpu, corr_gpu = lbg.match_device(l_gpu, r_gpu, cfg, corrmap=need_corrmap)
    torch.cuda.synchronize()
    t_match = (time.perf_counter() - tick) * 1e3
    print(f"{t_match:.3f}ms (match)\t", end="", file=out)
    tick = time.perf_counter()
    disp = disp_gpu.cpu().numpy()
    corr = corr_gpu.cpu().numpy() if need_corrmap and corr_gpu is not None else None
    t_down = (time.perf_counter() - tick) * 1e3
    print(f"{t_down:.3f}ms (download)", file=out)

    save_image(disp, a.out, out, err)
    if corr is not None:
        base, ext = os.path.splitext(a.out)
        save_image(corr, base + "-corrmap" + ext, out, err)

    if a.qmatrix is not None:
        q = imageio.read_matrix(a.qmatrix, "Q")
        pts = lbg.reproject(disp_gpu, q).cpu().numpy()
        xyz = os.path.splitext(a.out)[0] + ".xyz"
        counts = pointcloud.save_pointcloud(pts, disp, a.allow_negative_z, xyz)
        print(f"Saved pointcloud in ascii-format to\t{xyz}", file=out)
        if counts["nonfinite"] > 0:
            print(f"Skipped {counts['nonfinite']} points with non-finite fp values", file=err)
        if counts["negative_z"] > 0:
            print(f"Skipped {counts['negative_z']} points with negative Z values", file=err)
    return 0


if __name__ == "__main__":
    sys.exit(main())
