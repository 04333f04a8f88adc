"""CPU restatement of bicos-cli's point-cloud step.  TEST INFRASTRUCTURE ONLY.

* :func:`reproject` -- cv::reprojectImageTo3D(disp, points, Q, false,
  CV_32F) as libBICOS's CLI calls it (src/cli.cpp:228-236): per pixel
  [X Y Z W]^T = Q [x y d 1]^T in FP64, stored as float32 (X/W, Y/W, Z/W),
  W = 0 giving (0, 0, 0).  OpenCV is not available here, so the rounding of
  OpenCV's own loop is not pinned: the GPU kernel is checked against this
  FP64 restatement with an error bound.
* :func:`xyz_lines` -- save_pointcloud (include/fileutils.hpp:44-90): skip
  pixels with an invalid disparity (INT16_MIN, or NaN for float maps),
  points with a non-finite coordinate, and (unless allowed) points with
  Z < 0; each kept point is one "x y z" line in the C++ stream's default
  float format (%g, 6 significant digits).
"""
from __future__ import annotations

import math

import numpy as np

INVALID_I16 = -32768


def reproject(disp: np.ndarray, q) -> np.ndarray:
    q = np.asarray(q, dtype=np.float64).reshape(4, 4)
    rows, cols = disp.shape
    ys, xs = np.mgrid[0:rows, 0:cols].astype(np.float64)
    d = disp.astype(np.float64)
    h = [q[i, 0] * xs + q[i, 1] * ys + q[i, 2] * d + q[i, 3] for i in range(4)]
    with np.errstate(divide="ignore", invalid="ignore"):
        iw = np.where(h[3] != 0.0, 1.0 / np.where(h[3] != 0.0, h[3], 1.0), 0.0)
        out = np.stack([h[0] * iw, h[1] * iw, h[2] * iw], axis=-1)
    out[~np.isfinite(d)] = np.nan  # NaN disparities propagate
    return out.astype(np.float32)


def xyz_lines(points: np.ndarray, disp: np.ndarray, allow_negative_z: bool):
    """(lines, n_nonfinite, n_negative_z), pixels in row-major order."""
    lines, nonfinite, negative = [], 0, 0
    rows, cols = disp.shape
    for r in range(rows):
        for c in range(cols):
            d = disp[r, c]
            if (disp.dtype == np.int16 and d == INVALID_I16) or (disp.dtype != np.int16 and math.isnan(d)):
                continue
            x, y, z = (float(v) for v in points[r, c])
            if not (math.isfinite(x) and math.isfinite(y) and math.isfinite(z)):
                nonfinite += 1
                continue
            if not allow_negative_z and z < 0.0:
                negative += 1
                continue
            lines.append("%g %g %g" % (x, y, z))
    return lines, nonfinite, negative
