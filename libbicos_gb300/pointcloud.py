"""Point clouds from disparity maps: the GPU reprojection
(:func:`libbicos_gb300.reproject`, bicos_reproject_v1) and the ASCII .xyz
writer of libBICOS's CLI (save_pointcloud, include/fileutils.hpp:44-90).

The writer keeps a pixel when its disparity is valid (not INT16_MIN, not
NaN), all three coordinates are finite and, unless negative Z is allowed,
Z >= 0; it writes one "x y z" line per kept point, row-major, each value
in C's %g format (the C++ stream default the reference prints with).
"""
from __future__ import annotations

import numpy as np

INVALID_I16 = -32768


def keep_mask(points: np.ndarray, disparity: np.ndarray, allow_negative_z: bool):
    """(mask of written points, number of non-finite points, number of
    points dropped for Z < 0), counted over valid disparities."""
    if disparity.dtype == np.int16:
        valid = disparity != INVALID_I16
    else:
        valid = ~np.isnan(disparity)
    finite = np.isfinite(points).all(axis=-1)
    nonfinite = int((valid & ~finite).sum())
    keep = valid & finite
    negative = 0
    if not allow_negative_z:
        neg = keep & (points[..., 2] < 0.0)
        negative = int(neg.sum())
        keep &= ~neg
    return keep, nonfinite, negative


def save_pointcloud(points, disparity, allow_negative_z: bool, outfile: str) -> dict:
    """Write the .xyz file for host (rows, cols, 3) float32 points and the
    (rows, cols) disparity they came from.  Returns the counts the reference
    reports: written, nonfinite, negative_z."""
    points = np.asarray(points, dtype=np.float32)
    disparity = np.asarray(disparity)
    if points.shape[:2] != disparity.shape or points.shape[-1] != 3:
        raise ValueError("save_pointcloud: invalid sizes")
    keep, nonfinite, negative = keep_mask(points, disparity, allow_negative_z)
    kept = points[keep].astype(np.float64)
    with open(outfile, "w") as f:
        if len(kept):
            f.write("\n".join("%g %g %g" % (x, y, z) for x, y, z in kept.tolist()))
            f.write("\n")
    return {"written": int(len(kept)), "nonfinite": nonfinite, "negative_z": negative}
