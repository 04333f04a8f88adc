"""bicos_match_points_v1: the match and its point cloud in one call
(bicos-cli's match followed by cv::reprojectImageTo3D, src/cli.cpp:188-194,
228-250).  The disparity and corrmap equal bicos_match_v1's bit for bit, and
the points equal the separate reprojection pass (bicos_reproject_v1) of
that disparity bit for bit, whether the agreement kernels wrote them
(every NCC form, with a threshold) or the pass ran after the search."""
import numpy as np
import pytest

import libbicos_gb300 as lbg
from gpu_util import assert_same, dev, host
from libbicos_gb300 import pybicos, scenes

pytestmark = pytest.mark.gpu

# a rectified pair's reprojection matrix: focal 1200 px, principal point
# (150, 30), baseline 0.1 (Q[3][2] = -1/Tx), equal principal points
Q = np.array([[1.0, 0.0, 0.0, -150.0],
              [0.0, 1.0, 0.0, -30.0],
              [0.0, 0.0, 0.0, 1200.0],
              [0.0, 0.0, 10.0, 0.0]])


def cfg(thr=0.9, step=None, double=False, form=0, cons=None):
    c = pybicos.Config()
    c.nxcorr_threshold, c.subpixel_step, c.min_variance = thr, step, 2.0
    c.precision = pybicos.Double if double else pybicos.Single
    c.nxcorr_form = form
    if cons:
        c.variant = pybicos.Variant.Consistency(*cons)
    return c


@pytest.mark.parametrize("bits", [8, 12])
@pytest.mark.parametrize("thr,step,double,form,cons", [
    (0.9, None, False, 0, None),       # fused: in-place agreement, int16
    (0.9, 0.1, False, 0, None),        # fused: single-precision sweep
    (0.9, 0.25, True, 0, (1, False)),  # fused: double-precision sweep
    (None, None, False, 0, None),      # no agreement stage: pass after the search
    (0.9, None, False, 1, None),       # fused: moment form, integer disparity
    (0.9, 0.1, False, 1, (1, False)),  # fused: moment form, single-precision sweep
    (0.9, 0.1, True, 1, None),         # fused: moment form, double-precision sweep
    (0.9, 0.1, False, 2, None),        # fused: learned form (proposals and the list's sweep)
    (0.9, 0.1, True, 2, (1, False)),   # fused: learned form, double precision
])
def test_points_equal_separate_reprojection(cuda, bits, thr, step, double, form, cons):
    sc = scenes.make_scene(60, 300, 12, seed=bits + form, bits=bits)
    L, R = dev(sc.left, cuda), dev(sc.right, cuda)
    c = cfg(thr, step, double, form, cons)
    d0, c0 = lbg.match_device(L, R, c)
    d1, c1, pts = lbg.match_device(L, R, c, q=Q)
    assert_same(host(d1), host(d0), "disparity")
    if c0 is not None:
        assert_same(host(c1), host(c0), "corrmap")
    want = lbg.reproject(d0, Q)
    assert_same(host(pts), host(want), "points")
    # the points are those of the disparity: finite where the match is valid
    valid = np.isfinite(host(d0).astype(np.float32)) & (host(d0) != -32768)
    assert np.isfinite(host(pts)[valid]).all()


def test_points_argument_checks(cuda):
    import torch
    sc = scenes.make_scene(16, 64, 6, seed=1)
    L, R = dev(sc.left, cuda), dev(sc.right, cuda)
    bad = torch.empty((16, 63, 3), dtype=torch.float32, device=cuda)
    with pytest.raises(pybicos.Exception, match="three-channel float32 image"):
        lbg.match_device(L, R, cfg(), q=Q, points=bad)
    qn = Q.copy()
    qn[0, 0] = np.nan
    with pytest.raises(ValueError, match="Q must be finite"):
        lbg.match_device(L, R, cfg(), q=qn)
