"""Moment form of the agreement (extension, Config.nxcorr_form = 1): the
CUDA path -- Sxy band on the tensor cores, exact integer moments,
closed-form correlation of the unrounded interpolant -- equals the oracle's
restatement bit for bit; its difference from the reference's FP64 sweep is
measured and stated here."""
import numpy as np
import pytest

import libbicos_gb300 as lbg
from gpu_util import assert_same, dev, host
from libbicos_gb300 import pybicos, scenes

pytestmark = pytest.mark.gpu


def cfg(thr=0.9, step=None, mv=2.0, double=True, form=1, full=False):
    c = pybicos.Config()
    c.nxcorr_threshold = thr
    c.subpixel_step = step
    c.min_variance = mv
    c.precision = pybicos.Double if double else pybicos.Single
    c.mode = pybicos.Full if full else pybicos.Limited
    c.nxcorr_form = form
    return c


def raw_disparity(cuda, sc, full=False):
    d, _ = lbg.match_device(dev(sc.left, cuda), dev(sc.right, cuda), cfg(thr=None, full=full))
    return host(d)


@pytest.mark.parametrize("bits,n", [(8, 12), (8, 33), (12, 16), (8, 65), (12, 20)])
@pytest.mark.parametrize("double", [True, False])
@pytest.mark.parametrize("step", [None, 0.1, 0.25])
def test_moment_form_vs_oracle(cuda, oracle, bits, n, double, step):
    sc = scenes.make_scene(40, 300, n, seed=n + bits, bits=bits)
    full = bits == 12 and n <= 16
    raw = raw_disparity(cuda, sc, full)
    d, corr = lbg.match_device(dev(sc.left, cuda), dev(sc.right, cuda), cfg(0.9, step, 2.0, double, full=full))
    wd, wc = oracle.moments(raw, sc.left, sc.right, 0.9, step, 2.0 * n, double)
    assert_same(host(d), wd, "disparity")
    assert_same(host(corr), wc, "corrmap")


@pytest.mark.parametrize("bits,n", [(8, 33), (12, 20)])
@pytest.mark.parametrize("step,mv", [(0.01, 2.0), (0.02, None), (0.1, 400.0), (0.05, 2500.0)])
def test_moment_form_screening_edges(cuda, oracle, bits, n, step, mv):
    """the double sweep's single-precision screening (FP64 only for the
    points its bracket cannot rule out): fine steps (up to 201 points, many
    near-equal neighbours), no min-variance test, and thresholds close to
    the pixels' own variances (the test decided in FP64 when the bracket
    straddles it) -- all bit for bit with the restatement, which evaluates
    every point in FP64"""
    sc = scenes.make_scene(24, 240, n, seed=3 * n + bits, bits=bits)
    raw = raw_disparity(cuda, sc)
    d, corr = lbg.match_device(dev(sc.left, cuda), dev(sc.right, cuda), cfg(0.5, step, mv, True))
    wd, wc = oracle.moments(raw, sc.left, sc.right, 0.5, step, None if mv is None else mv * n, True)
    assert_same(host(d), wd, "disparity")
    assert_same(host(corr), wc, "corrmap")


@pytest.mark.parametrize("step", [None, 0.1])
def test_moment_form_full_16bit(cuda, oracle, step):
    """16-bit samples over the full range (up to 65535, beyond the 6+6-bit
    split's exact range): tiles holding a sample of 4096 or more take the
    exact SIMT sums, so the moments stay exact integers and the results
    equal the restatement bit for bit"""
    sc = scenes.make_scene(24, 256, 20, seed=11, bits=12)
    left = (sc.left.astype(np.uint32) * 16 + 7).clip(0, 65535).astype(np.uint16)
    right = (sc.right.astype(np.uint32) * 16 + 7).clip(0, 65535).astype(np.uint16)
    assert left.max() >= 4096
    raw, _ = lbg.match_device(dev(left, cuda), dev(right, cuda), cfg(thr=None))
    raw = host(raw)
    d, corr = lbg.match_device(dev(left, cuda), dev(right, cuda), cfg(0.5, step, 2.0, True))
    wd, wc = oracle.moments(raw, left, right, 0.5, step, 2.0 * 20, True)
    assert_same(host(d), wd, "disparity")
    assert_same(host(corr), wc, "corrmap")


def test_moment_form_window_fallback(cuda, oracle):
    """tiles whose disparities spread wider than the 64-column window (here:
    planar patches of 5..200 px next to the smooth field, and no threshold on
    the raw match) take the SIMT path: same results"""
    sc = scenes.make_scene(16, 600, 12, seed=5, d_range=(5.0, 200.0))
    raw = raw_disparity(cuda, sc)
    d, corr = lbg.match_device(dev(sc.left, cuda), dev(sc.right, cuda), cfg(0.5, 0.25, None, True))
    wd, wc = oracle.moments(raw, sc.left, sc.right, 0.5, 0.25, None, True)
    assert_same(host(d), wd)
    assert_same(host(corr), wc)


def test_moment_form_error_vs_reference_sweep(cuda, oracle):
    """stated error of the moment form against the FP64 restatement of the
    reference (precision double), on the 640x480 n=12 workload:
    integer disparities: identical decisions up to rounding ties, |d rho| <= 1e-12;
    subpixel (step 0.1): the reference rounds its interpolants, so rho and
    the chosen offset differ; reported here and bounded loosely."""
    sc = scenes.workload_scene("vga_n12", seed=2)
    raw = raw_disparity(cuda, sc)
    d0, c0 = lbg.match_device(dev(sc.left, cuda), dev(sc.right, cuda), cfg(0.9, None, 2.0, True))
    r0, rc0 = oracle.agree(raw, sc.left, sc.right, 0.9, 2.0 * 12, True)
    both = np.isfinite(host(c0)) & np.isfinite(rc0)
    drho = np.abs(host(c0)[both] - rc0[both])
    print(f"\nmoment form, integer disparity: max |d rho| = {drho.max():.3e} over {both.sum()} pixels; "
          f"disparity decisions differing: {(host(d0) != r0).sum()}")
    assert drho.max() <= 1e-12
    d1, c1 = lbg.match_device(dev(sc.left, cuda), dev(sc.right, cuda), cfg(0.9, 0.1, 2.0, True))
    r1, rc1 = oracle.agree_subpixel(raw, sc.left, sc.right, 0.9, 0.1, 2.0 * 12, True)
    g1, gc1 = host(d1), host(c1)
    both = np.isfinite(g1) & np.isfinite(r1)
    dd = np.abs(g1[both] - r1[both])
    dr = np.abs(gc1[both] - rc1[both])
    print(f"moment form, step 0.1: |d disparity| median {np.median(dd):.3f}, p95 {np.percentile(dd, 95):.3f}, "
          f"rms {np.sqrt(np.mean(dd ** 2)):.4f} px; |d rho| median {np.median(dr):.2e}, "
          f"max {dr.max():.2e}; validity agreement {np.mean(np.isfinite(g1) == np.isfinite(r1)):.4f}")
    assert np.sqrt(np.mean(dd ** 2)) < 0.15
    assert np.mean(np.isfinite(g1) == np.isfinite(r1)) > 0.97
