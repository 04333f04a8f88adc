"""NCC agreement and subpixel sweep on the GPU vs the oracle.  Integer
disparities, float disparities and correlations are bit-exact in single
precision (the kernels use the reference's IEEE operation order) and in
double precision (vs the FP64 restatement of nxcorrd)."""
import numpy as np
import pytest

import libbicos_gb300 as lbg
from conftest import golden
from gpu_util import assert_same, dev, host

pytestmark = pytest.mark.gpu


def test_agree_golden(cuda):
    z = golden("agree.npz")
    for c in sorted({k.split("_")[0] for k in z.files}, key=lambda s: int(s[1:])):
        thr, step, mv = float(z[c + "_thr"]), float(z[c + "_step"]), float(z[c + "_minvar"])
        mv = None if mv < 0 else mv
        s0, s1 = dev(z[c + "_s0"], cuda), dev(z[c + "_s1"], cuda)
        raw = dev(z[c + "_raw"], cuda)
        if step < 0:
            d, corr = lbg.agree(raw, s0, s1, thr, mv)
        else:
            d, corr = lbg.agree_subpixel(raw, s0, s1, thr, step, mv)
        assert_same(host(d), z[c + "_disp"], c + " disparity")
        assert_same(host(corr), z[c + "_corr"], c + " corrmap")


def _case(rng, dt, n, rows, cols):
    s0 = rng.integers(0, np.iinfo(dt).max + 1, size=(n, rows, cols), dtype=dt)
    s1 = rng.integers(0, np.iinfo(dt).max + 1, size=(n, rows, cols), dtype=dt)
    disp = rng.integers(-2, cols, size=(rows, cols)).astype(np.int16)
    disp[rng.random((rows, cols)) < 0.1] = -32768
    # make ~half of the pairs correlated
    r_idx, c_idx = np.nonzero((disp != -32768) & (rng.random((rows, cols)) < 0.5))
    c1 = c_idx - disp[r_idx, c_idx]
    ok = (c1 >= 0) & (c1 < cols)
    noise = rng.integers(-4, 5, size=(n, ok.sum()))
    s1[:, r_idx[ok], c1[ok]] = np.clip(s0[:, r_idx[ok], c_idx[ok]].astype(np.int64) + noise, 0,
                                       np.iinfo(dt).max).astype(dt)
    return s0, s1, disp


@pytest.mark.parametrize("dt", [np.uint8, np.uint16])
@pytest.mark.parametrize("n", [2, 5, 10, 16, 24, 33, 40, 65])
@pytest.mark.parametrize("double", [False, True])
def test_agree_vs_oracle(cuda, oracle, dt, n, double):
    rng = np.random.default_rng(n + 100 * double)
    s0, s1, disp = _case(rng, dt, n, 9, 203)
    for thr, mv in ((0.5, None), (0.9, 2.0 * n), (-0.5, 75.0 * n)):
        d, corr = lbg.agree(dev(disp, cuda), dev(s0, cuda), dev(s1, cuda), thr, mv, double)
        wd, wc = oracle.agree(disp, s0, s1, thr, mv, double)
        assert_same(host(d), wd, f"disp n={n} thr={thr}")
        assert_same(host(corr), wc, f"corr n={n} thr={thr}")


@pytest.mark.parametrize("dt", [np.uint8, np.uint16])
@pytest.mark.parametrize("n", [3, 10, 12, 33, 48])
@pytest.mark.parametrize("step", [0.1, 0.25, 0.5, 0.01])
@pytest.mark.parametrize("double", [False, True])
def test_agree_subpixel_vs_oracle(cuda, oracle, dt, n, step, double):
    rng = np.random.default_rng(n * 3 + int(step * 100) + 7 * double)
    s0, s1, disp = _case(rng, dt, n, 5, 150)
    for thr, mv in ((0.5, None), (0.9, 2.0 * n)):
        d, corr = lbg.agree_subpixel(dev(disp, cuda), dev(s0, cuda), dev(s1, cuda), thr, step, mv, double)
        wd, wc = oracle.agree_subpixel(disp, s0, s1, thr, step, mv, double)
        assert_same(host(d), wd, f"disp n={n} step={step}")
        assert_same(host(corr), wc, f"corr n={n} step={step}")
