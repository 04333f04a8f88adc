"""The CPU oracle reproduces every golden vector made by libBICOS's own CPU
backend (tests/golden/make_golden.py), bit for bit."""
import numpy as np
import pytest

from conftest import golden


def _cases(z, prefix, key):
    return sorted({k.split("_")[0] for k in z.files if k.startswith(prefix) and k.endswith(key)},
                  key=lambda s: int(s[1:]))


def test_transform_golden(oracle):
    z = golden("transform.npz")
    cases = _cases(z, "t", "_stack")
    assert len(cases) == 42
    for c in cases:
        s, d, full = z[c + "_stack"], z[c + "_desc"], bool(z[c + "_full"])
        out = oracle.transform(s, full, d.shape[-1])
        assert np.array_equal(out, d), c


def test_search_golden(oracle):
    z = golden("search.npz")
    cases = _cases(z, "s", "_d0")
    assert len(cases) == 32
    for c in cases:
        out = oracle.search(z[c + "_d0"], z[c + "_d1"], int(z[c + "_flags"]), int(z[c + "_lr"]))
        assert np.array_equal(out, z[c + "_disp"]), c


def test_agree_golden(oracle):
    z = golden("agree.npz")
    cases = _cases(z, "a", "_s0")
    assert len(cases) == 12
    for c in cases:
        thr, step, mv = float(z[c + "_thr"]), float(z[c + "_step"]), float(z[c + "_minvar"])
        mv = None if mv < 0 else mv
        if step < 0:
            d, corr = oracle.agree(z[c + "_raw"], z[c + "_s0"], z[c + "_s1"], thr, mv)
        else:
            d, corr = oracle.agree_subpixel(z[c + "_raw"], z[c + "_s0"], z[c + "_s1"], thr, step, mv)
        assert np.array_equal(d, z[c + "_disp"], equal_nan=True), c
        assert np.array_equal(corr, z[c + "_corr"], equal_nan=True), c


def match_cfg(oracle, v, double=False):
    thr, step, mv, full, lr, nd = v
    return oracle.make_config(threshold=None if np.isnan(thr) else float(thr),
                              step=None if np.isnan(step) else float(step),
                              min_variance=None if np.isnan(mv) else float(mv), full=bool(full),
                              consistency=None if lr < 0 else (int(lr), bool(nd)), double=double)


def test_match_golden(oracle):
    z = golden("match.npz")
    cases = _cases(z, "m", "_cfg")
    assert len(cases) == 24
    for c in cases:
        label = str(z[c + "_scene"])
        d, corr = oracle.match(z[label + "_left"], z[label + "_right"], match_cfg(oracle, z[c + "_cfg"]))
        assert np.array_equal(d, z[c + "_disp"], equal_nan=True), c
        if c + "_corr" in z.files:
            assert np.array_equal(corr, z[c + "_corr"], equal_nan=True), c
        else:
            assert corr is None


def test_double_nxcorr_close_to_float(oracle):
    """The FP64 restatement (agree.cuh:35-65) agrees with the float one to FP32 accuracy."""
    rng = np.random.default_rng(5)
    for _ in range(200):
        n = int(rng.integers(2, 66))
        x = rng.integers(0, 256, n).astype(np.float64)
        y = (x + rng.normal(0, 20, n)).clip(0, 255).round()
        f, d = oracle.nxcorr_f(x, y), oracle.nxcorr_d(x, y)
        if np.isfinite(d):
            assert abs(f - d) <= 1e-5


def test_oracle_independent_of_threads(oracle):
    """The restatement splits rows over threads (the CPU baseline uses all
    cores); every stage gives the same bits with 1, 3 or all threads."""
    from libbicos_gb300 import scenes
    sc = scenes.make_scene(37, 90, 12, seed=21)
    runs = []
    for nt in (1, 3, 0):
        cfg = oracle.make_config(threshold=0.9, step=0.1, min_variance=2.0)
        d, c = oracle.match(sc.left, sc.right, cfg, nthreads=nt)
        desc = oracle.transform(sc.left, False, nthreads=nt)
        cons = oracle.match(sc.left, sc.right, oracle.make_config(threshold=0.5, consistency=(1, True)),
                            nthreads=nt)[0]
        runs.append((d, c, desc, cons))
    for r in runs[1:]:
        for a, b in zip(runs[0], r):
            assert np.array_equal(a, b, equal_nan=True)
