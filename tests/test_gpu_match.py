"""The whole matching path on the GPU through each public entry point --
C ABI (bicos_match_v1 via match_device), pybicos over host arrays
(bicos_match_host_v1), and the C++ BICOS::match -- vs the oracle and the
reference's golden vectors."""
import os
import subprocess

import numpy as np
import pytest

import libbicos_gb300 as lbg
from conftest import ROOT, golden
from gpu_util import assert_same, dev, host
from libbicos_gb300 import pybicos, scenes

pytestmark = pytest.mark.gpu


def py_cfg(thr=0.5, step=None, mv=None, full=False, cons=None, double=False):
    c = pybicos.Config()
    c.nxcorr_threshold = thr
    c.subpixel_step = step
    c.min_variance = mv
    c.mode = pybicos.Full if full else pybicos.Limited
    c.precision = pybicos.Double if double else pybicos.Single
    c.variant = pybicos.Variant.NoDuplicates() if cons is None else pybicos.Variant.Consistency(*cons)
    return c


def golden_cases():
    z = golden("match.npz")
    for c in sorted({k.split("_")[0] for k in z.files if k.startswith("m")}, key=lambda s: int(s[1:])):
        thr, step, mv, full, lr, nd = z[c + "_cfg"]
        cfg = py_cfg(None if np.isnan(thr) else float(thr), None if np.isnan(step) else float(step),
                     None if np.isnan(mv) else float(mv), bool(full), None if lr < 0 else (int(lr), bool(nd)))
        label = str(z[c + "_scene"])
        yield c, z[label + "_left"], z[label + "_right"], cfg, z[c + "_disp"], z.get(c + "_corr")


def test_match_device_golden(cuda):
    for c, left, right, cfg, wd, wc in golden_cases():
        d, corr = lbg.match_device(dev(left, cuda), dev(right, cuda), cfg)
        assert_same(host(d), wd, c)
        if wc is not None:
            assert_same(host(corr), wc, c + " corrmap")
        else:
            assert corr is None


def test_pybicos_golden(cuda):
    for c, left, right, cfg, wd, wc in golden_cases():
        d, corr = pybicos.match(list(left), list(right), cfg)
        assert_same(d, wd, c)
        if wc is not None:
            assert_same(corr, wc, c + " corrmap")


def _ocfg(oracle, thr=0.5, step=None, mv=None, full=False, cons=None, double=False, max_bits=256):
    return oracle.make_config(threshold=thr, step=step, min_variance=mv, full=full, consistency=cons,
                              double=double, max_bits=max_bits)


@pytest.mark.parametrize("double", [False, True])
@pytest.mark.parametrize("cons", [None, (1, False), (2, True)])
@pytest.mark.parametrize("step", [None, 0.1])
def test_vga_scene_vs_oracle(cuda, oracle, double, cons, step):
    """640x480, n=12, limited (the small seeded workload), both precisions"""
    sc = scenes.workload_scene("vga_n12", seed=1)
    d, corr = lbg.match_device(dev(sc.left, cuda), dev(sc.right, cuda),
                               py_cfg(0.9, step, 2.0, cons=cons, double=double))
    wd, wc = oracle.match(sc.left, sc.right, _ocfg(oracle, 0.9, step, 2.0, cons=cons, double=double))
    assert_same(host(d), wd, "disparity")
    assert_same(host(corr), wc, "corrmap")


@pytest.mark.parametrize("n,full", [(2, False), (3, True), (16, True), (65, False), (9, False), (10, False)])
def test_edge_stack_sizes(cuda, oracle, n, full):
    sc = scenes.make_scene(24, 97, n, seed=n, bits=8)
    for step in (None, 0.25):
        d, corr = lbg.match_device(dev(sc.left, cuda), dev(sc.right, cuda), py_cfg(0.5, step, full=full))
        wd, wc = oracle.match(sc.left, sc.right, _ocfg(oracle, 0.5, step, full=full))
        assert_same(host(d), wd, f"n={n}")
        assert_same(host(corr), wc, f"n={n} corr")


@pytest.mark.parametrize("n", [9, 17, 33])
def test_periodic_texture_ties(cuda, oracle, n):
    """column-periodic stacks (every descriptor repeats every 7 columns) on
    4096-column rows: the search's column-coded keys must pick the
    reference's first minimum and flag every duplicate (n = 9, 17, 33 use
    30, 62 and 126 of 32, 64 and 128 bit positions: exactly the two spare
    slots the code needs)"""
    rng = np.random.default_rng(n)
    base = rng.integers(0, 256, size=(n, 1, 7), dtype=np.uint8)
    left = np.tile(base, (1, 3, 586))[:, :, :4096].copy()
    right = np.roll(left, 3, axis=2).copy()
    left[:, 1, 1000] ^= 0x55  # one unique texel in the middle row
    # binary random frames: many partial ties
    bl = rng.integers(0, 2, size=(n, 2, 4096), dtype=np.uint8)
    br = np.roll(bl, 5, axis=2).copy()
    for sl, sr in ((left, right), (bl, br)):
        for cons in (None, (1, False), (2, True)):
            for thr in (None, 0.5):
                d, corr = lbg.match_device(dev(sl, cuda), dev(sr, cuda), py_cfg(thr, cons=cons))
                wd, wc = oracle.match(sl, sr, _ocfg(oracle, thr, cons=cons))
                assert_same(host(d), wd, f"n={n} cons={cons} thr={thr}")
                if thr is not None:
                    assert_same(host(corr), wc, f"n={n} cons={cons} corr")


def test_no_threshold_returns_raw_int16(cuda, oracle):
    sc = scenes.make_scene(16, 120, 8, seed=5)
    d, corr = lbg.match_device(dev(sc.left, cuda), dev(sc.right, cuda), py_cfg(None))
    assert corr is None and str(d.dtype) == "torch.int16"
    wd, _ = oracle.match(sc.left, sc.right, _ocfg(oracle, None))
    assert_same(host(d), wd)
    dp, cp = pybicos.match(list(sc.left), list(sc.right), py_cfg(None))
    assert cp is None
    assert_same(dp, wd)


def test_u16_full_12bit(cuda, oracle):
    sc = scenes.make_scene(40, 200, 16, seed=2, bits=12)
    for cons in (None, (1, False)):
        d, corr = lbg.match_device(dev(sc.left, cuda), dev(sc.right, cuda), py_cfg(0.9, 0.1, full=True, cons=cons))
        wd, wc = oracle.match(sc.left, sc.right, _ocfg(oracle, 0.9, 0.1, full=True, cons=cons))
        assert_same(host(d), wd)
        assert_same(host(corr), wc)


def test_full_mode_beyond_256_bits(cuda, oracle):
    """extension: FULL n=20 (363 bits) with max_bits=512, vs the generalised oracle"""
    sc = scenes.make_scene(20, 160, 20, seed=3, bits=12)
    with pytest.raises(ValueError, match="would require 363 bits"):
        lbg.match_device(dev(sc.left, cuda), dev(sc.right, cuda), py_cfg(0.9, 0.1, full=True))
    d, corr = lbg.match_device(dev(sc.left, cuda), dev(sc.right, cuda), py_cfg(0.9, 0.1, full=True, cons=(1, False)),
                               max_bits=512)
    wd, wc = oracle.match(sc.left, sc.right, _ocfg(oracle, 0.9, 0.1, full=True, cons=(1, False), max_bits=512))
    assert_same(host(d), wd)
    assert_same(host(corr), wc)


def test_production_size_rows_vs_oracle(cuda, oracle):
    """1936x1216, n=33 (the production workload) on the GPU; every stage is
    row-local, so oracle rows computed alone must equal the GPU rows."""
    sc = scenes.workload_scene("mv1936_n33", seed=0)
    for double in (False, True):
        d, corr = lbg.match_device(dev(sc.left, cuda), dev(sc.right, cuda), py_cfg(0.96, 0.1, 2.0, double=double))
        d, corr = host(d), host(corr)
        rows = [0, 1, 607, 1215] + list(np.random.default_rng(double).integers(0, 1216, 6))
        for r in rows:
            wd, wc = oracle.match(sc.left[:, r:r + 1], sc.right[:, r:r + 1],
                                  _ocfg(oracle, 0.96, 0.1, 2.0, double=double))
            assert_same(d[r:r + 1], wd, f"row {r}")
            assert_same(corr[r:r + 1], wc, f"row {r} corr")
        # size-independent properties of the whole map
        valid = np.isfinite(d)
        assert valid.mean() > 0.5
        assert np.all(corr[valid] >= np.float32(0.96))
        assert np.nanmax(np.abs(d - sc.disparity)) < 300


def test_cpp_api(cuda, oracle, tmp_path):
    """BICOS::match from C++ (g++ against include/BICOS, linked to the library)"""
    from libbicos_gb300 import build
    exe = tmp_path / "match_cpp"
    libdir = os.path.dirname(build.LIB)
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "match_cpp.cpp"), "-L", libdir, "-lbicos_gb300",
                    "-Wl,-rpath," + libdir, "-o", str(exe)], check=True)
    sc = scenes.make_scene(30, 140, 12, seed=4)
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        f.write(np.array([12, 30, 140], np.int32).tobytes())
        f.write(sc.left.tobytes())
        f.write(sc.right.tobytes())
    for mode, (step, cons) in enumerate(((None, None), (0.1, None), (None, (1, True)))):
        out = tmp_path / f"out{mode}.bin"
        r = subprocess.run([str(exe), str(inp), str(out), str(mode)])
        assert r.returncode == 0, r.returncode
        raw = out.read_bytes()
        wd, wc = oracle.match(sc.left, sc.right, _ocfg(oracle, 0.9, step, 2.0, cons=cons))
        nd = wd.nbytes
        assert_same(np.frombuffer(raw[:nd], wd.dtype).reshape(wd.shape), wd, f"mode {mode}")
        assert_same(np.frombuffer(raw[nd:], np.float32).reshape(wc.shape), wc, f"mode {mode} corr")


def test_streams_and_reuse(cuda, oracle):
    """calls on two streams share the scratch cache without races"""
    import torch
    sc_a = scenes.make_scene(64, 256, 12, seed=10)
    sc_b = scenes.make_scene(80, 300, 16, seed=11)
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    la, ra, lb, rb = (dev(x, cuda) for x in (sc_a.left, sc_a.right, sc_b.left, sc_b.right))
    torch.cuda.synchronize()
    outs = []
    for i in range(4):
        st = s1 if i % 2 == 0 else s2
        with torch.cuda.stream(st):
            outs.append(lbg.match_device(la if i % 2 == 0 else lb, ra if i % 2 == 0 else rb, py_cfg(0.9, 0.1),
                                         stream=st))
    torch.cuda.synchronize()
    wa, _ = oracle.match(sc_a.left, sc_a.right, _ocfg(oracle, 0.9, 0.1))
    wb, _ = oracle.match(sc_b.left, sc_b.right, _ocfg(oracle, 0.9, 0.1))
    for i, (d, _) in enumerate(outs):
        assert_same(host(d), wa if i % 2 == 0 else wb, f"call {i}")


@pytest.mark.parametrize("layout", ["stack", "frames", "pitched"])
def test_host_path_row_bands_equal_device(cuda, layout):
    """bicos_match_host_v1 splits images of >= 32 M samples into row bands
    with overlapped uploads: every layout of the host frames (one evenly
    spaced stack, separate frame buffers, pitched rows) gives the device
    path's results bit for bit"""
    import libbicos_gb300 as lbg
    from gpu_util import dev, host
    from libbicos_gb300 import pybicos, scenes
    sc = scenes.make_scene(1024, 1024, 33, seed=17)
    c = pybicos.Config()
    c.nxcorr_threshold = 0.9
    c.subpixel_step = 0.1
    c.min_variance = 2.0
    if layout == "stack":
        f0, f1 = list(sc.left), list(sc.right)
    elif layout == "frames":
        f0 = [np.ascontiguousarray(a) for a in sc.left]
        f1 = [np.ascontiguousarray(a) for a in sc.right]
    else:
        pad0 = np.zeros((33, 1024, 1024 + 40), np.uint8)
        pad1 = np.zeros((33, 1024, 1024 + 40), np.uint8)
        pad0[:, :, :1024] = sc.left
        pad1[:, :, :1024] = sc.right
        f0, f1 = list(pad0[:, :, :1024]), list(pad1[:, :, :1024])
    d, corr = pybicos.match(f0, f1, c)
    wd, wc = lbg.match_device(dev(sc.left, cuda), dev(sc.right, cuda), c)
    assert_same(d, host(wd), "disparity")
    assert_same(corr, host(wc), "corrmap")
