"""Learned subpixel form, host side: the FP64 network oracle pinned by
finite differences, the model file format, and the library's model store
(parsing, validation, install/uninstall) -- no GPU needed."""
import os

import numpy as np
import pytest

from oracle import mlp
from libbicos_gb300 import learned


def _model(seed=0):
    rng = np.random.default_rng(seed)
    p = learned.init_params(seed).astype(np.float64)
    p += rng.normal(0, 0.05, p.shape)  # nonzero biases
    mean = rng.normal(0, 0.3, 7)
    std = rng.uniform(0.5, 2.0, 7)
    return np.concatenate([p, mean, std])


def _samples(count, seed=1):
    rng = np.random.default_rng(seed)
    s = np.empty((count, 8))
    s[:, 2] = rng.uniform(0.5, 1.0, count)
    for k in (0, 1, 3, 4):
        s[:, k] = s[:, 2] - rng.uniform(0.0, 0.3, count)
    s[rng.random(count) < 0.05, 0] = np.nan  # missing rho(-2): counts as -1
    s[:, 5] = rng.uniform(10, 3000, count)
    s[:, 6] = rng.uniform(10, 3000, count)
    s[:, 7] = rng.uniform(-1, 1, count)
    return s


def test_layout_matches_library(native):
    a, b = native.C.c_int(), native.C.c_int()
    native.load().bicos_mlp_sizes(native.C.byref(a), native.C.byref(b))
    assert (a.value, b.value) == (mlp.N_PARAMS, mlp.MODEL_FLOATS) == (learned.N_PARAMS, learned.MODEL_FLOATS)


def test_oracle_gradient_finite_differences():
    """the FP64 gradient the kernels are checked against, checked itself by
    central differences on every parameter of a 12-sample batch"""
    model, s = _model(), _samples(12)
    _, g = mlp.loss_and_grad(model, s)
    h = 1e-6
    fd = np.empty(mlp.N_PARAMS)
    for i in range(mlp.N_PARAMS):
        mp, mm = model.copy(), model.copy()
        mp[i] += h
        mm[i] -= h
        fd[i] = (mlp.loss_and_grad(mp, s)[0] - mlp.loss_and_grad(mm, s)[0]) / (2 * h)
    err = np.abs(fd - g)
    assert err.max() <= 1e-6 * max(1.0, np.abs(g).max()), err.max()


def test_oracle_adam_matches_formula():
    p, g = np.array([1.0, -2.0]), np.array([0.5, -4.0])
    p1, m, v = mlp.adam_step(p, g, np.zeros(2), np.zeros(2), 1, 0.01, 1.0)
    # the first bias-corrected step moves each parameter by lr * sign(g)
    assert np.allclose(p1, p - 0.01 * np.sign(g), atol=1e-9)


def test_model_file_round_trip():
    rng = np.random.default_rng(3)
    params = rng.normal(0, 1, learned.N_PARAMS).astype(np.float32)
    mean, std = rng.normal(0, 1, 7).astype(np.float32), rng.uniform(0.1, 2, 7).astype(np.float32)
    data = learned.model_bytes(params, mean, std)
    assert data[:8] == b"BICOSMLP" and len(data) == 24 + 56 + 2 * learned.N_PARAMS
    p2, m2, s2 = learned.parse_model(data)
    assert np.array_equal(p2, mlp.bf16(params)) and np.array_equal(m2, mean) and np.array_equal(s2, std)


@pytest.fixture
def restore_model():
    yield
    data = open(learned.MODEL_PATH, "rb").read() if os.path.exists(learned.MODEL_PATH) else None
    learned.install(data)


def test_library_model_store(native, restore_model):
    rng = np.random.default_rng(4)
    params = rng.normal(0, 1, learned.N_PARAMS).astype(np.float32)
    mean, std = rng.normal(0, 1, 7).astype(np.float32), rng.uniform(0.1, 2, 7).astype(np.float32)
    learned.install(learned.model_bytes(params, mean, std))
    assert native.load().bicos_learned_model_installed() == 1
    got = learned.installed_model()
    assert np.array_equal(got, learned.model_floats(mlp.bf16(params), mean, std))
    learned.install(None)
    assert native.load().bicos_learned_model_installed() == 0
    with pytest.raises(native.NativeError, match="no learned subpixel model"):
        learned.installed_model()


@pytest.mark.parametrize("damage,message", [
    (lambda d: b"X" + d[1:], "not a BICOSMLP file"),
    (lambda d: d[:8] + (2).to_bytes(4, "little") + d[12:], "unsupported version 2"),
    (lambda d: d[:12] + (8).to_bytes(4, "little") + d[16:], "does not match the network"),
    (lambda d: d[:-2], "size"),
    (lambda d: d[:24 + 28] + np.float32(-1).tobytes() + d[24 + 32:], "normalisation"),
])
def test_library_rejects_bad_files(native, restore_model, damage, message):
    data = learned.model_bytes(np.zeros(learned.N_PARAMS, np.float32), np.zeros(7, np.float32),
                               np.ones(7, np.float32))
    with pytest.raises(native.NativeError, match=message) as e:
        learned.install(damage(data))
    assert e.value.status == native.ERR_INVALID_ARGUMENT


def test_committed_model_is_valid():
    if not os.path.exists(learned.MODEL_PATH):
        pytest.skip("no trained model file in the package")
    params, mean, std = learned.parse_model(open(learned.MODEL_PATH, "rb").read())
    assert np.all(np.isfinite(params)) and np.all(std > 0)


def test_proposal_accuracy_against_sweep_grid(oracle):
    """Why the learned form keeps one check: its subpixel error against the
    FP64 step-0.01 sweep, on 48 rows of the 1936x1216 n=33 workload, when
    the proposal is used as is, or snapped to the best of the 2 or 4 step-0.1
    sweep positions around it (each position evaluated in the reference's
    arithmetic, here through the oracle's check with no rejection).  Only
    the 4-position window approaches the plain step-0.1 sweep -- at four
    reference evaluations per pixel on top of the network, more than the
    sweep it would replace."""
    from libbicos_gb300 import scenes
    sc = scenes.workload_scene("mv1936_n33", seed=3, rows=48)
    n = sc.left.shape[0]
    thr, mv = 0.96, 2.0 * n
    raw, _ = oracle.match(sc.left, sc.right, oracle.make_config(threshold=None))
    ref, _ = oracle.agree_subpixel(raw, sc.left, sc.right, thr, 0.01, mv, double=True)
    plain, _ = oracle.agree_subpixel(raw, sc.left, sc.right, thr, 0.1, mv)
    feats = oracle.features(raw, sc.left, sc.right)
    path = os.path.join(os.path.dirname(learned.__file__), "learned_subpixel.bsm")
    model = learned.model_floats(*learned.parse_model(open(path, "rb").read()))
    rows, cols = raw.shape
    prop = mlp.propose(model, feats.reshape(-1, 8)).reshape(rows, cols).astype(np.float32)
    xs = [np.float32(-1.0)]
    while np.float32(xs[-1] + np.float32(0.1)) <= 1.0:
        xs.append(np.float32(xs[-1] + np.float32(0.1)))
    xs = np.array(xs, np.float32)
    # rho at every sweep position, the reference's float arithmetic
    rho = np.stack([oracle.learned_check(raw, sc.left, sc.right, -1.0, np.full((rows, cols), x, np.float32), feats,
                                         mv, False, drop=1e30)[1] for x in xs])
    col1 = np.arange(cols)[None, :] - raw.astype(np.int64)
    inner = (raw != -32768) & (col1 >= 1) & (col1 <= cols - 2) & np.isfinite(ref) & np.isfinite(plain)
    d = raw.astype(np.float32)
    kbest = np.argmax(np.where(np.isfinite(rho), rho, -2.0), axis=0)  # the sweep's first maximum

    def window(lo, w):
        lo = np.clip(lo, 0, len(xs) - w)
        r = np.stack([np.take_along_axis(rho, (lo + j)[None], 0)[0] for j in range(w)])
        return lo + np.argmax(np.where(np.isfinite(r), r, -2.0), axis=0)

    below = np.clip(np.searchsorted(xs, prop, side="right") - 1, 0, len(xs) - 2)
    k2, k4 = window(below, 2), window(below - 1, 4)

    def rms(v):
        return float(np.sqrt(np.mean((v[inner] - ref[inner]) ** 2)))
    e = {"plain sweep": rms(plain), "proposal": rms(d - prop), "best of 2": rms(d - xs[k2]),
         "best of 4": rms(d - xs[k4])}
    agree = {"best of 2": float(np.mean((k2 == kbest)[inner])), "best of 4": float(np.mean((k4 == kbest)[inner]))}
    print(f"\nRMS vs FP64 step-0.01 sweep (px): {e}; same position as the sweep: {agree}")
    assert abs(rms(d - xs[kbest]) - e["plain sweep"]) < 1e-6  # the table reproduces the sweep
    assert e["plain sweep"] <= e["best of 4"] < e["best of 2"] < e["proposal"]
    assert agree["best of 2"] < agree["best of 4"] < 1.0
