"""Pins the oracle restatement to libBICOS's own CPU backend on seeded
random inputs.  Runs only where the reference CPU build (oracle/_ref) can be
made from the reference sources; elsewhere the golden vectors carry the pin."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def ref(oracle):
    if not oracle.ref_available():
        try:
            oracle.build_ref()
        except Exception:
            pass
    if not oracle.ref_available():
        pytest.skip("reference CPU build unavailable (no reference sources on this host)")
    return oracle


@pytest.mark.parametrize("dt", [np.uint8, np.uint16])
@pytest.mark.parametrize("full", [False, True])
def test_transform_matches_reference(ref, dt, full):
    rng = np.random.default_rng(11 + full)
    ns = range(2, 66) if not full else range(2, 17)
    for n in ns:
        s = rng.integers(0, np.iinfo(dt).max + 1, size=(n, 3, 17), dtype=dt)
        nw = ref.descriptor_words(ref.required_bits(n, full))
        assert np.array_equal(ref.transform(s, full, nw), ref.transform(s, full, nw, use_ref=True)), n


@pytest.mark.parametrize("nw", [1, 2, 4, 8])
def test_search_matches_reference(ref, nw):
    rng = np.random.default_rng(nw)
    for flags in (0, 1, 2, 3):
        for lr in (0, 1, 3):
            d0 = rng.integers(0, 64, size=(5, 97, nw), dtype=np.uint32)
            d1 = rng.integers(0, 64, size=(5, 97, nw), dtype=np.uint32)
            assert np.array_equal(ref.search(d0, d1, flags, lr), ref.search(d0, d1, flags, lr, use_ref=True))


def test_match_matches_reference(ref):
    from libbicos_gb300 import scenes
    for seed, bits in ((3, 8), (4, 12)):
        sc = scenes.make_scene(20, 150, 12, seed=seed, bits=bits)
        for thr in (None, 0.5, 0.9):
            for step in (None, 0.1, 0.25, 0.3):
                for mv in (None, 2.0):
                    for cons in (None, (1, False), (2, True), (0, False)):
                        for full in (False, True):
                            cfg = ref.make_config(threshold=thr, step=step, min_variance=mv, consistency=cons,
                                                  full=full)
                            a, ca = ref.match(sc.left, sc.right, cfg)
                            b, cb = ref.match(sc.left, sc.right, cfg, use_ref=True)
                            assert np.array_equal(a, b, equal_nan=True)
                            if ca is not None:
                                assert np.array_equal(ca, cb, equal_nan=True)


def test_errors_match_reference(ref):
    s = np.zeros((66, 4, 8), np.uint8)
    cfg = ref.make_config()
    for use_ref in (False, True):
        with pytest.raises(ref.OracleError, match="would require 257 bits") as e:
            ref.match(s, s, cfg, use_ref=use_ref)
        assert e.value.code == ref.ERR_INVALID_ARGUMENT
    cfg = ref.make_config(full=True)
    s = np.zeros((17, 4, 8), np.uint8)
    for use_ref in (False, True):
        with pytest.raises(ref.OracleError, match="would require 258 bits"):
            ref.match(s, s, cfg, use_ref=use_ref)


def test_golden_files_regenerate(ref):
    """tests/golden/*.npz are what tests/golden/make_golden.py computes from
    the reference build: regenerated here in memory, every array equal."""
    import importlib.util
    import os
    from conftest import ROOT
    path = os.path.join(ROOT, "tests", "golden", "make_golden.py")
    spec = importlib.util.spec_from_file_location("make_golden", path)
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    rng = np.random.default_rng(20241203)  # the generator's seed, in its call order
    fresh = {"transform": mg.transform_cases(rng), "search": mg.search_cases(rng),
             "agree": mg.agree_cases(rng), "match": mg.match_cases()}
    for name, arrays in fresh.items():
        with np.load(os.path.join(ROOT, "tests", "golden", name + ".npz")) as z:
            assert sorted(z.files) == sorted(arrays), name
            for k, v in arrays.items():
                want = np.asarray(v)
                assert np.array_equal(z[k], want, equal_nan=want.dtype.kind in "fc"), (name, k)
