"""Property test: the oracle restatement equals libBICOS's own CPU backend
(compiled from its sources into oracle/_ref) on generated cases over
(n, mode, sample type, rows, cols, variant, threshold, step, min_variance),
bit for bit, disparity and correlation map.  Runs where both the reference
build and hypothesis exist; the seeded cases of test_ref_pin.py and the
golden vectors cover the other hosts."""
import numpy as np
import pytest

hypothesis = pytest.importorskip("hypothesis")
from hypothesis import HealthCheck, given, settings  # noqa: E402
from hypothesis import strategies as st  # noqa: E402


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


@st.composite
def cases(draw):
    full = draw(st.booleans())
    n = draw(st.integers(2, 16 if full else 65))
    u16 = draw(st.booleans())
    rows, cols = draw(st.integers(1, 5)), draw(st.integers(1, 80))
    seed = draw(st.integers(0, 2 ** 31 - 1))
    variant = draw(st.sampled_from([None, (1, False), (2, True), (0, False), (5, True)]))
    thr = draw(st.sampled_from([None, -1.0, 0.0, 0.5, 0.9]))
    step = draw(st.sampled_from([None, 0.1, 0.25, 0.5, 0.3]))
    minvar = draw(st.sampled_from([None, 0.0, 2.0, 40.0]))
    # textured left frames; the right side is the left shifted by a few
    # columns plus noise (valid matches), with flat patches (variance mask,
    # duplicate costs) and, for some cases, a small value range (many ties)
    rng = np.random.default_rng(seed)
    top = draw(st.sampled_from([4, 256, 4096 if u16 else 256, 65536 if u16 else 256]))
    dt = np.uint16 if u16 else np.uint8
    left = rng.integers(0, top, size=(n, rows, cols + 8))
    shift = int(rng.integers(0, 8))
    right = np.roll(left, shift, axis=2) + rng.integers(-2, 3, size=left.shape)
    left, right = left[:, :, :cols], np.clip(right[:, :, :cols], 0, top - 1)
    if cols > 4:
        c0 = int(rng.integers(0, cols - 3))
        left[:, :, c0:c0 + 3] = int(rng.integers(0, top))
    return (left.astype(dt), right.astype(dt), full, variant, thr, step, minvar)


@settings(max_examples=300, deadline=None, derandomize=True,
          suppress_health_check=[HealthCheck.function_scoped_fixture])
@given(case=cases())
def test_restatement_equals_reference(ref, case):
    left, right, full, variant, thr, step, minvar = case
    cfg = ref.make_config(threshold=thr, step=step, min_variance=minvar, full=full, consistency=variant)
    want = ref.match(left, right, cfg, use_ref=True)
    got = ref.match(left, right, cfg)
    assert np.array_equal(got[0], want[0], equal_nan=True)
    if want[1] is None:
        assert got[1] is None
    else:
        assert np.array_equal(got[1], want[1], equal_nan=True)
