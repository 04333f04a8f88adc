"""Known-answer tests, worked out by hand from libBICOS's rules, that pin
the oracle independently of the reference build:

* limited descriptors for n = 2..5 (include/impl/cpu/descriptor_transform.hpp
  :32-73): three bits per step t < n-2 (a<b, a<c, a<mean), a pair-sum bit
  once the sum two steps back exists (the ring starts at -1 = absent), then
  the tail a<b, a<mean, b<mean and "sum two steps back < a+b" (always set
  when that sum is absent, -1 being below any sum);
* full descriptors for n = 2..5 (descriptor_transform.hpp:75-123): the same
  per-step and tail bits, then sum[t] < sum[i] for every ordered pair of
  adjacent-pair sums at least two apart;
* the search (include/impl/cpu/bicos.hpp:50-113): the first minimum wins;
  with no-duplicates a later equal cost invalidates, but only one seen after
  the last new minimum; the consistency average (col0 + rev) / 2 - best
  truncates, and |col0 - rev| > max_lr_diff invalidates;
* the agreement (include/impl/cpu/agree.hpp:27-185): exact NCC values, the
  strict variance mask, NaN passing the threshold, out-of-range and border
  columns, and the sweep's first strictly-better offset on an exact grid.
"""
import numpy as np
import pytest

INV = -32768


def _transform_cases():
    # (pixel sequence, descriptor bits as an integer), each derived by hand:
    return [
        ([10, 20], 0b1011),      # 10<20, 10<15, not 20<15, -1 < 30
        ([20, 10], 0b1100),      # only 10<15 and the absent-sum bit
        ([7, 7], 0b1000),        # ties set nothing; mean 7
        ([1, 5, 3], 0b1000111),  # t=0: 1<5, 1<3, 1<3; tail: none, -1 < 8
        ([4, 2, 6, 0], 298),     # bits 1 (4<6), 3 (2<6), 5 (2<3), 8 (0<3); 6 < 6 is false
        ([1, 2, 3, 4, 5], 9983),  # bits 0..7, 9 (3 < 7), 10 (4<5), 13 (5 < 9)
    ]


@pytest.mark.parametrize("pix,want", _transform_cases())
def test_limited_descriptor_kat(oracle, pix, want):
    n = len(pix)
    stack = np.array(pix, dtype=np.uint8).reshape(n, 1, 1)
    d = oracle.transform(stack, False)
    assert d.shape == (1, 1, 1)
    assert int(d[0, 0, 0]) == want, (pix, bin(int(d[0, 0, 0])), bin(want))
    s16 = (stack.astype(np.uint16) * 16).astype(np.uint16)  # scaling keeps every comparison
    assert int(oracle.transform(s16, False)[0, 0, 0]) == want
    if oracle.ref_available():  # the reference's own CPU backend, where its sources exist
        assert int(oracle.transform(stack, False, use_ref=True)[0, 0, 0]) == want


def _rows(costs):
    """Query row of identical zero descriptors against candidates whose
    popcounts are `costs` (one 32-bit word each)."""
    cols = len(costs)
    d0 = np.zeros((1, cols, 1), np.uint32)
    d1 = np.array([(1 << c) - 1 for c in costs], np.uint32).reshape(1, cols, 1)
    return d0, d1


@pytest.mark.parametrize("costs,flags,lr,want", [
    # duplicated minimum (cost 1 at columns 1 and 2)
    ([3, 1, 1, 2, 4], 0, -1, [-1, 0, 1, 2, 3]),
    ([3, 1, 1, 2, 4], 1, -1, [INV] * 5),
    # a duplicate before a new minimum does not count
    ([2, 1, 3, 1, 0], 1, -1, [-4, -3, -2, -1, 0]),
    ([2, 1, 3, 1, 0], 0, -1, [-4, -3, -2, -1, 0]),
    # consistency: the reverse search over identical queries picks column 0;
    # (1 + 0) / 2 truncates to 0; columns farther than 1 from 0 are rejected
    ([2, 1, 3, 1, 0], 2, 1, [-4, -4, INV, INV, INV]),
    ([2, 1, 3, 1, 0], 2, 3, [-4, -4, -3, -3, INV]),
    # with no-duplicates the reverse search sees only ties: all invalid
    ([2, 1, 3, 1, 0], 3, 3, [INV] * 5),
])
def test_search_kat(oracle, costs, flags, lr, want):
    d0, d1 = _rows(costs)
    got = oracle.search(d0, d1, flags, lr)
    assert got.dtype == np.int16 and got.tolist() == [want]
    if oracle.ref_available():
        assert oracle.search(d0, d1, flags, lr, use_ref=True).tolist() == [want]


def _full_cases():
    # FULL mode (include/impl/cpu/descriptor_transform.hpp:75-123): the same
    # three bits per step t < n-2 and the tail a<b, a<mean, b<mean, then, for
    # every ordered pair (t, i) of the n-1 adjacent-pair sums with |t-i| >= 2,
    # t outer and i inner, the bit sum[t] < sum[i]; n^2 - 2n + 3 bits in all.
    return [
        ([10, 20], 0b011),       # tail only: 10<20, 10<15
        ([20, 10], 0b100),       # 10<15
        ([7, 7], 0),
        ([1, 5, 3], 0b000111),   # no pair of sums two apart exists for n=3
        ([4, 2, 6, 0], 298),     # bits 1, 3, 5, 8; sums 6, 8, 6: 6<6 twice false
        ([1, 2, 3, 4], 639),     # bits 0..6 and 9 (sum 3 < sum 7); 7 < 3 false
        ([1, 2, 3, 4, 5], 29439),     # bits 0..7, 9, 12, 13, 14
        ([5, 4, 3, 2, 1], 232448),    # bits 10, 11 (tail), 15, 16, 17
    ]


@pytest.mark.parametrize("pix,want", _full_cases())
def test_full_descriptor_kat(oracle, pix, want):
    n = len(pix)
    stack = np.array(pix, dtype=np.uint8).reshape(n, 1, 1)
    d = oracle.transform(stack, True)
    assert int(d[0, 0, 0]) == want, (pix, bin(int(d[0, 0, 0])), bin(want))
    assert want < (1 << (n * n - 2 * n + 3))  # nothing past the descriptor's bit count
    s16 = (stack.astype(np.uint16) * 16).astype(np.uint16)
    assert int(oracle.transform(s16, True)[0, 0, 0]) == want
    if oracle.ref_available():
        assert int(oracle.transform(stack, True, use_ref=True)[0, 0, 0]) == want


NAN = float("nan")


@pytest.mark.parametrize("x,y,min_var,want", [
    ([0, 2, 4], [1, 3, 5], None, 1.0),    # diffs equal: cov = var0 = var1 = 8
    ([0, 2, 4], [5, 3, 1], None, -1.0),
    ([0, 2, 4], [3, 1, 5], None, 0.5),    # cov 4, var 8 and 8
    ([0, 2, 4], [7, 7, 7], None, NAN),    # 0 / sqrt(0)
    ([0, 2, 4], [7, 7, 7], 1.0, -1.0),    # variance below the mask
    ([0, 2, 4], [1, 3, 5], 8.0, 1.0),     # the mask is strict: var 8 is not below 8
    ([0, 2, 4], [1, 3, 5], 8.5, -1.0),
])
def test_nxcorr_kat(oracle, x, y, min_var, want):
    """include/impl/cpu/agree.hpp:27-50: means, fused sums in frame order,
    then -1 under the (already n-scaled) variance mask."""
    for f in (oracle.nxcorr_f, oracle.nxcorr_d):
        got = f(np.array(x, float), np.array(y, float), min_var)
        assert (np.isnan(got) and np.isnan(want)) or got == want, (f.__name__, got, want)


def _agree_scene():
    """One row, five columns, n = 3; every left column holds (0, 2, 4)."""
    s0 = np.array([[0, 2, 4]] * 5, np.uint8).T.reshape(3, 1, 5)
    right = [[1, 3, 5], [5, 3, 1], [3, 1, 5], [7, 7, 7], [1, 3, 5]]
    s1 = np.array(right, np.uint8).T.reshape(3, 1, 5)
    return s0, s1


@pytest.mark.parametrize("min_var,want_d,want_c", [
    # col 0: d=-2 -> right col 2, rho 0.5, not below 0.5: kept
    # col 1: d=0 -> rho -1: invalid;  col 2: already invalid, no corrmap write
    # col 3: d=0 -> flat right column: rho NaN, which passes the threshold
    # col 4: d=5 -> right col -1: invalid, no corrmap write
    (None, [-2, INV, INV, 0, INV], [0.5, -1.0, NAN, NAN, NAN]),
    (1.0, [-2, INV, INV, INV, INV], [0.5, -1.0, NAN, -1.0, NAN]),
])
def test_agree_kat(oracle, min_var, want_d, want_c):
    """include/impl/cpu/agree.hpp:52-92."""
    s0, s1 = _agree_scene()
    disp = np.array([[-2, 0, INV, 0, 5]], np.int16)
    for double in (False, True):
        d, corr = oracle.agree(disp, s0, s1, 0.5, min_var, double=double)
        assert d.tolist() == [want_d]
        assert np.array_equal(corr[0], np.array(want_c), equal_nan=True), corr
    if oracle.ref_available():
        d, corr = oracle.agree(disp, s0, s1, 0.5, min_var, use_ref=True)
        assert d.tolist() == [want_d]
        assert np.array_equal(corr[0], np.array(want_c), equal_nan=True)


def _subpixel_scene():
    """Three rows, five columns, n = 3.  Right columns 1..3 of rows 0-1 are a
    linear ramp in x per frame (y0 + y2 = 2 y1, so the quadratic term is 0)
    and the interpolant round(b x + c) is exact on the 0.5 grid."""
    y0, y1, y2 = [0, 30, 10], [10, 20, 10], [20, 10, 10]
    s0 = np.zeros((3, 3, 5), np.uint8)
    s1 = np.zeros((3, 3, 5), np.uint8)
    # row 0: the left column equals the interpolant at x = +0.5 -> d - 0.5
    s1[:, 0, 1], s1[:, 0, 2], s1[:, 0, 3] = y0, y1, y2
    s0[:, 0, 3] = [15, 15, 10]
    # row 0 borders: right col 0 (rho 1) and right col 4 (rho -1), plain NCC
    s0[:, 0, 0], s1[:, 0, 0] = [0, 2, 4], [1, 3, 5]
    s0[:, 0, 4], s1[:, 0, 4] = [0, 2, 4], [5, 3, 1]
    # row 1: no gradient, every x ties at rho 1: the first, x = -1, is kept
    s1[:, 1, 1] = s1[:, 1, 2] = s1[:, 1, 3] = y1
    s0[:, 1, 3] = y1
    # row 2: a flat left column: under the mask every x gives -1 and none is
    # strictly better than the initial -1, so x stays 0
    s1[:, 2, 1], s1[:, 2, 2], s1[:, 2, 3] = y0, y1, y2
    s0[:, 2, 3] = [7, 7, 7]
    return s0, s1


@pytest.mark.parametrize("thr,min_var,want_d,want_c", [
    (0.5, 1.0,
     [[0.0, NAN, NAN, 0.5, NAN], [NAN, NAN, NAN, 2.0, NAN], [NAN, NAN, NAN, NAN, NAN]],
     [[1.0, NAN, NAN, 1.0, -1.0], [NAN, NAN, NAN, 1.0, NAN], [NAN, NAN, NAN, -1.0, NAN]]),
    (-1.0, 1.0,  # -1 is not below -1: the border and the masked pixel are kept
     [[0.0, NAN, NAN, 0.5, 0.0], [NAN, NAN, NAN, 2.0, NAN], [NAN, NAN, NAN, 1.0, NAN]],
     [[1.0, NAN, NAN, 1.0, -1.0], [NAN, NAN, NAN, 1.0, NAN], [NAN, NAN, NAN, -1.0, NAN]]),
])
def test_agree_subpixel_kat(oracle, thr, min_var, want_d, want_c):
    """include/impl/cpu/agree.hpp:94-185 with step 0.5 (x = -1, -0.5, 0, 0.5, 1)."""
    s0, s1 = _subpixel_scene()
    disp = np.full((3, 5), INV, np.int16)
    disp[0, 0] = 0   # right col 0: border
    disp[0, 3] = 1   # right col 2
    disp[0, 4] = 0   # right col 4: border
    disp[0, 2] = 5   # right col -3: out of range
    disp[1, 3] = 1
    disp[2, 3] = 1
    runs = [dict(double=False), dict(double=True)]
    if oracle.ref_available():
        runs.append(dict(use_ref=True))
    for kw in runs:
        out, corr = oracle.agree_subpixel(disp, s0, s1, thr, 0.5, min_var, **kw)
        assert np.array_equal(out, np.array(want_d, np.float32), equal_nan=True), (kw, out)
        assert np.array_equal(corr, np.array(want_c), equal_nan=True), (kw, corr)
