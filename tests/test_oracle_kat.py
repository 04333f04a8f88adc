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
  truncates, and |col0 - rev| > max_lr_diff invalidates.
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
