"""Hamming arg-min + postfilter on the GPU vs the oracle, bit-exact: every
descriptor width, flags 0/NODUPES/CONSISTENCY/both, tie-heavy inputs,
widths past one shared-memory chunk."""
import numpy as np
import pytest

import libbicos_gb300 as lbg
from conftest import golden
from gpu_util import assert_same, dev, host

pytestmark = pytest.mark.gpu


def _desc(rng, rows, cols, nw, bits=8):
    return rng.integers(0, 1 << bits, size=(rows, cols, nw), dtype=np.uint64).astype(np.uint32)


@pytest.mark.parametrize("nw", [1, 2, 4, 8, 12, 16])
@pytest.mark.parametrize("flags", [0, 1, 2, 3])
def test_search_vs_oracle(cuda, oracle, nw, flags):
    rng = np.random.default_rng(nw * 10 + flags)
    for bits, cols in ((4, 257), (8, 300), (32, 129)):
        d0, d1 = _desc(rng, 7, cols, nw, bits), _desc(rng, 7, cols, nw, bits)
        for lr in (0, 1, 3):
            got = host(lbg.search(dev(d0.view(np.int32), cuda), dev(d1.view(np.int32), cuda), flags, lr))
            assert_same(got, oracle.search(d0, d1, flags, lr), f"nw={nw} flags={flags} bits={bits} lr={lr}")


@pytest.mark.parametrize("nw", [1, 2, 4, 8, 12, 16])
@pytest.mark.parametrize("flags", [0, 1, 2, 3])
def test_search_declared_bits_vs_oracle(cuda, oracle, nw, flags):
    """bicos_search_bits_v1: with at most 32*nw-2 bit positions the
    tensor-core search takes its column-coded form (the candidate's column
    in the top two slots of the FP8 operands); tie-heavy value ranges and
    rows of up to 4096 columns (every tile pair), the declared count at the
    bound and below it"""
    rng = np.random.default_rng(nw * 100 + flags)
    for bits, cols, rows in ((1, 4096, 2), (2, 1000, 3), (4, 257, 7), (8, 300, 7), (29, 129, 5)):
        d0, d1 = _desc(rng, rows, cols, nw, bits), _desc(rng, rows, cols, nw, bits)
        for declared in (32 * nw - 2, 32 * (nw - 1) + bits):
            for lr in (0, 2):
                got = host(lbg.search(dev(d0.view(np.int32), cuda), dev(d1.view(np.int32), cuda), flags, lr,
                                      bits=declared))
                assert_same(got, oracle.search(d0, d1, flags, lr),
                            f"nw={nw} flags={flags} bits={bits} declared={declared} lr={lr}")


def test_search_declared_bits_all_ties(cuda, oracle):
    """every candidate ties (identical descriptors): first column without
    no-duplicates, invalid with it; and one unique best per row at the
    far end of a 4096-column row"""
    for nw in (1, 4, 16):
        d = np.zeros((2, 4096, nw), np.uint32)
        d[:, :, 0] = 0x5A5A5A5
        for flags in (0, 1, 2, 3):
            got = host(lbg.search(dev(d.view(np.int32), cuda), dev(d.view(np.int32), cuda), flags, 1,
                                  bits=32 * nw - 2))
            assert_same(got, oracle.search(d, d, flags, 1), f"nw={nw} flags={flags}")
        d1 = d.copy()
        d1[:, 4095, 0] ^= 1
        q = d.copy()
        q[:, :, 0] ^= 1
        for flags in (0, 1):
            got = host(lbg.search(dev(q.view(np.int32), cuda), dev(d1.view(np.int32), cuda), flags, 1,
                                  bits=32 * nw - 2))
            assert_same(got, oracle.search(q, d1, flags, 1), f"nw={nw} flags={flags} far best")


def test_search_bits_rejected(cuda):
    d = dev(np.zeros((1, 8, 1), np.int32), cuda)
    for bits in (0, 33, -1):
        with pytest.raises(ValueError, match="bit count"):
            lbg.search(d, d, 0, bits=bits)


def test_search_golden(cuda):
    z = golden("search.npz")
    for c in sorted({k.split("_")[0] for k in z.files}):
        d0, d1 = z[c + "_d0"], z[c + "_d1"]
        got = host(lbg.search(dev(d0.view(np.int32), cuda), dev(d1.view(np.int32), cuda), int(z[c + "_flags"]),
                              int(z[c + "_lr"])))
        assert_same(got, z[c + "_disp"], c)


@pytest.mark.parametrize("nw,cols", [(1, 12500), (4, 3500), (8, 1700)])
def test_search_wide_rows(cuda, oracle, nw, cols):
    """rows wider than one shared-memory chunk of candidates"""
    rng = np.random.default_rng(cols)
    d0, d1 = _desc(rng, 2, cols, nw, 16), _desc(rng, 2, cols, nw, 16)
    for flags in (1, 3):
        got = host(lbg.search(dev(d0.view(np.int32), cuda), dev(d1.view(np.int32), cuda), flags, 2))
        assert_same(got, oracle.search(d0, d1, flags, 2), f"cols={cols} flags={flags}")


def test_search_single_column(cuda, oracle):
    rng = np.random.default_rng(1)
    d0, d1 = _desc(rng, 3, 1, 2), _desc(rng, 3, 1, 2)
    for flags in (0, 1, 2, 3):
        got = host(lbg.search(dev(d0.view(np.int32), cuda), dev(d1.view(np.int32), cuda), flags, 0))
        assert_same(got, oracle.search(d0, d1, flags, 0))


def test_no_kernel_wait_ran_out(cuda, native):
    """the tensor-core search's bounded waits never expired in this process"""
    assert native.load().bicos_kernel_faults() == 0


def test_fp8_rate_probe(cuda, native):
    """bicos_tc_fp8_rate_v1: the search's MMA stream alone gives a finite
    positive rate, the N = 256 shape no less than 0.8 of it, and no
    completion wait runs out"""
    r128, r256 = lbg.tc_fp8_rate(128), lbg.tc_fp8_rate(256)
    assert 0.0 < r128 < 20000.0 and 0.0 < r256 < 20000.0
    assert r256 > 0.8 * r128
    assert native.load().bicos_kernel_faults() == 0


def test_search_known_answers(cuda):
    """the hand-worked cases of tests/test_oracle_kat.py on the GPU, in the
    plain and the column-coded form"""
    from test_oracle_kat import _rows, INV
    cases = [([3, 1, 1, 2, 4], 0, -1, [-1, 0, 1, 2, 3]), ([3, 1, 1, 2, 4], 1, -1, [INV] * 5),
             ([2, 1, 3, 1, 0], 1, -1, [-4, -3, -2, -1, 0]), ([2, 1, 3, 1, 0], 2, 1, [-4, -4, INV, INV, INV]),
             ([2, 1, 3, 1, 0], 2, 3, [-4, -4, -3, -3, INV]), ([2, 1, 3, 1, 0], 3, 3, [INV] * 5)]
    for costs, flags, lr, want in cases:
        d0, d1 = _rows(costs)
        for bits in (None, 30):
            got = host(lbg.search(dev(d0.view(np.int32), cuda), dev(d1.view(np.int32), cuda), flags, lr, bits=bits))
            assert got.tolist() == [want], (costs, flags, lr, bits)
