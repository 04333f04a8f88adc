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
