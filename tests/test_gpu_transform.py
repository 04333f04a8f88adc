"""Descriptor transform on the GPU vs the oracle: bit-exact for every
descriptor width (32..256 bits, and the 384/512-bit full-mode extension),
both input depths, both modes, ragged widths."""
import numpy as np
import pytest

import libbicos_gb300 as lbg
from conftest import golden
from gpu_util import assert_same, dev, host

pytestmark = pytest.mark.gpu

LIMITED_NS = [2, 3, 4, 5, 8, 9, 10, 12, 17, 18, 24, 33, 34, 50, 65]
FULL_NS = [2, 3, 4, 5, 6, 7, 8, 9, 12, 13, 16, 17, 20, 21, 23]


@pytest.mark.parametrize("dt", [np.uint8, np.uint16])
@pytest.mark.parametrize("full,n", [(False, n) for n in LIMITED_NS] + [(True, n) for n in FULL_NS])
def test_transform_vs_oracle(cuda, oracle, dt, full, n):
    rng = np.random.default_rng(n * 7 + full)
    hi = np.iinfo(dt).max + 1 if n % 2 else 9  # small ranges make ties
    s = rng.integers(0, hi, size=(n, 19, 301), dtype=dt)
    got = host(lbg.descriptor_transform(dev(s, cuda), full))
    want = oracle.transform(s, full, got.shape[-1])
    assert_same(got, want, f"n={n} full={full}")


def test_transform_golden(cuda):
    z = golden("transform.npz")
    for c in sorted({k.split("_")[0] for k in z.files}):
        s, d, full = z[c + "_stack"], z[c + "_desc"], bool(z[c + "_full"])
        got = host(lbg.descriptor_transform(dev(s, cuda), full))
        assert_same(got, d, c)


def test_transform_pitched_frames(cuda, oracle):
    """frames with a row pitch wider than the row, passed as separate images"""
    import torch
    rng = np.random.default_rng(3)
    s = rng.integers(0, 256, size=(12, 33, 100), dtype=np.uint8)
    big = torch.zeros((12, 33, 160), dtype=torch.uint8, device=cuda)
    big[:, :, :100] = dev(s, cuda)
    frames = [big[i, :, :100] for i in range(12)]
    got = host(lbg.descriptor_transform(frames, False))
    assert_same(got, oracle.transform(s, False, got.shape[-1]))


def test_limited_known_answers(cuda):
    """the hand-worked descriptors of tests/test_oracle_kat.py on the GPU"""
    from test_oracle_kat import _transform_cases
    for pix, want in _transform_cases():
        n = len(pix)
        stack = dev(np.array(pix, dtype=np.uint8).reshape(n, 1, 1), cuda)
        d = host(lbg.descriptor_transform(stack, False))
        assert int(d.reshape(-1)[0]) == want, pix
