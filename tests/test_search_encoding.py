"""The tensor-core search's operand encoding and key arithmetic, checked on
the CPU (csrc/search_tc.cu, csrc/fp8_tiles.cuh).

The kernel turns each descriptor bit into an FP8 (e4m3) value whose sign is
the bit, multiplies query and candidate tiles on the tensor cores and reads
the arg-min out of the accumulator.  This file restates that integer
arithmetic (the multiply-and-mask nibble expansion, the e4m3 column code,
the column-coded keys and their decode, the plain form's FP32 keys
dot -/+ column/4096 up to the 4096-column bound) with the byte patterns taken from
the kernel source, decodes every byte with torch's own float8_e4m3fn, and
checks the decoded result against the oracle's search
(include/impl/cpu/bicos.hpp:50-113: first minimum, no-duplicates).  The GPU
tests check the kernel itself; this pins the design's arithmetic.
"""
import os
import re

import numpy as np
import pytest
import torch

from conftest import ROOT

# the byte patterns live in the tile header shared by the search and the
# transform, the rest in the search
SRC = "".join(open(os.path.join(ROOT, "libbicos_gb300", "csrc", f)).read()
              for f in ("fp8_tiles.cuh", "search_tc.cu"))
CONST = {k: int(v, 16) for k, v in re.findall(r"constexpr uint32_t (k\w+) = (0x[0-9A-Fa-f]+)u;", SRC)}
M32 = 0xFFFFFFFF
INV = -32768
E4M3 = torch.arange(256, dtype=torch.int32).to(torch.uint8).view(torch.float8_e4m3fn).float().numpy()


def fp8_lo(x, clear4):
    return ((((x & 0xF) * 0x10204080) & M32) & 0x80808080) ^ clear4


def fp8_hi(x, clear4):
    return ((((x & 0xF0) * 0x01020408) & M32) & 0x80808080) ^ clear4


def e4m3_small(v):
    e = (v | 1).bit_length() - 1
    return (((e + 7) << 3) | ((v << (3 - e)) & 7)) if v else 0


def column_code(c):
    return (e4m3_small(c & 15) << 16) | (e4m3_small(c >> 4) << 24)


def expand(words, clear4, code=None):
    """One descriptor (NW uint32 words) -> its 32*NW FP8 bytes in K order."""
    out = []
    nw = len(words)
    for w, x in enumerate(words):
        for h in range(2):
            y = (x >> (16 * h)) & 0xFFFF
            z = y >> 8
            top = fp8_hi(z, clear4)
            if code is not None and w == nw - 1 and h == 1:
                top = (top & 0xFFFF) | code
            for u in (fp8_lo(y, clear4), fp8_hi(y, clear4), fp8_lo(z, clear4), top):
                out += [(u >> (8 * i)) & 0xFF for i in range(4)]
    return out


def test_constants_decode():
    assert E4M3[CONST["kClearPlain"] & 0xFF] == -1.0
    assert E4M3[CONST["kClearQuery"] & 0xFF] == -16.0
    assert E4M3[CONST["kClearCand"] & 0xFF] == -8.0
    for k in ("kClearPlain", "kClearQuery", "kClearCand"):
        b = CONST[k] & 0xFF
        assert CONST[k] == b * 0x01010101
        assert E4M3[b ^ 0x80] == -E4M3[b]  # a set bit flips the sign
    q = CONST["kQueryCode"]
    assert q & 0xFFFF == 0
    assert (E4M3[(q >> 16) & 0xFF], E4M3[q >> 24]) == (-1.0, -16.0)


def test_nibble_expansion_exhaustive():
    """Byte i of fp8_lo / fp8_hi carries bit i (resp. 4 + i) of the byte in
    its sign, for all 256 byte values and each clear pattern."""
    for clear in (CONST["kClearPlain"], CONST["kClearQuery"], CONST["kClearCand"]):
        for x in range(256):
            lo, hi = fp8_lo(x, clear), fp8_hi(x, clear)
            for i in range(4):
                assert (lo >> (8 * i)) & 0xFF == (clear & 0xFF) ^ (0x80 * ((x >> i) & 1))
                assert (hi >> (8 * i)) & 0xFF == (clear & 0xFF) ^ (0x80 * ((x >> (4 + i)) & 1))


def test_column_code_is_e4m3():
    for v in range(16):
        want = torch.tensor([float(v)]).to(torch.float8_e4m3fn).view(torch.uint8).item()
        assert e4m3_small(v) == want, v
    q = CONST["kQueryCode"]
    qv = E4M3[(q >> 16) & 0xFF], E4M3[q >> 24]
    for c in range(256):
        code = column_code(c)
        assert code & 0xFFFF == 0
        cv = E4M3[(code >> 16) & 0xFF], E4M3[code >> 24]
        assert qv[0] * cv[0] + qv[1] * cv[1] == -c


def _keys(d0, d1, nodup):
    """The column-coded search of one row: accumulators from the FP8 bytes,
    per tile pair max D and max(D + 2c), merged into global keys, decoded."""
    cols, nw = d0.shape
    rows_q = np.array([[E4M3[b] for b in expand([int(w) for w in d], CONST["kClearQuery"], CONST["kQueryCode"])]
                       for d in d0])
    rows_c = np.array([[E4M3[b] for b in expand([int(w) for w in d], CONST["kClearCand"], column_code(j % 256))]
                       for j, d in enumerate(d1)])
    acc = rows_q @ rows_c.T  # exact: integers below 2^17
    assert np.all(np.abs(acc) < 2 ** 17) and np.all(acc == np.round(acc))
    out = np.empty(cols, np.int64)
    for i in range(cols):
        ga = gb = -(2 ** 31)
        for pair in range((cols + 255) // 256):
            lo, hi = 256 * pair, min(cols, 256 * pair + 256)
            dv = acc[i, lo:hi]
            c = np.arange(hi - lo)
            a, b = int(dv.max()), int((dv + 2 * c).max())
            ca = (-a) & 255
            ga = max(ga, ((a + ca) >> 8) * 8192 - (pair * 256 + ca))
            cb = b & 255
            gb = max(gb, ((b - cb) >> 8) * 8192 + (pair * 256 + cb))
        best = (-ga) & 8191
        valid = not nodup or (gb & 8191) == best
        out[i] = i - best if valid else INV
    return out


@pytest.mark.parametrize("nw", [1, 2, 4, 8])
@pytest.mark.parametrize("cols", [1, 7, 130, 300])
def test_coded_keys_match_oracle(oracle, nw, cols):
    rng = np.random.default_rng(nw * 1000 + cols)
    bits = 32 * nw - 2  # the widest descriptors the coded form takes
    top = np.uint32((1 << (bits - 32 * (nw - 1))) - 1)

    def rand(k):
        d = rng.integers(0, 2 ** 32, size=(k, nw), dtype=np.uint64).astype(np.uint32)
        d[:, -1] &= top
        return d
    # distinct candidates, then a third of the columns copied from others:
    # unique and duplicated minima, first and last columns apart
    d1 = rand(cols)
    dup = rng.random(cols) < 1 / 3
    d1[dup] = d1[rng.integers(0, cols, size=int(dup.sum()))]
    # queries near a candidate: a few flipped bits, every third exact
    d0 = d1[rng.integers(0, cols, size=cols)].copy()
    flips = rand(cols) & rand(cols) & rand(cols) & rand(cols)
    flips[::3] = 0
    d0 ^= flips
    results = []
    for nodup in (False, True):
        want = oracle.search(d0.reshape(1, cols, nw), d1.reshape(1, cols, nw), int(nodup))[0]
        got = _keys(d0, d1, nodup)
        assert np.array_equal(got, want.astype(np.int64)), (nw, cols, nodup)
        results.append(want)
    if cols >= 100:  # both outcomes of the no-duplicates rule occur
        assert 0 < int((results[1] == INV).sum()) < cols


def _plain_keys(d0, d1, nodup):
    """The plain form (descriptor width unknown, every K slot a bit): FP32
    keys dot - j/4096 and dot + j/4096 in the kernel's operation order
    (per 32-column chunk: dot -/+ k*s, then -/+ j0*s), decoded by the
    fractional part."""
    cols, nw = d0.shape
    clear = CONST["kClearPlain"]
    q = np.array([[E4M3[b] for b in expand([int(w) for w in d], clear)] for d in d0])
    c = np.array([[E4M3[b] for b in expand([int(w) for w in d], clear)] for d in d1])
    dot = (q @ c.T).astype(np.float32)  # K - 2 * Hamming, exact
    s = np.float32(1.0 / 4096.0)
    j = np.arange(cols)
    k = (j % 32).astype(np.float32)
    j0 = (j - j % 32).astype(np.float32)
    ka = (dot - k * s) - j0 * s
    kb = (dot + k * s) + j0 * s
    assert ka.dtype == np.float32
    ma, mb = ka.max(axis=1), kb.max(axis=1)
    best = ((np.ceil(ma) - ma) * np.float32(4096.0)).astype(np.int64)
    last = ((mb - np.floor(mb)) * np.float32(4096.0)).astype(np.int64)
    valid = (last == best) if nodup else np.ones(cols, bool)
    return np.where(valid, j - best, INV)


@pytest.mark.parametrize("nw", [1, 2, 4, 8])
@pytest.mark.parametrize("cols", [1, 33, 300])
def test_plain_keys_match_oracle(oracle, nw, cols):
    rng = np.random.default_rng(nw * 77 + cols)
    d1 = rng.integers(0, 2 ** 32, size=(cols, nw), dtype=np.uint64).astype(np.uint32)
    dup = rng.random(cols) < 1 / 3
    d1[dup] = d1[rng.integers(0, cols, size=int(dup.sum()))]
    d0 = d1[rng.integers(0, cols, size=cols)].copy()
    flips = np.bitwise_and.reduce(rng.integers(0, 2 ** 32, size=(4, cols, nw), dtype=np.uint64).astype(np.uint32))
    d0 ^= flips
    for nodup in (False, True):
        want = oracle.search(d0.reshape(1, cols, nw), d1.reshape(1, cols, nw), int(nodup))[0]
        assert np.array_equal(_plain_keys(d0, d1, nodup), want.astype(np.int64)), (nw, cols, nodup)


def test_widest_row_both_forms(oracle):
    """4096 columns, the width bound of the tensor-core search: the last
    column's keys stay exact in both forms."""
    cols, nw = 4096, 1
    rng = np.random.default_rng(5)
    d1 = (rng.integers(0, 2 ** 30, size=(cols, nw), dtype=np.uint64)).astype(np.uint32)
    d1[-1] = d1[0]          # the minimum of query 0 at the first and the last column
    d1[-2] = d1[-3]
    d0 = d1[[0, cols - 1, cols - 2, cols - 3] + list(rng.integers(0, cols, size=cols - 4))].copy()
    for nodup in (False, True):
        want = oracle.search(d0.reshape(1, cols, nw), d1.reshape(1, cols, nw), int(nodup))[0].astype(np.int64)
        assert np.array_equal(_plain_keys(d0, d1, nodup), want), nodup
        sub = slice(0, 64)  # the coded model is slower: a prefix of the queries, all candidates
        assert np.array_equal(_keys(d0, d1, nodup)[sub], want[sub]), nodup
    assert want[0] == INV and want[1] == INV  # duplicated minima under no-duplicates
