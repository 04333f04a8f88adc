"""The subpixel sweep's conversion-free rounding, checked on the CPU
(csrc/ncc.cuh, csrc/agree.cu).

The reference converts each interpolant with (TInput)roundevenf(v)
(include/impl/cpu/agree.hpp:164; the CUDA backend's (TInput)__float2int_rn,
include/impl/cuda/agree.cuh:235): round half to even, then wrap modulo 2^8 or
2^16.  The kernels get the same value without a conversion instruction:
q + 1.5 * 2^23 rounds q to an integer (ulp 1 in [2^23, 2^24)), the low
mantissa bits are that integer in two's complement, masked to the input
width and put back into a float with the 2^23 exponent.  This restates those
bit operations in numpy FP32 (IEEE round to nearest even, as __fadd_rn) and
compares them with the oracle's definition over every value the interpolant
can take: |a x^2 + b x + c| < 2^18 for 16-bit samples and |x| <= 1, well
inside the trick's |q| < 2^22.
"""
import os
import re

import numpy as np
import pytest

from conftest import ROOT

NCC = open(os.path.join(ROOT, "libbicos_gb300", "csrc", "ncc.cuh")).read()
F32 = np.float32
MAGIC = F32(12582912.0)  # 1.5 * 2^23


def body(name):
    m = re.search(name + r"\(float q\) \{(.*?)\n\}", NCC, re.S)
    assert m, name
    return m.group(1)


def test_constants_in_source():
    rw = body("round_wrap_f")
    assert "12582912.0f" in rw and "0x4B000000u" in rw and "8388608.0f" in rw
    assert "0xFFu" in rw and "0xFFFFu" in rw
    assert "12582912.0f" in body("round_wrap_bits")
    assert "0x4B400000 + v" in NCC and "12582912.0f" in NCC  # small_int_to_float


def round_wrap_f(q, bits):
    f = (q.astype(F32) + MAGIC).astype(F32)
    u = (f.view(np.uint32) & np.uint32((1 << bits) - 1)) | np.uint32(0x4B000000)
    return (u.view(F32) - F32(8388608.0)).astype(F32)


def round_wrap_bits(q, bits):
    f = (q.astype(F32) + MAGIC).astype(F32)
    return (f.view(np.uint32) & np.uint32((1 << bits) - 1)).astype(np.int64)


def reference(q, bits):
    """The oracle's round_wrap: rintf (half to even), then the wrap."""
    return np.rint(q.astype(F32)).astype(np.int64) % (1 << bits)


def _values(rng, span):
    grid = np.arange(-span * 64, span * 64 + 1, dtype=np.int64).astype(np.float64) / 64  # every 1/64
    ties = np.arange(-span, span, dtype=np.float64) + 0.5
    near = np.concatenate([np.nextafter(ties.astype(F32), F32(np.inf)), np.nextafter(ties.astype(F32), F32(-np.inf))])
    rand = rng.uniform(-span, span, size=1_000_000)
    return np.concatenate([grid, ties, near.astype(np.float64), rand]).astype(F32)


@pytest.mark.parametrize("bits,span", [(8, 1024), (16, 1 << 18)])
def test_round_wrap_matches_reference(bits, span):
    q = _values(np.random.default_rng(bits), span)
    want = reference(q, bits)
    assert np.array_equal(round_wrap_bits(q, bits), want)
    got = round_wrap_f(q, bits)
    assert np.array_equal(got.astype(np.int64), want) and np.all(got == np.floor(got))
    # ties go to even, as roundevenf
    assert reference(np.array([0.5, 1.5, 2.5, -0.5, -1.5], F32), bits).tolist() == \
        [0, 2, 2, 0, (1 << bits) - 2]


def test_interpolant_range():
    """The largest interpolant: 16-bit samples, |x| <= 1."""
    y = np.array([0, 65535], np.float64)
    worst = 0.0
    for y0 in y:
        for y1 in y:
            for y2 in y:
                a, b, c = 0.5 * (y0 - 2 * y1 + y2), 0.5 * (y2 - y0), y1
                x = np.linspace(-1, 1, 2001)
                worst = max(worst, float(np.abs(a * x * x + b * x + c).max()))
    assert worst < 2 ** 18 < 2 ** 22


def test_small_int_to_float_exhaustive():
    v = np.arange(-(1 << 22) + 1, 1 << 22, dtype=np.int64)
    u = (np.int64(0x4B400000) + v).astype(np.uint32)
    got = (u.view(F32) - MAGIC).astype(F32)
    assert np.array_equal(got, v.astype(F32))


def test_moment_band_exactness_bounds():
    """The moment form's tensor-core band (csrc/moments.cu): FP16 operands,
    FP32 sums.  Every operand must be an FP16 integer (below 2048) and every
    partial sum below 2^24 for the band to be exact -- which holds for 8-bit
    samples and for 16-bit samples below 4096, the range the kernel sends
    to the tensor cores."""
    n_max = 65
    assert 255 * 255 * n_max < 2 ** 24                      # 8-bit samples
    hi, lo = 4095 >> 6, 4095 & 63                           # 12-bit: 6 + 6 bits
    assert max(hi, lo) < 2048
    assert hi * hi * n_max < 2 ** 24                        # xh . yh
    assert (hi * lo + lo * hi) * n_max < 2 ** 24            # xh . yl + xl . yh (one accumulator)
    assert lo * lo * n_max < 2 ** 24
    x = np.arange(4096, dtype=np.int64)
    assert np.array_equal(4096 * ((x >> 6) * (x >> 6)) + 64 * (2 * (x >> 6) * (x & 63)) + (x & 63) ** 2, x * x)
    # past 12 bits the high part reaches 1023 and its sums pass 2^24 from
    # n = 17 on: a tile that stages a sample of 4096 or more takes the exact
    # SIMT sums instead (moments.cu; checked on the GPU in
    # tests/test_gpu_moments.py::test_moment_form_full_16bit)
    hi16 = 65535 >> 6
    assert hi16 < 2048 and hi16 * hi16 * 16 < 2 ** 24 <= hi16 * hi16 * 17
    s = np.float32(0)
    for _ in range(17):
        s = np.float32(s + np.float32(hi16 * hi16))
    assert int(s) != 17 * hi16 * hi16                       # FP32 accumulation rounds there


AGREE = open(os.path.join(ROOT, "libbicos_gb300", "csrc", "agree.cu")).read()


def test_integer_built_doubles():
    """exact_double (agree.cu): the FP64 sweep turns samples and rounded
    interpolants (non-negative, below 2^16) into doubles with integer
    instructions -- exponent 1023 + e from the leading one at bit e, the
    value shifted up to the 52-bit mantissa -- instead of a conversion on
    the FP64 pipe.  Restated here bit for bit over every value below 2^20."""
    m = re.search(r"double exact_double\(int v\) \{(.*?)\n\}", AGREE, re.S)
    assert m and "1023 + e" in m.group(1) and "52 - e" in m.group(1) and "0xFFFFFFFFFFFFFull" in m.group(1)
    v = np.arange(1 << 20, dtype=np.uint64)
    u = v | np.uint64(1)
    e = np.floor(np.log2(u.astype(np.float64))).astype(np.uint64)  # exact: u < 2^20
    mant = (v << (np.uint64(52) - e)) & np.uint64(0xFFFFFFFFFFFFF)
    bits = ((np.uint64(1023) + e) << np.uint64(52)) | mant
    bits[v == 0] = 0
    assert np.array_equal(bits.view(np.float64), v.astype(np.float64))
