"""The C-ABI library builds, loads and exports every entry point that
include/bicos_c.h declares; host-side validation and error behaviour work
without a GPU (no compute is launched here)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "bicos_c.h")).read()
    decl = r"^(?:const\s+)?[A-Za-z_]\w*\s*\*?\s*(bicos_\w+)\s*\("
    return sorted(set(re.findall(decl, src, re.MULTILINE)))


def test_exports_every_declared_symbol(native):
    so = native.lib_path()
    out = subprocess.run(["nm", "-D", "--defined-only", so], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r" T (\w+)", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    lib = native.load()
    for s in declared_symbols():
        assert hasattr(lib, s)


def test_cpp_api_exported(native):
    out = subprocess.run(["nm", "-DC", "--defined-only", native.lib_path()], capture_output=True, text=True,
                         check=True).stdout
    assert "BICOS::match(" in out
    assert "BICOS::Image::create(" in out


def test_config_defaults(native):
    c = native.default_config()  # include/common.hpp:73-82
    assert c.has_threshold == 1 and abs(c.nxcorr_threshold - 0.5) < 1e-7
    assert c.has_subpixel_step == 0 and c.has_min_variance == 0
    assert c.mode == 0 and c.precision == 0 and c.variant == 0
    assert c.max_lr_diff == 1 and c.no_dupes == 0 and c.max_bits == 256


def test_output_types(native):
    lib = native.load()
    c = native.default_config()
    dt, ct = C.c_int32(), C.c_int32()
    lib.bicos_output_types(C.byref(c), C.byref(dt), C.byref(ct))
    assert (dt.value, ct.value) == (native.BICOS_16S, native.BICOS_32F)
    c.has_subpixel_step, c.subpixel_step, c.precision = 1, 0.1, 1
    lib.bicos_output_types(C.byref(c), C.byref(dt), C.byref(ct))
    assert (dt.value, ct.value) == (native.BICOS_32F, native.BICOS_64F)
    c.has_threshold = 0
    lib.bicos_output_types(C.byref(c), C.byref(dt), C.byref(ct))
    assert (dt.value, ct.value) == (native.BICOS_16S, -1)


def test_descriptor_words_table(native, oracle):
    lib = native.load()
    for n in range(2, 66):
        for mode in (0, 1):
            for mb in (256, 512):
                want = oracle.descriptor_words(oracle.required_bits(n, mode == 1), mb)
                if mode == 0 and want > 8:
                    want = -1  # the 512-bit extension is for full mode only
                assert lib.bicos_descriptor_words(n, mode, mb) == want, (n, mode, mb)


def _stack(native, n, type_=0, rows=4, cols=8):
    arr = (native.Image * max(n, 1))()
    for i in range(n):
        arr[i] = native.image(0x1000 * (i + 1), rows, cols, type_, cols * 2)
    return arr


def test_errors_before_any_device_work(native):
    lib = native.load()
    c = native.default_config()
    d = native.image(0x10, 4, 8, native.BICOS_16S, 16)
    s = _stack(native, 1)
    assert lib.bicos_match_v1(s, s, 1, C.byref(d), None, C.byref(c), None) == native.ERR_EXCEPTION
    assert lib.bicos_last_error() == b"need at least two images"
    s = _stack(native, 3, type_=native.BICOS_32F)
    assert lib.bicos_match_v1(s, s, 3, C.byref(d), None, C.byref(c), None) == native.ERR_EXCEPTION
    assert lib.bicos_last_error() == b"bad input depths, only CV_8UC1 and CV_16UC1 are supported"
    s = _stack(native, 66)
    assert lib.bicos_match_v1(s, s, 66, C.byref(d), None, C.byref(c), None) == native.ERR_INVALID_ARGUMENT
    assert lib.bicos_last_error() == b"input stacks too large, would require 257 bits"
    c.mode = 1
    s = _stack(native, 17)
    assert lib.bicos_match_v1(s, s, 17, C.byref(d), None, C.byref(c), None) == native.ERR_INVALID_ARGUMENT
    assert lib.bicos_last_error() == b"input stacks too large, would require 258 bits"
    c.mode = 0
    c.has_subpixel_step, c.subpixel_step = 1, 0.0
    s = _stack(native, 4)
    assert lib.bicos_match_v1(s, s, 4, C.byref(d), None, C.byref(c), None) == native.ERR_EXCEPTION
    assert b"subpixel step" in lib.bicos_last_error()
    # wrong output type: subpixel needs float32
    c.subpixel_step = 0.1
    assert lib.bicos_match_v1(s, s, 4, C.byref(d), None, C.byref(c), None) == native.ERR_EXCEPTION
    assert b"float32" in lib.bicos_last_error()
    # mismatched frame sizes
    s2 = _stack(native, 4, rows=5)
    c.has_subpixel_step = 0
    assert lib.bicos_match_v1(s, s2, 4, C.byref(d), None, C.byref(c), None) == native.ERR_EXCEPTION


def test_points_entry_checks_before_any_device_work(native):
    """bicos_match_points_v1 validates Q and the points image on the host"""
    lib = native.load()
    c = native.default_config()
    d = native.image(0x10, 4, 8, native.BICOS_16S, 16)
    s = _stack(native, 4)
    q = (C.c_double * 16)(*([1.0] * 16))
    pts = native.image(0x10, 4, 8, native.TYPE_32FC3, 8 * 12)
    assert lib.bicos_match_points_v1(s, s, 4, C.byref(d), None, C.byref(c), None, C.byref(pts), None) == \
        native.ERR_INVALID_ARGUMENT
    small = native.image(0x10, 4, 7, native.TYPE_32FC3, 7 * 12)
    assert lib.bicos_match_points_v1(s, s, 4, C.byref(d), None, C.byref(c), q, C.byref(small), None) == \
        native.ERR_EXCEPTION
    assert b"three-channel float32" in lib.bicos_last_error()
    q[5] = float("inf")
    assert lib.bicos_match_points_v1(s, s, 4, C.byref(d), None, C.byref(c), q, C.byref(pts), None) == \
        native.ERR_INVALID_ARGUMENT
    assert lib.bicos_last_error() == b"Q must be finite"


def test_tc_rate_argument_checks(native):
    """the FP8 rate probe refuses shapes other than N = 128 / 256 before any
    device work"""
    lib = native.load()
    v = C.c_double()
    for n in (0, 64, 192, 512):
        assert lib.bicos_tc_fp8_rate_v1(n, C.byref(v)) == native.ERR_INVALID_ARGUMENT
    assert lib.bicos_tc_fp8_rate_v1(128, None) == native.ERR_INVALID_ARGUMENT
    assert b"n must be 128 or 256" in lib.bicos_last_error()


def test_version(native):
    assert b"sm_103a" in native.load().bicos_version()


def test_batch_handle_host_side(native):
    """handle life cycle and tuning validation need no GPU"""
    import ctypes as C
    lib = native.load()
    h = C.c_void_p()
    assert lib.bicos_batch_create(C.byref(h)) == native.OK
    t = native.BatchTuning()
    assert lib.bicos_batch_get_tuning_v1(h, C.byref(t)) == native.OK
    assert (t.transform_block, t.ctas_per_sm, t.claim, t.branches, t.persistent) == (256, 8, 2, 4, 3)
    bad = native.BatchTuning(100, 1, 1, 1, 3)
    assert lib.bicos_batch_set_tuning_v1(h, C.byref(bad)) == native.ERR_INVALID_ARGUMENT
    assert b"out of range" in lib.bicos_last_error()
    good = native.BatchTuning(128, 4, 1, 2, 1)
    assert lib.bicos_batch_set_tuning_v1(h, C.byref(good)) == native.OK
    assert lib.bicos_match_batch_v1(h, None, 0, None) == native.OK  # empty batch: nothing to do
    assert lib.bicos_batch_captures(h) == 0
    assert lib.bicos_batch_destroy(h) == native.OK


def test_ingest_handle_validation(native):
    """bicos_ingest_create rejects bad stack shapes before any device work
    (the reference's exception texts); null handles are rejected too."""
    lib = native.load()
    h = C.c_void_p()
    cases = [((8, 8, 1, native.BICOS_8U), "need at least two images"),
             ((8, 8, 66, native.BICOS_8U), "Bad number of images"),
             ((8, 8, 4, native.BICOS_16S), "bad input depths"),
             ((0, 8, 4, native.BICOS_8U), "empty images"),
             ((8, 40000, 4, native.BICOS_8U), "int16 disparity range")]
    for args, msg in cases:
        assert lib.bicos_ingest_create(C.byref(h), *args) == native.ERR_EXCEPTION
        assert msg in lib.bicos_last_error().decode()
        assert not h.value
    assert lib.bicos_ingest_create(None, 8, 8, 4, native.BICOS_8U) == native.ERR_INVALID_ARGUMENT
    assert lib.bicos_ingest_destroy(None) == 0
    assert lib.bicos_ingest_push_v1(None, 0, None, None, 8, None) == native.ERR_INVALID_ARGUMENT
    assert lib.bicos_ingest_match_v1(None, None, None, None, None) == native.ERR_INVALID_ARGUMENT


C_PROGRAM = r"""
#include <bicos_c.h>
#include <stdio.h>
#include <string.h>

int main(void) {
    bicos_config c;
    bicos_image frames[66], disp;
    int i;
    if (bicos_config_default(&c) != BICOS_OK || !c.has_threshold || c.nxcorr_threshold != 0.5f ||
        c.has_subpixel_step || c.mode != BICOS_MODE_LIMITED || c.max_lr_diff != 1)
        return 10;
    for (i = 0; i < 66; ++i) { /* never dereferenced: validation fails first */
        frames[i].data = (void*)0x10; frames[i].step = 16; frames[i].rows = 4; frames[i].cols = 8;
        frames[i].type = BICOS_8U; frames[i].reserved = 0;
    }
    disp = frames[0];
    disp.type = BICOS_16S;
    if (bicos_match_v1(frames, frames, 1, &disp, NULL, &c, NULL) != BICOS_ERR_EXCEPTION ||
        strcmp(bicos_last_error(), "need at least two images") != 0)
        return 11;
    if (bicos_match_v1(frames, frames, 66, &disp, NULL, &c, NULL) != BICOS_ERR_INVALID_ARGUMENT ||
        strcmp(bicos_last_error(), "input stacks too large, would require 257 bits") != 0)
        return 12;
    printf("%s\n", bicos_version());
    return 0;
}
"""


def test_c_header_is_plain_c(native, tmp_path):
    """include/bicos_c.h compiles as strict C99 and a C caller links, reads the
    defaults and gets the reference's error texts (no device work)."""
    src, exe = tmp_path / "caller.c", tmp_path / "caller"
    src.write_text(C_PROGRAM)
    libdir = os.path.dirname(native.lib_path())
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I",
                    os.path.join(ROOT, "include"), str(src), "-L", libdir, "-lbicos_gb300",
                    "-Wl,-rpath," + libdir, "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, (r.returncode, r.stderr)
    assert "sm_103a" in r.stdout


def test_cpp_api_compiles_and_links(native, tmp_path):
    """The C++ drop-in (include/BICOS/match.hpp) builds against the library
    the way a libBICOS user's program does; running it needs a GPU."""
    libdir = os.path.dirname(native.lib_path())
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "match_cpp.cpp"), "-L", libdir, "-lbicos_gb300",
                    "-Wl,-rpath," + libdir, "-o", str(tmp_path / "match_cpp")], check=True)


def test_ingest_frame_checks_on_host():
    """Ingest.push checks each frame against the handle before the C call,
    which copies rows x cols samples from a bare pointer."""
    import torch
    import libbicos_gb300 as lbg
    from libbicos_gb300 import _native as N
    ing = lbg.Ingest.__new__(lbg.Ingest)  # no device handle: only the host checks run
    ing.rows, ing.cols, ing.n, ing._type, ing._h, ing._keep = 4, 8, 3, N.BICOS_8U, None, {}
    ok = np.zeros((4, 8), np.uint8)
    assert ing._host(ok)[2] == 8
    assert ing._host(torch.zeros((4, 8), dtype=torch.uint8))[2] == 8
    assert ing._host(np.zeros((4, 16), np.uint8)[:, ::2])[2] == 8  # made contiguous
    bad = [np.zeros((4, 7), np.uint8), np.zeros((3, 8), np.uint8), np.zeros((4, 8), np.uint16),
           np.zeros((4, 8), np.float32), np.zeros((2, 4, 8), np.uint8),
           torch.zeros((4, 8), dtype=torch.float32), torch.zeros((4, 8), dtype=torch.bool),
           torch.zeros((4, 8), dtype=torch.uint8, device="meta"), torch.zeros((8, 4), dtype=torch.uint8).t()]
    for b in bad:
        with pytest.raises(ValueError):
            ing.push(0, b, ok)
        with pytest.raises(ValueError):
            ing.push(0, ok, b)
    ing._type = N.BICOS_16U
    assert ing._host(np.zeros((4, 8), np.uint16))[2] == 16
    with pytest.raises(ValueError):
        ing._host(ok)


class _FakeDevice:
    """Stands in for a CUDA tensor in host-side argument checks (no GPU
    here): shape and dtype of a CPU tensor, reported as on the device."""
    is_cuda = True

    def __init__(self, *shape, dtype=None):
        import torch
        self._t = torch.zeros(*shape, dtype=dtype or torch.float32)
        self.shape, self.dtype = self._t.shape, self._t.dtype

    def is_contiguous(self):
        return True

    def dim(self):
        return self._t.dim()

    def numel(self):
        return self._t.numel()

    def element_size(self):
        return self._t.element_size()


def test_mlp_buffer_checks_on_host():
    """The MLP entry points take bare pointers: the wrappers check every
    buffer's residency, type and size before the call."""
    import torch
    from libbicos_gb300 import learned as L
    F = _FakeDevice
    model, params = F(L.MODEL_FLOATS), F(L.N_PARAMS)
    rows = F(10, L.N_IN + 1)
    L._check(model, "model", L.MODEL_FLOATS)
    L._check(rows, "rows", row=8)
    bad_calls = [
        lambda: L.grad(F(L.N_PARAMS), rows, params, F(1)),          # model without input statistics
        lambda: L.grad(model, F(10, 7), params, F(1)),               # rows of 7
        lambda: L.grad(model, rows, F(L.N_PARAMS - 1), F(1)),
        lambda: L.grad(model, rows, params, F(0)),
        lambda: L.grad(model, F(10, 8, dtype=torch.float64), params, F(1)),
        lambda: L.grad(torch.zeros(L.MODEL_FLOATS), rows, params, F(1)),  # host tensor
        lambda: L.adam(params, params, F(L.N_PARAMS - 1), params, 1, 1e-3, 1.0),
        lambda: L.propose(model, F(10, 9)),
        lambda: L.propose(F(L.N_PARAMS), rows),
    ]
    for call in bad_calls:
        with pytest.raises(ValueError):
            call()


def test_search_descriptor_checks_on_host():
    import torch
    import libbicos_gb300 as lbg
    F = _FakeDevice
    a = F(2, 16, 4, dtype=torch.int32)
    for d0, d1 in [(a, F(2, 15, 4, dtype=torch.int32)), (a, F(2, 16, 2, dtype=torch.int32)),
                   (a, F(2, 16, 4, dtype=torch.float32)), (a, F(2, 16, 4, dtype=torch.int64)),
                   (F(32, 4, dtype=torch.int32), F(32, 4, dtype=torch.int32)),
                   (a, torch.zeros((2, 16, 4), dtype=torch.int32))]:
        with pytest.raises(ValueError, match="descriptors"):
            lbg.search(d0, d1, 0)


def test_device_views_refuse_host_memory():
    """Kernels write through bicos_image views of tensors: a host tensor
    (an `out` buffer, a disparity to agree on) is refused before any call."""
    import torch
    import libbicos_gb300 as lbg
    from libbicos_gb300 import _native as N
    h16 = torch.zeros((4, 8), dtype=torch.int16)
    with pytest.raises(ValueError, match="CUDA"):
        N.tensor_image(h16)
    with pytest.raises(ValueError, match="CUDA"):
        N.points_image(torch.zeros((4, 8, 3), dtype=torch.float32))
    with pytest.raises(ValueError, match="CUDA"):
        lbg.reproject(h16, np.eye(4))


# The parts of OpenCV's CUDA core API the adapter uses (cv::cuda::GpuMat's
# header fields, channels/depth/create, CV_* type codes, Stream::Null and
# StreamAccessor::getStream), declared as OpenCV 4 declares them.  OpenCV is
# not installed here; the stand-in lets the adapter's OpenCV branch compile
# and link against the library in the CPU suite.
FAKE_CV_CUDA = r"""
#pragma once
#include <cstddef>
#include <cuda_runtime.h>
#define CV_8U 0
#define CV_16U 2
#define CV_16S 3
#define CV_32F 5
#define CV_64F 6
#define CV_16SC1 CV_16S
#define CV_32FC1 CV_32F
#define CV_64FC1 CV_64F
namespace cv { namespace cuda {
class GpuMat {
public:
    int flags = 0, rows = 0, cols = 0;
    size_t step = 0;
    unsigned char* data = nullptr;
    int depth() const { return flags & 7; }
    int channels() const { return 1; }
    void create(int r, int c, int type) { rows = r; cols = c; flags = type; }
};
class Stream {
public:
    static Stream& Null() { static Stream s; return s; }
    cudaStream_t s_ = nullptr;
};
struct StreamAccessor {
    static cudaStream_t getStream(const Stream& s) { return s.s_; }
};
} }
"""

ADAPTER_CALLER = r"""
#include <BICOS/opencv.hpp>
#ifndef EXPECT_OPENCV
#ifdef BICOS_HAVE_OPENCV_CUDA
#error "adapter active without OpenCV headers"
#endif
int main() { return 0; }
#else
#ifndef BICOS_HAVE_OPENCV_CUDA
#error "adapter not active"
#endif
int main() {
    std::vector<cv::cuda::GpuMat> s0(2), s1(2);
    cv::cuda::GpuMat disp, corr;
    BICOS::Config cfg;
    cfg.subpixel_step = 0.1f;
    void (*fn)(const std::vector<cv::cuda::GpuMat>&, const std::vector<cv::cuda::GpuMat>&, cv::cuda::GpuMat&,
               BICOS::Config, cv::cuda::GpuMat*, cv::cuda::Stream&) = &BICOS::match;
    (void)fn;
    (void)cfg;
    return 0;
}
#endif
"""


@pytest.mark.parametrize("with_cv", [False, True])
def test_opencv_adapter_compiles(native, tmp_path, with_cv):
    """include/BICOS/opencv.hpp (the cv::cuda::GpuMat / cv::cuda::Stream&
    signature of libBICOS include/match.hpp:30-40) stays out of the way
    without OpenCV and, given OpenCV's CUDA core headers (a stand-in here),
    compiles and links against the library."""
    src = tmp_path / "adapter.cpp"
    src.write_text(ADAPTER_CALLER)
    flags = []
    if with_cv:
        cv = tmp_path / "cv" / "opencv2" / "core"
        cv.mkdir(parents=True)
        (cv / "cuda.hpp").write_text(FAKE_CV_CUDA)
        (cv / "cuda_stream_accessor.hpp").write_text("#pragma once\n#include <opencv2/core/cuda.hpp>\n")
        cuda_inc = "/usr/local/cuda/include"
        if not os.path.isdir(cuda_inc):
            pytest.skip("CUDA headers not found")
        flags = ["-DEXPECT_OPENCV", "-I", str(tmp_path / "cv"), "-I", cuda_inc]
    libdir = os.path.dirname(native.lib_path())
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), *flags, str(src),
                    "-L", libdir, "-lbicos_gb300", "-Wl,-rpath," + libdir, "-o", str(tmp_path / "adapter")],
                   check=True)
