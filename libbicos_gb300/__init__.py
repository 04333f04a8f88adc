"""bicos_gb300: GB300-native (sm_103a) BICOS stereo matching.

The matching path of libBICOS -- binary temporal descriptor transform,
row-wise Hamming arg-min with the no-duplicates / consistency postfilter,
NCC agreement with optional subpixel sweep -- as hand-written CUDA kernels
behind a C ABI (include/bicos_c.h), a C++ ``BICOS::match`` API
(include/BICOS/) and the ``pybicos`` Python surface (``.pybicos``).

Device-side helpers here take CUDA tensors (torch is only the container for
device memory and streams); they call the C ABI directly with zero copies.
"""
from __future__ import annotations

import ctypes as C

from . import _native as N
from . import pybicos
from .pybicos import Config, Precision, TransformMode, Variant

__all__ = ["pybicos", "Config", "Precision", "TransformMode", "Variant", "match_device",
           "descriptor_transform", "search", "agree", "agree_subpixel", "descriptor_words",
           "subpixel_features", "agree_learned", "Batch", "tc_fp8_rate",
           "load_library", "required_bits"]


def load_library():
    """Load the native library; raises ImportError when it is not built."""
    return N.load()


def required_bits(n: int, full: bool) -> int:
    return n * n - 2 * n + 3 if full else 4 * n - 7


def descriptor_words(n: int, full: bool, max_bits: int = 256) -> int:
    return N.load().bicos_descriptor_words(n, 1 if full else 0, max_bits)


def _stream_ptr(stream):
    import torch
    s = torch.cuda.current_stream() if stream is None else stream
    return C.c_void_p(s.cuda_stream)


def _frames(stack):
    """A (n, rows, cols) tensor or a sequence of 2-D tensors -> bicos_image[]."""
    frames = [stack[i] for i in range(stack.shape[0])] if hasattr(stack, "dim") and stack.dim() == 3 else list(stack)
    for f in frames:
        if not f.is_cuda:
            raise ValueError("device API expects CUDA tensors")
    return N.image_array([N.tensor_image(f) for f in frames]), len(frames), frames[0]


def _raise(st):
    try:
        N.check(st)
    except N.NativeError as e:
        pybicos.raise_native(e)


def match_device(stack0, stack1, cfg: Config | None = None, stream=None, out=None, corrmap=True,
                 max_bits: int = 256, q=None, points=None):
    """BICOS::match on CUDA tensors.  Returns (disparity, corrmap or None),
    or (disparity, corrmap, points) when a reprojection matrix ``q`` (4x4)
    is given.

    stack0/stack1: (n, rows, cols) uint8/uint16 CUDA tensors or lists of
    2-D ones.  ``out`` may supply (disparity, corrmap) tensors to reuse and
    ``points`` a (rows, cols, 3) float32 tensor.  With ``q`` the point cloud
    is written in the same pass (bicos_match_points_v1).  Enqueued on
    ``stream`` (torch's current stream by default); returns without
    synchronising.
    """
    import torch
    cfg = Config() if cfg is None else cfg
    nc = cfg.native()
    nc.max_bits = max_bits
    a0, n, f0 = _frames(stack0)
    a1, n1, _ = _frames(stack1)
    if n1 != n:
        raise pybicos.Exception("both stacks must hold the same number of images")
    dt, ct = C.c_int32(), C.c_int32()
    N.check(N.load().bicos_output_types(C.byref(nc), C.byref(dt), C.byref(ct)))
    rows, cols = f0.shape
    if out is not None:
        disp, corr = out
    else:
        disp = torch.empty((rows, cols), dtype=torch.int16 if dt.value == N.BICOS_16S else torch.float32,
                           device=f0.device)
        corr = None
        if corrmap and ct.value >= 0:
            corr = torch.empty((rows, cols), dtype=torch.float64 if ct.value == N.BICOS_64F else torch.float32,
                               device=f0.device)
    di = N.tensor_image(disp)
    ci = N.tensor_image(corr) if corr is not None else None
    if q is None:
        st = N.load().bicos_match_v1(a0, a1, n, C.byref(di), C.byref(ci) if ci is not None else None,
                                     C.byref(nc), _stream_ptr(stream))
        _raise(st)
        return disp, corr
    import numpy as np
    qa = np.ascontiguousarray(np.asarray(q, dtype=np.float64).reshape(4, 4))
    if points is None:
        points = torch.empty((rows, cols, 3), dtype=torch.float32, device=f0.device)
    pi = N.points_image(points)
    st = N.load().bicos_match_points_v1(a0, a1, n, C.byref(di), C.byref(ci) if ci is not None else None,
                                        C.byref(nc), qa.ctypes.data_as(C.POINTER(C.c_double)), C.byref(pi),
                                        _stream_ptr(stream))
    _raise(st)
    return disp, corr, points


def descriptor_transform(stack, full: bool, stream=None):
    """Descriptors of one stack: (rows, cols, nwords) uint32 as int32 tensor."""
    import torch
    arr, n, f0 = _frames(stack)
    nw = descriptor_words(n, full, 512)
    if nw < 0:
        raise ValueError(f"input stacks too large, would require {required_bits(n, full)} bits")
    rows, cols = f0.shape
    out = torch.empty((rows, cols, nw), dtype=torch.int32, device=f0.device)
    _raise(N.load().bicos_descriptor_transform_v1(arr, n, 1 if full else 0, nw, C.c_void_p(out.data_ptr()),
                                                  _stream_ptr(stream)))
    return out


def search(desc0, desc1, flags: int, max_lr_diff: int = -1, stream=None, bits=None):
    """Hamming arg-min of (rows, cols, nwords) descriptor tensors -> int16
    disparity.  bits: the descriptors' bit count when known (higher bits
    zero, as the transform writes them; bicos_search_bits_v1)."""
    import torch
    # the C call takes bare pointers and the sizes of desc0: both tensors
    # must hold exactly rows x cols x nwords 32-bit words on the device
    if desc0.dim() != 3 or tuple(desc1.shape) != tuple(desc0.shape):
        raise ValueError(f"descriptors must be (rows, cols, nwords) tensors of one shape, got "
                         f"{tuple(desc0.shape)} and {tuple(desc1.shape)}")
    for d in (desc0, desc1):
        if not d.is_cuda or not d.is_contiguous() or d.element_size() != 4 or d.dtype.is_floating_point:
            raise ValueError("descriptors must be contiguous 32-bit integer CUDA tensors")
    rows, cols, nw = desc0.shape
    out = torch.empty((rows, cols), dtype=torch.int16, device=desc0.device)
    oi = N.tensor_image(out)
    lib = N.load()
    d0, d1 = C.c_void_p(desc0.data_ptr()), C.c_void_p(desc1.data_ptr())
    if bits is None:
        _raise(lib.bicos_search_v1(d0, d1, rows, cols, nw, flags, max_lr_diff, C.byref(oi), _stream_ptr(stream)))
    else:
        _raise(lib.bicos_search_bits_v1(d0, d1, rows, cols, nw, int(bits), flags, max_lr_diff, C.byref(oi),
                                        _stream_ptr(stream)))
    return out


def reproject(disparity, q, out=None, stream=None):
    """Point cloud of a disparity map (bicos_reproject_v1; bicos-cli's
    cv::reprojectImageTo3D(disp, points, Q, false, CV_32F) step,
    src/cli.cpp:228-250): a (rows, cols, 3) float32 CUDA tensor of
    (X/W, Y/W, Z/W), [X Y Z W] = Q [x y d 1].  disparity: int16 or float32
    CUDA tensor; q: 4x4 array-like."""
    import numpy as np
    import torch
    qa = np.ascontiguousarray(np.asarray(q, dtype=np.float64).reshape(4, 4))
    if out is None:
        out = torch.empty((disparity.shape[0], disparity.shape[1], 3), dtype=torch.float32, device=disparity.device)
    di, pi = N.tensor_image(disparity), N.points_image(out)
    _raise(N.load().bicos_reproject_v1(C.byref(di), qa.ctypes.data_as(C.POINTER(C.c_double)), C.byref(pi),
                                       _stream_ptr(stream)))
    return out


def tc_fp8_rate(n: int = 128) -> float:
    """FP8 tensor-core rate of the current device in TFLOP/s for the
    search's MMA shape (bicos_tc_fp8_rate_v1): n = 128 the search's
    M = 128 x N = 128 x K = 32 instructions issued alone, n = 256 the
    largest single-CTA shape.  A measurement tool, the denominator of the
    search's roofline."""
    v = C.c_double()
    _raise(N.load().bicos_tc_fp8_rate_v1(int(n), C.byref(v)))
    return v.value


def agree(disp, stack0, stack1, threshold: float, min_var=None, double=False, stream=None):
    """In-place NCC agreement on an int16 disparity; returns (disp, corrmap).
    min_var is the per-stack value (min_variance * n)."""
    import torch
    a0, n, f0 = _frames(stack0)
    a1, _, _ = _frames(stack1)
    corr = torch.empty(disp.shape, dtype=torch.float64 if double else torch.float32, device=disp.device)
    di, ci = N.tensor_image(disp), N.tensor_image(corr)
    _raise(N.load().bicos_agree_v1(C.byref(di), a0, a1, n, threshold, int(min_var is not None),
                                   float(min_var or 0.0), int(double), C.byref(ci), _stream_ptr(stream)))
    return disp, corr


def agree_subpixel(raw, stack0, stack1, threshold: float, step: float, min_var=None, double=False, stream=None):
    """NCC agreement with subpixel sweep; returns (float32 disparity, corrmap)."""
    import torch
    a0, n, f0 = _frames(stack0)
    a1, _, _ = _frames(stack1)
    out = torch.empty(raw.shape, dtype=torch.float32, device=raw.device)
    corr = torch.empty(raw.shape, dtype=torch.float64 if double else torch.float32, device=raw.device)
    ri, oi, ci = N.tensor_image(raw), N.tensor_image(out), N.tensor_image(corr)
    _raise(N.load().bicos_agree_subpixel_v1(C.byref(ri), a0, a1, n, threshold, step, int(min_var is not None),
                                            float(min_var or 0.0), int(double), C.byref(oi), C.byref(ci),
                                            _stream_ptr(stream)))
    return out, corr


def subpixel_features(raw, stack0, stack1, stream=None):
    """Feature rows of the learned subpixel form for an int16 raw disparity:
    (rows, cols, 8) float32 -- rho at col1-2..col1+2, left and right
    per-frame variances, validity flag."""
    import torch
    a0, n, f0 = _frames(stack0)
    a1, _, _ = _frames(stack1)
    rows, cols = raw.shape
    feats = torch.empty((rows, cols, 8), dtype=torch.float32, device=raw.device)
    ri = N.tensor_image(raw)
    fi = N.image(feats.data_ptr(), rows, 8 * cols, N.BICOS_32F, 32 * cols)
    _raise(N.load().bicos_subpixel_features_v1(C.byref(ri), a0, a1, n, C.byref(fi), _stream_ptr(stream)))
    return feats


def agree_learned(raw, stack0, stack1, threshold: float, step: float, min_var=None, double=False, stream=None):
    """Learned-form agreement of an int16 raw disparity: returns (float32
    disparity, corrmap, proposals, number of pixels that took the sweep).
    min_var is the per-stack value (min_variance * n)."""
    import torch
    a0, n, f0 = _frames(stack0)
    a1, _, _ = _frames(stack1)
    out = torch.empty(raw.shape, dtype=torch.float32, device=raw.device)
    corr = torch.empty(raw.shape, dtype=torch.float64 if double else torch.float32, device=raw.device)
    prop = torch.empty(raw.shape, dtype=torch.float32, device=raw.device)
    ri, oi, ci, pi = N.tensor_image(raw), N.tensor_image(out), N.tensor_image(corr), N.tensor_image(prop)
    count = C.c_int32(-1)
    _raise(N.load().bicos_agree_learned_v1(C.byref(ri), a0, a1, n, threshold, step, int(min_var is not None),
                                           float(min_var or 0.0), int(double), C.byref(oi), C.byref(ci),
                                           C.byref(pi), C.byref(count), _stream_ptr(stream)))
    (torch.cuda.current_stream(raw.device) if stream is None else stream).synchronize()  # the count is host memory
    return out, corr, prop, int(count.value)


class Ingest:
    """Frame-by-frame ingest (bicos_ingest_*): device frames for one stack
    shape; push(t, left, right) uploads frame t of both sides as it arrives
    (host numpy arrays or pinned torch CPU tensors, 2-D uint8/uint16), and
    match(cfg) runs BICOS::match on the resident frames once all n were
    pushed.  Pushed host buffers are referenced until they are replaced or
    the handle is closed (pinned memory is copied asynchronously)."""

    def __init__(self, rows: int, cols: int, n: int, dtype="uint8"):
        self._lib = N.load()
        self.rows, self.cols, self.n = rows, cols, n
        self._type = N.BICOS_8U if str(dtype).endswith("uint8") else N.BICOS_16U
        h = C.c_void_p()
        _raise(self._lib.bicos_ingest_create(C.byref(h), rows, cols, n, self._type))
        self._h = h
        self._keep = {}

    def close(self):
        if self._h:
            self._lib.bicos_ingest_destroy(self._h)
            self._h = None
        self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _host(self, a):
        """(keep-alive object, host pointer, row step) of one frame, checked
        against the handle's shape and sample type: the C call copies
        rows x cols samples from the pointer and cannot check the buffer."""
        esize = 1 if self._type == N.BICOS_8U else 2
        if hasattr(a, "data_ptr"):  # torch tensor
            if a.device.type != "cpu":
                raise ValueError("frames are host buffers: numpy arrays or CPU torch tensors")
            if a.dtype.is_floating_point or a.dtype.is_complex or str(a.dtype) == "torch.bool" \
                    or a.element_size() != esize:
                raise ValueError(f"expected {8 * esize}-bit integer frames, got {a.dtype}")
            if tuple(a.shape) != (self.rows, self.cols) or a.stride(1) != 1:
                raise ValueError(f"expected {self.rows}x{self.cols} frames with unit column stride, "
                                 f"got shape {tuple(a.shape)}")
            return a, a.data_ptr(), a.stride(0) * a.element_size()
        import numpy as np
        a = np.ascontiguousarray(a)
        want = np.uint8 if esize == 1 else np.uint16
        if a.dtype != want:
            raise ValueError(f"expected {np.dtype(want).name} frames, got {a.dtype}")
        if a.shape != (self.rows, self.cols):
            raise ValueError(f"expected {self.rows}x{self.cols} frames, got shape {a.shape}")
        return a, a.ctypes.data, a.strides[0]

    def push(self, t: int, left, right, stream=None):
        l, lp, ls = self._host(left)
        r, rp, rs = self._host(right)
        if ls != rs:
            raise ValueError("both frames must share the row step")
        _raise(self._lib.bicos_ingest_push_v1(self._h, t, C.c_void_p(lp), C.c_void_p(rp), ls, _stream_ptr(stream)))
        self._keep[t] = (l, r)

    def match(self, cfg: Config | None = None, stream=None, out=None, corrmap=True):
        """(disparity, corrmap or None) CUDA tensors, as match_device."""
        import torch
        cfg = Config() if cfg is None else cfg
        nc = cfg.native()
        dt, ct = C.c_int32(), C.c_int32()
        N.check(self._lib.bicos_output_types(C.byref(nc), C.byref(dt), C.byref(ct)))
        if out is not None:
            disp, corr = out
        else:
            dev = torch.device("cuda")
            disp = torch.empty((self.rows, self.cols), dtype=torch.int16 if dt.value == N.BICOS_16S else torch.float32,
                               device=dev)
            corr = None
            if corrmap and ct.value >= 0:
                corr = torch.empty((self.rows, self.cols),
                                   dtype=torch.float64 if ct.value == N.BICOS_64F else torch.float32, device=dev)
        di = N.tensor_image(disp)
        ci = N.tensor_image(corr) if corr is not None else None
        _raise(self._lib.bicos_ingest_match_v1(self._h, C.byref(di), C.byref(ci) if ci is not None else None,
                                               C.byref(nc), _stream_ptr(stream)))
        return disp, corr


class Batch:
    """Many stacks per call (bicos_match_batch_v1): one CUDA graph per batch
    signature, persistent multi-stack launches, an autotuner over launch
    shapes.  Each job is (stack0, stack1, cfg) with CUDA tensors as for
    match_device; outputs are (disparity, corrmap or None) per job.  Reuse
    the outputs of one call (``outs``) to replay its graph."""

    def __init__(self):
        self._lib = N.load()
        h = C.c_void_p()
        N.check(self._lib.bicos_batch_create(C.byref(h)))
        self._h = h

    def close(self):
        if self._h:
            self._lib.bicos_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def outputs(jobs):
        import torch
        outs = []
        for stack0, _, cfg in jobs:
            nc = cfg.native()
            dt, ct = C.c_int32(), C.c_int32()
            N.check(N.load().bicos_output_types(C.byref(nc), C.byref(dt), C.byref(ct)))
            f0 = stack0[0]
            disp = torch.empty(tuple(f0.shape), dtype=torch.int16 if dt.value == N.BICOS_16S else torch.float32,
                               device=f0.device)
            corr = None
            if ct.value >= 0:
                corr = torch.empty(tuple(f0.shape), dtype=torch.float64 if ct.value == N.BICOS_64F else torch.float32,
                                   device=f0.device)
            outs.append((disp, corr))
        return outs

    def _items(self, jobs, outs, max_bits):
        keep, items = [], (N.BatchItem * len(jobs))()
        for k, ((stack0, stack1, cfg), (disp, corr)) in enumerate(zip(jobs, outs)):
            a0, n, _ = _frames(stack0)
            a1, n1, _ = _frames(stack1)
            if n1 != n:
                raise pybicos.Exception("both stacks must hold the same number of images")
            nc = cfg.native()
            nc.max_bits = max_bits
            di = N.tensor_image(disp)
            ci = N.tensor_image(corr) if corr is not None else None
            keep += [a0, a1, nc, di, ci]
            items[k] = N.BatchItem(a0, a1, n, C.pointer(di), C.pointer(ci) if ci is not None else None,
                                   C.pointer(nc))
        return items, keep

    def match(self, jobs, outs=None, stream=None, max_bits: int = 256):
        outs = self.outputs(jobs) if outs is None else outs
        items, keep = self._items(jobs, outs, max_bits)
        _raise(self._lib.bicos_match_batch_v1(self._h, items, len(jobs), _stream_ptr(stream)))
        return outs

    def autotune(self, jobs, outs, stream=None, max_bits: int = 256) -> dict:
        items, keep = self._items(jobs, outs, max_bits)
        t = N.BatchTuning()
        _raise(self._lib.bicos_batch_autotune_v1(self._h, items, len(jobs), _stream_ptr(stream), C.byref(t)))
        return {f: getattr(t, f) for f, _ in N.BatchTuning._fields_}

    def set_tuning(self, tuning: dict | None):
        t = None if tuning is None else N.BatchTuning(**tuning)
        _raise(self._lib.bicos_batch_set_tuning_v1(self._h, C.byref(t) if t is not None else None))

    @property
    def captures(self) -> int:
        return self._lib.bicos_batch_captures(self._h)
