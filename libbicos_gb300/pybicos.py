"""pybicos: the Python surface of libBICOS, on the GB300 library.

Same names, argument meaning and errors as the reference's pybind11 module
(src/pybicos.cpp:121-177): ``Config``, ``Precision``, ``TransformMode``,
``Variant.NoDuplicates``, ``Variant.Consistency``, ``Exception``,
``match(stack0, stack1, cfg) -> (disparity, corrmap)`` over numpy host
images, and ``invalid_disparity(dtype)``.  Enum values are also exported at
module level (``pybicos.Full``, ``pybicos.Double`` ...), as
``py::enum_::export_values`` does.

``match`` runs on the GPU.  Given host images (numpy) it goes through
``bicos_match_host_v1``: upload, the CUDA path, download, like the
reference's CUDA build of pybicos (src/pybicos.cpp:81-95), and returns
numpy arrays.  Given device images -- torch CUDA tensors or any object with
``__cuda_array_interface__`` (CuPy, Numba, ...) -- it matches them where
they lie, without copies, through ``bicos_match_v1`` and returns torch CUDA
tensors, enqueued on the producer's stream (torch's current stream, or the
interface's ``stream``) without a host synchronisation.

One deliberate difference: when ``nxcorr_threshold`` is None the reference
module fails while converting the never-created correlation map; here
``corrmap`` is returned as None.
"""
from __future__ import annotations

import builtins
import ctypes as C
import enum
import types

import numpy as np

from . import _native as N

__all__ = ["Config", "Precision", "TransformMode", "Variant", "Exception", "match",
           "invalid_disparity", "Single", "Double", "Full", "Limited"]


class Exception(builtins.Exception):  # noqa: A001
    """pybicos.Exception: BICOS::Exception raised by the library."""


class Precision(enum.Enum):
    Double = 1
    Single = 0

    def __repr__(self):
        return f"<Precision.{self.name}: {self.value}>"


class TransformMode(enum.Enum):
    Full = 1
    Limited = 0

    def __repr__(self):
        return f"<TransformMode.{self.name}: {self.value}>"


Single, Double = Precision.Single, Precision.Double
Full, Limited = TransformMode.Full, TransformMode.Limited


class _NoDuplicates:
    def __repr__(self):
        return "NoDuplicates"

    def __eq__(self, other):
        return isinstance(other, _NoDuplicates)


class _Consistency:
    def __init__(self, max_lr_diff: int = 1, no_dupes: bool = False):
        self.max_lr_diff = int(max_lr_diff)
        self.no_dupes = bool(no_dupes)

    def __repr__(self):
        return (f"Consistency( max_lr_diff = {self.max_lr_diff}, "
                f"no_dupes = {'true' if self.no_dupes else 'false'} )")

    def __eq__(self, other):
        return (isinstance(other, _Consistency) and other.max_lr_diff == self.max_lr_diff
                and other.no_dupes == self.no_dupes)


_NoDuplicates.__name__ = _NoDuplicates.__qualname__ = "NoDuplicates"
_Consistency.__name__ = _Consistency.__qualname__ = "Consistency"
Variant = types.SimpleNamespace(NoDuplicates=_NoDuplicates, Consistency=_Consistency)


def _f32(v):
    return None if v is None else float(np.float32(v))


def _fmt_opt(v):
    # fmt's std::optional formatting: optional(x) / none
    return "none" if v is None else "optional(" + str(np.float32(v)) + ")"


class Config:
    """BICOS::Config (include/common.hpp:73-82) with the CUDA build's precision."""

    def __init__(self):
        self._thr = 0.5
        self._step = None
        self._minvar = None
        self.mode = TransformMode.Limited
        self.precision = Precision.Single
        self.variant = Variant.NoDuplicates()
        # extension (not in the reference): 0 = the reference's two-pass NCC,
        # 1 = the moment form (tensor-core Sxy, unrounded subpixel interpolant),
        # 2 = the learned subpixel form (network proposal, one reference NCC
        # check, the reference sweep where the check fails)
        self.nxcorr_form = 0

    nxcorr_threshold = property(lambda s: s._thr, lambda s, v: setattr(s, "_thr", _f32(v)))
    subpixel_step = property(lambda s: s._step, lambda s, v: setattr(s, "_step", _f32(v)))
    min_variance = property(lambda s: s._minvar, lambda s, v: setattr(s, "_minvar", _f32(v)))

    def __repr__(self):
        return (f"Config( nxcorr_threshold = {_fmt_opt(self._thr)}, subpixel_step = {_fmt_opt(self._step)}, "
                f"min_variance = {_fmt_opt(self._minvar)}, mode = {self.mode.name}, "
                f"precision = {self.precision.name}, variant = {self.variant!r} )")

    def native(self) -> N.Config:
        c = N.default_config()
        c.has_threshold = self._thr is not None
        c.nxcorr_threshold = self._thr if self._thr is not None else 0.0
        c.has_subpixel_step = self._step is not None
        c.subpixel_step = self._step if self._step is not None else 0.0
        c.has_min_variance = self._minvar is not None
        c.min_variance = self._minvar if self._minvar is not None else 0.0
        if not isinstance(self.mode, TransformMode) or not isinstance(self.precision, Precision):
            raise TypeError("mode must be a TransformMode and precision a Precision")
        c.mode = self.mode.value
        c.precision = self.precision.value
        if self.nxcorr_form not in (0, 1, 2):
            raise ValueError("nxcorr_form must be 0 (reference), 1 (moments) or 2 (learned)")
        c.nxcorr_form = int(self.nxcorr_form)
        if isinstance(self.variant, _Consistency):
            c.variant = 1
            c.max_lr_diff = self.variant.max_lr_diff
            c.no_dupes = int(self.variant.no_dupes)
        elif isinstance(self.variant, _NoDuplicates):
            c.variant = 0
        else:
            raise TypeError("variant must be Variant.NoDuplicates() or Variant.Consistency(...)")
        return c


def raise_native(e: N.NativeError):
    if e.status == N.ERR_INVALID_ARGUMENT:
        raise ValueError(str(e)) from None
    raise Exception(str(e)) from None


def _as_image(a) -> np.ndarray:
    a = np.asarray(a)
    if a.ndim != 2:
        raise Exception(f"expected 2-D images, got shape {a.shape}")
    if a.dtype not in (np.uint8, np.uint16):
        raise Exception(f"unimplemented cvtype_of(dtype={a.dtype})")
    # unit column stride and a forward row step of at least one row (a
    # flipped view's negative step would reach the C call as a huge size_t)
    if a.strides[1] != a.itemsize or a.strides[0] < a.shape[1] * a.itemsize:
        a = np.ascontiguousarray(a)
    return a


def _is_device(a) -> bool:
    return hasattr(a, "__cuda_array_interface__") and not (hasattr(a, "is_cuda") and not a.is_cuda)


def _device_image(a):
    """(bicos_image, stream or None) of a 2-D device array given through
    __cuda_array_interface__ (version 2 or 3): data pointer, shape,
    typestr, strides in bytes (None: C-contiguous)."""
    cai = a.__cuda_array_interface__
    shape = tuple(cai["shape"])
    if len(shape) != 2:
        raise Exception(f"expected 2-D images, got shape {shape}")
    kinds = {"|u1": (N.BICOS_8U, 1), "<u2": (N.BICOS_16U, 2), "=u2": (N.BICOS_16U, 2)}
    if cai["typestr"] not in kinds:
        raise Exception(f"unimplemented cvtype_of(dtype={cai['typestr']})")
    itype, isz = kinds[cai["typestr"]]
    rows, cols = shape
    strides = cai.get("strides") or (cols * isz, isz)
    if strides[1] != isz or strides[0] < cols * isz:
        raise Exception("device images need unit column stride and a forward row step of at least one row")
    ptr = cai["data"][0]
    return N.image(ptr, rows, cols, itype, strides[0]), cai.get("stream")


def _frames_of(stack):
    """A list of 2-D images, or the 2-D slices of one 3-D (n, rows, cols)
    device array."""
    if _is_device(stack) and len(stack.__cuda_array_interface__["shape"]) == 3:
        return [stack[i] for i in range(stack.__cuda_array_interface__["shape"][0])]
    return list(stack)


def _match_device(stack0, stack1, cfg: Config):
    """Zero-copy match of device images through bicos_match_v1."""
    import torch

    from . import _stream_ptr
    imgs0, imgs1 = [_device_image(a) for a in stack0], [_device_image(a) for a in stack1]
    first = imgs0[0][0]
    for im, _ in imgs0 + imgs1:
        if (im.rows, im.cols, im.type) != (first.rows, first.cols, first.type):
            raise Exception("all images of both stacks must share size and type")
    streams = {s for _, s in imgs0 + imgs1 if s not in (None, 1, 2)}
    if len(streams) > 1:
        raise Exception("device images from more than one stream")
    is_torch = hasattr(stack0[0], "device") and hasattr(stack0[0], "data_ptr")
    dev = stack0[0].device if is_torch else torch.device("cuda", torch.cuda.current_device())
    stream = C.c_void_p(next(iter(streams))) if streams else _stream_ptr(None)
    nc = cfg.native()
    L = N.load()
    dt, ct = C.c_int32(), C.c_int32()
    N.check(L.bicos_output_types(C.byref(nc), C.byref(dt), C.byref(ct)))
    # outputs allocated for the stream the match runs on (torch's caching
    # allocator ties a block's reuse to its allocation stream)
    alloc_stream = torch.cuda.ExternalStream(stream.value, device=dev) if streams else torch.cuda.current_stream(dev)
    with torch.cuda.device(dev), torch.cuda.stream(alloc_stream):
        disp = torch.empty((first.rows, first.cols), dtype=torch.int16 if dt.value == N.BICOS_16S else torch.float32,
                           device=dev)
        corr = None
        if ct.value >= 0:
            corr = torch.empty((first.rows, first.cols),
                               dtype=torch.float64 if ct.value == N.BICOS_64F else torch.float32, device=dev)
    di = N.tensor_image(disp)
    ci = N.tensor_image(corr) if corr is not None else None
    a0 = N.image_array([im for im, _ in imgs0])
    a1 = N.image_array([im for im, _ in imgs1])
    st = L.bicos_match_v1(a0, a1, len(imgs0), C.byref(di), C.byref(ci) if ci is not None else None, C.byref(nc),
                          stream)
    try:
        N.check(st)
    except N.NativeError as e:
        raise_native(e)
    return disp, corr


def match(stack0, stack1, cfg: Config | None = None):
    """Match two lists of rectified images; returns (disparity, corrmap).

    disparity is int16 (INT16_MIN invalid), or float32 (NaN invalid) when a
    subpixel step is set; corrmap is float32 (float64 for Precision.Double),
    NaN where no correlation was computed, or None without a threshold.
    Host images give numpy results; device images (torch CUDA tensors,
    __cuda_array_interface__ objects, or one 3-D device stack per side)
    are matched in place and give torch CUDA tensors.
    """
    if stack0 is None or stack1 is None:
        raise TypeError("stacks must not be None")
    cfg = Config() if cfg is None else cfg
    stack0, stack1 = _frames_of(stack0), _frames_of(stack1)
    if stack0 and stack1 and (_is_device(stack0[0]) or _is_device(stack1[0])):
        if len(stack0) < 2:
            raise Exception("need at least two images")
        if len(stack1) != len(stack0):
            raise Exception("both stacks must hold the same number of images")
        if not all(_is_device(a) for a in stack0 + stack1):
            raise Exception("mixing host and device images")
        return _match_device(stack0, stack1, cfg)
    if not stack0 or not stack1:
        raise Exception("empty stacks")
    if len(stack0) < 2:
        raise Exception("need at least two images")
    if len(stack1) != len(stack0):
        raise Exception("both stacks must hold the same number of images")
    imgs0 = [_as_image(a) for a in stack0]
    imgs1 = [_as_image(a) for a in stack1]
    first = imgs0[0]
    rows, cols = first.shape
    step = first.strides[0]
    for a in imgs0 + imgs1:
        if a.shape != first.shape or a.dtype != first.dtype:
            raise Exception("all images of both stacks must share size and type")
        if a.strides[0] != step:
            step = None
    if step is None:
        imgs0 = [np.ascontiguousarray(a) for a in imgs0]
        imgs1 = [np.ascontiguousarray(a) for a in imgs1]
        step = cols * first.itemsize
    nc = cfg.native()
    L = N.load()
    dt, ct = C.c_int32(), C.c_int32()
    N.check(L.bicos_output_types(C.byref(nc), C.byref(dt), C.byref(ct)))
    disp = np.empty((rows, cols), np.int16 if dt.value == N.BICOS_16S else np.float32)
    corr = None
    if ct.value >= 0:
        corr = np.empty((rows, cols), np.float64 if ct.value == N.BICOS_64F else np.float32)
    n = len(imgs0)
    p0 = (C.c_void_p * n)(*[a.ctypes.data for a in imgs0])
    p1 = (C.c_void_p * n)(*[a.ctypes.data for a in imgs1])
    itype = N.BICOS_8U if first.dtype == np.uint8 else N.BICOS_16U
    st = L.bicos_match_host_v1(p0, p1, n, rows, cols, itype, step, disp.ctypes.data, disp.strides[0],
                               corr.ctypes.data if corr is not None else None,
                               corr.strides[0] if corr is not None else 0, C.byref(nc), None)
    try:
        N.check(st)
    except N.NativeError as e:
        raise_native(e)
    return disp, corr


def invalid_disparity(dtype):
    """INVALID_DISP<T> for int16 (INT16_MIN) and float32 (NaN)."""
    dt = np.dtype(dtype)
    if dt == np.int16:
        return int(np.iinfo(np.int16).min)
    if dt == np.float32:
        return float("nan")
    raise Exception(f"invalid_disparity undefined for {dt}")
