"""ctypes binding of the bicos_gb300 C ABI (include/bicos_c.h).

The shared library is built in-tree by ``libbicos_gb300.build``.  Loading
fails loudly when it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

BICOS_8U, BICOS_16U, BICOS_16S, BICOS_32F, BICOS_64F = 0, 2, 3, 5, 6
OK, ERR_EXCEPTION, ERR_INVALID_ARGUMENT, ERR_CUDA = 0, 1, 2, 3
NXCORR_REFERENCE, NXCORR_MOMENTS, NXCORR_LEARNED = 0, 1, 2
FLAG_NODUPES, FLAG_CONSISTENCY = 1, 2

_TYPE_OF_DTYPE = {"uint8": BICOS_8U, "uint16": BICOS_16U, "int16": BICOS_16S,
                  "float32": BICOS_32F, "float64": BICOS_64F}


class Image(C.Structure):
    _fields_ = [("data", C.c_void_p), ("step", C.c_size_t), ("rows", C.c_int32),
                ("cols", C.c_int32), ("type", C.c_int32), ("reserved", C.c_int32)]


class Config(C.Structure):
    _fields_ = [
        ("has_threshold", C.c_int32), ("nxcorr_threshold", C.c_float),
        ("has_subpixel_step", C.c_int32), ("subpixel_step", C.c_float),
        ("has_min_variance", C.c_int32), ("min_variance", C.c_float),
        ("mode", C.c_int32), ("precision", C.c_int32), ("variant", C.c_int32),
        ("max_lr_diff", C.c_int32), ("no_dupes", C.c_int32), ("max_bits", C.c_int32),
        ("nxcorr_form", C.c_int32),
    ]


class BatchItem(C.Structure):
    _fields_ = [("stack0", C.POINTER(Image)), ("stack1", C.POINTER(Image)), ("n", C.c_uint32),
                ("disparity", C.POINTER(Image)), ("corrmap", C.POINTER(Image)), ("cfg", C.POINTER(Config))]


class BatchTuning(C.Structure):
    _fields_ = [("transform_block", C.c_int32), ("ctas_per_sm", C.c_int32), ("claim", C.c_int32),
                ("branches", C.c_int32), ("persistent", C.c_int32)]


class NativeError(Exception):
    """A non-OK bicos_status with the library's message."""

    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


_lib = None


def lib_path() -> str:
    return _build.LIB


def load():
    """Load the in-tree library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        raise ImportError(f"bicos_gb300 native library not built ({path}); run libbicos_gb300.build.build()")
    lib = C.CDLL(path)
    P, I, U, F, S = C.c_void_p, C.c_int32, C.c_uint32, C.c_float, C.c_size_t
    IMG = C.POINTER(Image)
    CFG = C.POINTER(Config)
    sig = {
        "bicos_version": ([], C.c_char_p),
        "bicos_last_error": ([], C.c_char_p),
        "bicos_config_default": ([CFG], C.c_int),
        "bicos_output_types": ([CFG, C.POINTER(I), C.POINTER(I)], C.c_int),
        "bicos_descriptor_words": ([U, I, I], I),
        "bicos_match_v1": ([IMG, IMG, U, IMG, IMG, CFG, P], C.c_int),
        "bicos_match_host_v1": ([C.POINTER(P), C.POINTER(P), U, I, I, I, S, P, S, P, S, CFG, P], C.c_int),
        "bicos_release_scratch": ([], C.c_int),
        "bicos_stage_timing": ([I], C.c_int),
        "bicos_kernel_faults": ([], I),
        "bicos_tc_fp8_rate_v1": ([I, C.POINTER(C.c_double)], C.c_int),
        "bicos_stage_times": ([C.POINTER(C.c_float), C.POINTER(I)], C.c_int),
        "bicos_descriptor_transform_v1": ([IMG, U, I, U, P, P], C.c_int),
        "bicos_search_v1": ([P, P, I, I, U, I, I, IMG, P], C.c_int),
        "bicos_search_bits_v1": ([P, P, I, I, U, I, I, I, IMG, P], C.c_int),
        "bicos_reproject_v1": ([IMG, C.POINTER(C.c_double), IMG, P], C.c_int),
        "bicos_match_points_v1": ([IMG, IMG, U, IMG, IMG, CFG, C.POINTER(C.c_double), IMG, P], C.c_int),
        "bicos_png_unfilter": ([P, P, C.c_int32, S, C.c_int32], C.c_int32),
        "bicos_ingest_create": ([C.POINTER(P), I, I, U, I], C.c_int),
        "bicos_ingest_destroy": ([P], C.c_int),
        "bicos_ingest_push_v1": ([P, U, P, P, S, P], C.c_int),
        "bicos_ingest_match_v1": ([P, IMG, IMG, CFG, P], C.c_int),
        "bicos_search_noalloc_v1": ([P, P, I, I, U, I, I, IMG, P], C.c_int),
        "bicos_agree_v1": ([IMG, IMG, IMG, U, F, I, F, I, IMG, P], C.c_int),
        "bicos_agree_subpixel_v1": ([IMG, IMG, IMG, U, F, F, I, F, I, IMG, IMG, P], C.c_int),
        "bicos_subpixel_features_v1": ([IMG, IMG, IMG, U, IMG, P], C.c_int),
        "bicos_agree_learned_v1": ([IMG, IMG, IMG, U, F, F, I, F, I, IMG, IMG, IMG, C.POINTER(I), P], C.c_int),
        "bicos_learned_model_v1": ([P, S], C.c_int),
        "bicos_learned_model_installed": ([], C.c_int),
        "bicos_learned_model_floats_v1": ([P, C.c_int], C.c_int),
        "bicos_mlp_sizes": ([C.POINTER(C.c_int), C.POINTER(C.c_int)], None),
        "bicos_mlp_grad_v1": ([P, P, C.c_int, P, P, P], C.c_int),
        "bicos_mlp_adam_v1": ([P, P, P, P, C.c_int, F, F, P], C.c_int),
        "bicos_mlp_propose_v1": ([P, P, C.c_int, P, P], C.c_int),
        "bicos_batch_create": ([C.POINTER(P)], C.c_int),
        "bicos_batch_destroy": ([P], C.c_int),
        "bicos_match_batch_v1": ([P, C.POINTER(BatchItem), U, P], C.c_int),
        "bicos_batch_autotune_v1": ([P, C.POINTER(BatchItem), U, P, C.POINTER(BatchTuning)], C.c_int),
        "bicos_batch_get_tuning_v1": ([P, C.POINTER(BatchTuning)], C.c_int),
        "bicos_batch_set_tuning_v1": ([P, C.POINTER(BatchTuning)], C.c_int),
        "bicos_batch_captures": ([P], I),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def check(status: int) -> None:
    if status != OK:
        raise NativeError(status, load().bicos_last_error().decode())


def default_config() -> Config:
    c = Config()
    load().bicos_config_default(C.byref(c))
    return c


def image(ptr: int, rows: int, cols: int, type_: int, step: int) -> Image:
    return Image(C.c_void_p(ptr), step, rows, cols, type_, 0)


def type_of(dtype) -> int:
    name = str(dtype).replace("torch.", "")
    if name not in _TYPE_OF_DTYPE:
        raise TypeError(f"unsupported dtype {dtype}")
    return _TYPE_OF_DTYPE[name]


def tensor_image(t) -> Image:
    """bicos_image view of a 2-D CUDA tensor (row-contiguous, any row pitch).
    Kernels write through these views, so host memory is refused here."""
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor (device memory)")
    if t.dim() != 2 or t.stride(1) != 1:
        raise ValueError("expected a 2-D tensor with unit column stride")
    return image(t.data_ptr(), t.shape[0], t.shape[1], type_of(t.dtype), t.stride(0) * t.element_size())


TYPE_32FC3 = 21


def points_image(t) -> Image:
    """bicos_image view of a (rows, cols, 3) float32 CUDA tensor (packed
    pixels, any row pitch)."""
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor (device memory)")
    if t.dim() != 3 or t.shape[2] != 3 or t.stride(2) != 1 or t.stride(1) != 3 or str(t.dtype) != "torch.float32":
        raise ValueError("expected a (rows, cols, 3) float32 tensor with packed pixels")
    return image(t.data_ptr(), t.shape[0], t.shape[1], TYPE_32FC3, t.stride(0) * 4)


def image_array(images) -> C.Array:
    arr = (Image * len(images))()
    for i, im in enumerate(images):
        arr[i] = im
    return arr
