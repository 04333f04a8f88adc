"""ctypes front end for the CPU oracle.  TEST INFRASTRUCTURE ONLY.

Two libraries sit behind it:

* ``liboracle.so`` -- the plain-C restatement of libBICOS's matching path
  (``bicos_oracle.c``), built on any host by :func:`build`.
* ``_ref/libbicos_ref.so`` -- libBICOS's own CPU backend compiled from the
  reference sources by ``ref_build.sh``; present only where the reference
  tree exists.  Used to pin the restatement and to make tests/golden/.

Only tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline arm
use this module.  Stacks are planar numpy arrays of shape (n, rows, cols),
dtype uint8 or uint16.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libbicos_ref.so")

OK, ERR_EXCEPTION, ERR_INVALID_ARGUMENT = 0, 1, 2
FLAG_NODUPES, FLAG_CONSISTENCY = 1, 2
INVALID_I16 = -32768


class OrcConfig(C.Structure):
    _fields_ = [
        ("has_threshold", C.c_int32), ("nxcorr_threshold", C.c_float),
        ("has_subpixel_step", C.c_int32), ("subpixel_step", C.c_float),
        ("has_min_variance", C.c_int32), ("min_variance", C.c_float),
        ("mode", C.c_int32), ("precision", C.c_int32), ("variant", C.c_int32),
        ("max_lr_diff", C.c_int32), ("no_dupes", C.c_int32), ("max_bits", C.c_int32),
    ]


def make_config(threshold=0.5, step=None, min_variance=None, full=False,
                double=False, consistency=None, max_bits=256) -> OrcConfig:
    """consistency: None for NoDuplicates, else (max_lr_diff, no_dupes)."""
    c = OrcConfig()
    c.has_threshold = threshold is not None
    c.nxcorr_threshold = threshold if threshold is not None else 0.0
    c.has_subpixel_step = step is not None
    c.subpixel_step = step if step is not None else 0.0
    c.has_min_variance = min_variance is not None
    c.min_variance = min_variance if min_variance is not None else 0.0
    c.mode = 1 if full else 0
    c.precision = 1 if double else 0
    c.variant = 0 if consistency is None else 1
    c.max_lr_diff = consistency[0] if consistency else 1
    c.no_dupes = int(bool(consistency[1])) if consistency else 0
    c.max_bits = max_bits
    return c


def build(force: bool = False) -> str:
    """Compile bicos_oracle.c into liboracle.so (gcc, -ffp-contract=off)."""
    src = os.path.join(HERE, "bicos_oracle.c")
    if (not force and os.path.exists(ORACLE_SO)
            and os.path.getmtime(ORACLE_SO) >= os.path.getmtime(src)):
        return ORACLE_SO
    cc = os.environ.get("CC", "gcc")
    subprocess.check_call([cc, "-O3", "-std=c11", "-ffp-contract=off", "-fPIC", "-shared",
                           "-o", ORACLE_SO, src, "-lm", "-lpthread"])
    return ORACLE_SO


def build_ref() -> str | None:
    """Compile the reference CPU backend into _ref/ when its sources exist."""
    subprocess.check_call(["sh", os.path.join(HERE, "ref_build.sh")])
    return REF_SO if os.path.exists(REF_SO) else None


_lib = None
_ref = None


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build()
        _lib = C.CDLL(ORACLE_SO)
        _lib.orc_match.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                   C.POINTER(OrcConfig), C.c_void_p, C.c_void_p, C.c_int,
                                   C.c_char_p, C.c_int]
        _lib.orc_transform.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                       C.c_int, C.c_void_p, C.c_int]
        _lib.orc_search.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                    C.c_int, C.c_void_p, C.c_int]
        _lib.orc_agree.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                   C.c_int, C.c_float, C.c_int, C.c_float, C.c_int, C.c_void_p,
                                   C.c_int]
        _lib.orc_agree_subpixel.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                            C.c_int, C.c_int, C.c_float, C.c_float, C.c_int,
                                            C.c_float, C.c_int, C.c_void_p, C.c_void_p, C.c_int]
        _lib.orc_nxcorr_f.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_float]
        _lib.orc_nxcorr_f.restype = C.c_float
        _lib.orc_nxcorr_d.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_double]
        _lib.orc_nxcorr_d.restype = C.c_double
        _lib.orc_num_threads.argtypes = [C.c_int]
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref():
    global _ref
    if _ref is None:
        _ref = C.CDLL(REF_SO)
        _ref.ref_match.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                   C.POINTER(OrcConfig), C.c_void_p, C.c_void_p, C.c_char_p, C.c_int]
        _ref.ref_transform.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                       C.c_int, C.c_void_p]
        _ref.ref_search.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                    C.c_int, C.c_void_p]
        _ref.ref_agree.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                   C.c_int, C.c_float, C.c_int, C.c_float, C.c_void_p]
        _ref.ref_agree_subpixel.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                            C.c_int, C.c_int, C.c_float, C.c_float, C.c_int,
                                            C.c_float, C.c_void_p, C.c_void_p]
    return _ref


class OracleError(Exception):
    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


def required_bits(n: int, full: bool) -> int:
    return n * n - 2 * n + 3 if full else 4 * n - 7


def descriptor_words(bits: int, max_bits: int = 256) -> int:
    if bits <= 32:
        return 1
    if bits <= 64:
        return 2
    if bits <= 128:
        return 4
    if bits <= 256:
        return 8
    if bits <= max_bits and bits <= 512:
        return ((bits + 127) // 128) * 4
    return -1


def _stack(s):
    s = np.ascontiguousarray(s)
    assert s.ndim == 3 and s.dtype in (np.uint8, np.uint16)
    return s


def match(stack0, stack1, cfg: OrcConfig, corrmap=True, nthreads=0, use_ref=False):
    """Full matching pipeline.  Returns (disparity, corrmap or None)."""
    s0, s1 = _stack(stack0), _stack(stack1)
    n, rows, cols = s0.shape
    eb = s0.dtype.itemsize
    subpix = cfg.has_threshold and cfg.has_subpixel_step
    disp = np.empty((rows, cols), np.float32 if subpix else np.int16)
    corr = None
    if corrmap and cfg.has_threshold:
        corr = np.empty((rows, cols), np.float64 if cfg.precision == 1 else np.float32)
    err = C.create_string_buffer(512)
    if use_ref:
        rc = ref().ref_match(_p(s0), _p(s1), eb, n, rows, cols, C.byref(cfg), _p(disp), _p(corr), err, 512)
    else:
        rc = lib().orc_match(_p(s0), _p(s1), eb, n, rows, cols, C.byref(cfg), _p(disp), _p(corr),
                             nthreads, err, 512)
    if rc != OK:
        raise OracleError(rc, err.value.decode())
    return disp, corr


def transform(stack, full: bool, nwords: int | None = None, nthreads=0, use_ref=False):
    s = _stack(stack)
    n, rows, cols = s.shape
    if nwords is None:
        nwords = descriptor_words(required_bits(n, full), 512)
    out = np.zeros((rows, cols, nwords), np.uint32)
    if use_ref:
        rc = ref().ref_transform(_p(s), s.dtype.itemsize, n, rows, cols, int(full), nwords, _p(out))
        if rc != OK:
            raise OracleError(rc, "ref_transform failed")
    else:
        lib().orc_transform(_p(s), s.dtype.itemsize, n, rows, cols, int(full), nwords, _p(out), nthreads)
    return out


def search(d0, d1, flags: int, max_lr_diff: int = -1, nthreads=0, use_ref=False):
    d0 = np.ascontiguousarray(d0, np.uint32)
    d1 = np.ascontiguousarray(d1, np.uint32)
    rows, cols, nwords = d0.shape
    out = np.empty((rows, cols), np.int16)
    if use_ref:
        rc = ref().ref_search(_p(d0), _p(d1), rows, cols, nwords, flags, max_lr_diff, _p(out))
        if rc != OK:
            raise OracleError(rc, "ref_search failed")
    else:
        lib().orc_search(_p(d0), _p(d1), rows, cols, nwords, flags, max_lr_diff, _p(out), nthreads)
    return out


def agree(disp, stack0, stack1, thr, min_var_scaled=None, double=False, nthreads=0, use_ref=False):
    """In-place-style NCC agreement; returns (new int16 disparity, corrmap).
    min_var_scaled is the per-stack threshold (min_variance * n)."""
    s0, s1 = _stack(stack0), _stack(stack1)
    n, rows, cols = s0.shape
    d = np.array(disp, np.int16, copy=True)
    corr = np.full((rows, cols), np.nan, np.float64 if double else np.float32)
    hm = min_var_scaled is not None
    mv = float(min_var_scaled) if hm else 0.0
    if use_ref:
        assert not double
        ref().ref_agree(_p(d), _p(s0), _p(s1), s0.dtype.itemsize, n, rows, cols, thr, int(hm), mv, _p(corr))
    else:
        lib().orc_agree(_p(d), _p(s0), _p(s1), s0.dtype.itemsize, n, rows, cols, thr, int(hm), mv,
                        int(double), _p(corr), nthreads)
    return d, corr


def agree_subpixel(disp, stack0, stack1, thr, step, min_var_scaled=None, double=False, nthreads=0,
                   use_ref=False):
    s0, s1 = _stack(stack0), _stack(stack1)
    n, rows, cols = s0.shape
    d = np.ascontiguousarray(disp, np.int16)
    out = np.empty((rows, cols), np.float32)
    corr = np.full((rows, cols), np.nan, np.float64 if double else np.float32)
    hm = min_var_scaled is not None
    mv = float(min_var_scaled) if hm else 0.0
    if use_ref:
        assert not double
        ref().ref_agree_subpixel(_p(d), _p(s0), _p(s1), s0.dtype.itemsize, n, rows, cols, thr, step,
                                 int(hm), mv, _p(out), _p(corr))
    else:
        lib().orc_agree_subpixel(_p(d), _p(s0), _p(s1), s0.dtype.itemsize, n, rows, cols, thr, step,
                                 int(hm), mv, int(double), _p(out), _p(corr), nthreads)
    return out, corr


def nxcorr_f(x, y, min_var=None):
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    return lib().orc_nxcorr_f(_p(x), _p(y), len(x), int(min_var is not None),
                              float(min_var or 0.0))


def nxcorr_d(x, y, min_var=None):
    x = np.ascontiguousarray(x, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    return lib().orc_nxcorr_d(_p(x), _p(y), len(x), int(min_var is not None),
                              float(min_var or 0.0))


def _moments_lib():
    L = lib()
    if not getattr(L, "_mom_sig", False):
        L.orc_moments.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                  C.c_float, C.c_float, C.c_int, C.c_float, C.c_int, C.c_int, C.c_void_p,
                                  C.c_void_p, C.c_int]
        L._mom_sig = True
    return L


def moments(disp, stack0, stack1, thr, step=None, min_var_scaled=None, double=True, nthreads=0):
    """Moment form of the agreement (the library's extension): returns
    (int16 disparity, corrmap) without a step, (float disparity, corrmap)
    with one."""
    s0, s1 = _stack(stack0), _stack(stack1)
    n, rows, cols = s0.shape
    d = np.ascontiguousarray(disp, np.int16)
    mode = 0 if step is None else 1
    out = np.empty((rows, cols), np.int16 if mode == 0 else np.float32)
    corr = np.empty((rows, cols), np.float64 if double else np.float32)
    hm = min_var_scaled is not None
    L = _moments_lib()
    L.orc_moments(_p(d), _p(s0), _p(s1), s0.dtype.itemsize, n, rows, cols, thr, step or 0.0, int(hm),
                  float(min_var_scaled or 0.0), int(double), mode, _p(out), _p(corr), nthreads)
    return out, corr


def features(disp, stack0, stack1, nthreads=0):
    """Feature rows of the learned subpixel form (orc_moments mode 2):
    (rows, cols, 8) float32."""
    s0, s1 = _stack(stack0), _stack(stack1)
    n, rows, cols = s0.shape
    d = np.ascontiguousarray(disp, np.int16)
    out = np.empty((rows, cols, 8), np.float32)
    L = _moments_lib()
    L.orc_moments(_p(d), _p(s0), _p(s1), s0.dtype.itemsize, n, rows, cols, 0.0, 0.0, 0, 0.0, 0, 2, _p(out),
                  None, nthreads)
    return out


def learned_check(disp, stack0, stack1, thr, proposal, feats, min_var_scaled=None, double=False, drop=0.002,
                  nthreads=0):
    """The learned form's check of given proposals: (float disparity,
    corrmap, fallback mask); fallback pixels are NaN here and decided by the
    sweep (agree_subpixel)."""
    s0, s1 = _stack(stack0), _stack(stack1)
    n, rows, cols = s0.shape
    d = np.ascontiguousarray(disp, np.int16)
    prop = np.ascontiguousarray(proposal, np.float32)
    ft = np.ascontiguousarray(feats, np.float32)
    out = np.empty((rows, cols), np.float32)
    corr = np.full((rows, cols), np.nan, np.float64 if double else np.float32)
    fb = np.zeros((rows, cols), np.uint8)
    hm = min_var_scaled is not None
    L = lib()
    if not getattr(L, "_lc_sig", False):
        L.orc_learned_check.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                        C.c_float, C.c_int, C.c_float, C.c_int, C.c_void_p, C.c_void_p,
                                        C.c_float, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        L._lc_sig = True
    L.orc_learned_check(_p(d), _p(s0), _p(s1), s0.dtype.itemsize, n, rows, cols, thr, int(hm),
                        float(min_var_scaled or 0.0), int(double), _p(prop), _p(ft), drop, _p(out), _p(corr),
                        _p(fb), nthreads)
    return out, corr, fb.astype(bool)
