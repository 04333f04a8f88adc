"""bicos_search_noalloc_v1: the search stage for callers that cannot
allocate device memory while they run (fixed memory plans, host frameworks
that own all device memory, code that must not hit an allocator mid-
pipeline).  Its consistency scratch is a fixed array inside the library, so
this checks it against the allocating bicos_search_v1 through the C ABI, on
two calls in a row (the second must not see the first's leftovers), and
that sizes past its fixed limit are refused.  Integer disparities: the
tolerance is exact equality, as for every search test.  Kept in a file
pytest collects last."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIMIT_PIXELS = 4 << 20


def _scene_descriptors(device, rows, cols, n, seed):
    import torch

    import libbicos_gb300 as lbg
    from libbicos_gb300 import scenes
    sc = scenes.make_scene(rows, cols, n, seed=seed)
    d0 = lbg.descriptor_transform(torch.from_numpy(sc.left).to(device), False)
    d1 = lbg.descriptor_transform(torch.from_numpy(sc.right).to(device), False)
    return d0, d1


def _run(native, entry, d0, d1, flags, lr):
    import torch
    rows, cols, nw = d0.shape
    out = torch.full((rows, cols), 7, dtype=torch.int16, device=d0.device)
    img = native.tensor_image(out)
    st = getattr(native.load(), entry)(C.c_void_p(d0.data_ptr()), C.c_void_p(d1.data_ptr()), rows, cols, nw,
                                       flags, lr, C.byref(img), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    native.check(st)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_noalloc_matches_allocating_search_twice(cuda, native):
    # two calls in a row with different inputs and sizes, all flag sets
    cases = [((96, 640, 12, 1), 3, 1), ((120, 700, 20, 2), 2, 2)]
    for (rows, cols, n, seed), flags, lr in cases:
        d0, d1 = _scene_descriptors(cuda, rows, cols, n, seed)
        want = _run(native, "bicos_search_v1", d0, d1, flags, lr)
        got = _run(native, "bicos_search_noalloc_v1", d0, d1, flags, lr)
        assert np.array_equal(got, want), (rows, cols, flags)
        assert (want != -32768).mean() > 0.3
    d0, d1 = _scene_descriptors(cuda, 64, 512, 9, 3)
    for flags in (0, 1, 2, 3):
        a = _run(native, "bicos_search_noalloc_v1", d0, d1, flags, 1)
        b = _run(native, "bicos_search_noalloc_v1", d0, d1, flags, 1)
        want = _run(native, "bicos_search_v1", d0, d1, flags, 1)
        assert np.array_equal(a, want) and np.array_equal(b, want), flags


def test_noalloc_refuses_sizes_past_its_scratch(cuda, native):
    import torch
    rows, cols = 2049, 2048  # one row past the 4 Mi-pixel limit
    assert rows * cols > LIMIT_PIXELS
    d = torch.zeros((1,), dtype=torch.int32, device=cuda)  # never read: refused before any launch
    out = torch.zeros((1,), dtype=torch.int16, device=cuda)
    img = native.image(out.data_ptr(), rows, cols, native.BICOS_16S, cols * 2)
    st = native.load().bicos_search_noalloc_v1(C.c_void_p(d.data_ptr()), C.c_void_p(d.data_ptr()), rows, cols, 4,
                                               3, 1, C.byref(img), None)
    assert st == native.ERR_INVALID_ARGUMENT
    assert b"4194304" in native.load().bicos_last_error()
