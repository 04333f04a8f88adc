"""Helpers for the GPU parity tests: upload numpy stacks, compare with the oracle."""
import numpy as np


def dev(a, device):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(device)


def host(t):
    import torch
    a = t.cpu()
    if a.dtype == torch.int32:
        return a.numpy().view(np.uint32)
    return a.numpy()


def assert_same(a, b, what=""):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape and a.dtype == b.dtype, (what, a.shape, b.shape, a.dtype, b.dtype)
    if a.dtype.kind == "f":
        eq = (a == b) | (np.isnan(a) & np.isnan(b))
    else:
        eq = a == b
    if not eq.all():
        idx = np.argwhere(~eq)[:5]
        raise AssertionError(f"{what}: {int((~eq).sum())} of {eq.size} differ, first at {idx.tolist()}: "
                             f"{[ (a[tuple(i)], b[tuple(i)]) for i in idx]}")
