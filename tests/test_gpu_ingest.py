"""Frame-by-frame ingest (bicos_ingest_*) on the GPU: frames pushed in any
order, from numpy or pinned torch buffers, match bit for bit the same stack
matched in one call; missing and out-of-range frames are errors; a frame
pushed again replaces the old one."""
import numpy as np
import pytest
import torch

import libbicos_gb300 as lbg
from gpu_util import assert_same, dev, host
from libbicos_gb300 import pybicos, scenes

pytestmark = pytest.mark.gpu


def _cfg(step=0.1):
    c = pybicos.Config()
    c.nxcorr_threshold, c.subpixel_step, c.min_variance = 0.9, step, 2.0
    c.mode = pybicos.Limited
    return c


@pytest.mark.parametrize("bits", [8, 12])
def test_ingest_equals_one_call(cuda, bits):
    sc = scenes.make_scene(40, 200, 12, seed=bits, bits=bits)
    ing = lbg.Ingest(40, 200, 12, sc.left.dtype)
    order = np.random.default_rng(bits).permutation(12)
    for k, t in enumerate(order):
        if k % 2:
            ing.push(int(t), sc.left[t], sc.right[t])
        else:  # pinned host tensors: asynchronous copies
            l = torch.from_numpy(sc.left[t].copy()).pin_memory()
            r = torch.from_numpy(sc.right[t].copy()).pin_memory()
            ing.push(int(t), l, r)
    for step in (None, 0.1):
        d, c = ing.match(_cfg(step))
        wd, wc = lbg.match_device(dev(sc.left, cuda), dev(sc.right, cuda), _cfg(step))
        assert_same(host(d), host(wd), f"bits={bits} step={step}")
        assert_same(host(c), host(wc), f"bits={bits} step={step} corr")
    ing.close()


def test_ingest_errors_and_replacement(cuda):
    sc = scenes.make_scene(16, 96, 6, seed=3)
    other = scenes.make_scene(16, 96, 6, seed=4)
    ing = lbg.Ingest(16, 96, 6)
    for t in range(5):
        ing.push(t, sc.left[t], sc.right[t])
    with pytest.raises(pybicos.Exception, match="frame 5 of the stack was not pushed"):
        ing.match(_cfg())
    with pytest.raises(ValueError, match="outside the stack"):
        ing.push(6, sc.left[0], sc.right[0])
    ing.push(5, other.left[5], other.right[5])
    ing.push(5, sc.left[5], sc.right[5])  # replaces the frame pushed before
    d, _ = ing.match(_cfg())
    wd, _ = lbg.match_device(dev(sc.left, cuda), dev(sc.right, cuda), _cfg())
    assert_same(host(d), host(wd))
    for t in range(6):
        ing.push(t, other.left[t], other.right[t])
    d, _ = ing.match(_cfg())
    wd, _ = lbg.match_device(dev(other.left, cuda), dev(other.right, cuda), _cfg())
    assert_same(host(d), host(wd))


def test_push_on_another_stream_after_match(cuda):
    """a capture thread pushes the next stack on its upload stream while the
    previous match still runs on a compute stream: the handle orders each
    push after the earlier matches, so both matches see their own stack"""
    a = scenes.make_scene(512, 1024, 12, seed=30)
    b = scenes.make_scene(512, 1024, 12, seed=31)
    pin = lambda x: torch.from_numpy(np.ascontiguousarray(x)).pin_memory()
    frames_b = [(pin(b.left[t]), pin(b.right[t])) for t in range(12)]
    compute, upload = torch.cuda.Stream(), torch.cuda.Stream()
    ing = lbg.Ingest(512, 1024, 12)
    for t in range(12):
        ing.push(t, a.left[t], a.right[t], stream=compute)
    torch.cuda.synchronize()
    for _ in range(3):
        with torch.cuda.stream(compute):
            da, ca = ing.match(_cfg(0.1), stream=compute)
        for t in range(12):  # no host synchronisation in between
            ing.push(t, frames_b[t][0], frames_b[t][1], stream=upload)
        with torch.cuda.stream(upload):
            db, cb = ing.match(_cfg(0.1), stream=upload)
        torch.cuda.synchronize()
        wa, wca = lbg.match_device(dev(a.left, cuda), dev(a.right, cuda), _cfg(0.1))
        wb, wcb = lbg.match_device(dev(b.left, cuda), dev(b.right, cuda), _cfg(0.1))
        assert_same(host(da), host(wa), "stack a")
        assert_same(host(ca), host(wca), "stack a corr")
        assert_same(host(db), host(wb), "stack b")
        assert_same(host(cb), host(wcb), "stack b corr")
        for t in range(12):
            ing.push(t, a.left[t], a.right[t], stream=compute)
    ing.close()
