"""pybicos.match on device images, matched where they lie: torch CUDA
tensors (lists, or one 3-D stack per side) and bare
__cuda_array_interface__ objects give the same results as host images
(which libBICOS's pybicos uploads and downloads on every call,
src/pybicos.cpp:81-82, 94-95) and as the oracle."""
import numpy as np
import pytest
import torch

from gpu_util import assert_same, dev
from libbicos_gb300 import pybicos, scenes

pytestmark = pytest.mark.gpu


class CaiOnly:
    """A device array known only through __cuda_array_interface__ (as CuPy
    or Numba arrays present themselves); optionally with a row pitch."""

    def __init__(self, t, stream=None):
        self._t = t  # keeps the memory alive
        self.__cuda_array_interface__ = {
            "shape": tuple(t.shape), "typestr": "|u1" if t.dtype == torch.uint8 else "<u2",
            "data": (t.data_ptr(), False), "version": 3,
            "strides": (t.stride(0) * t.element_size(), t.element_size()),
            "stream": stream}


def cfg(step=0.1, cons=None, double=False):
    c = pybicos.Config()
    c.nxcorr_threshold, c.subpixel_step, c.min_variance = 0.9, step, 2.0
    c.precision = pybicos.Double if double else pybicos.Single
    if cons:
        c.variant = pybicos.Variant.Consistency(*cons)
    return c


@pytest.mark.parametrize("bits", [8, 12])
@pytest.mark.parametrize("step,cons,double", [(0.1, None, False), (None, (1, False), False), (0.25, None, True)])
def test_device_images_equal_host_images(cuda, oracle, bits, step, cons, double):
    sc = scenes.make_scene(48, 200, 12, seed=bits, bits=bits)
    c = cfg(step, cons, double)
    hd, hc = pybicos.match(list(sc.left), list(sc.right), c)
    wd, wc = oracle.match(sc.left, sc.right, oracle.make_config(threshold=0.9, step=step, min_variance=2.0,
                                                                consistency=cons, double=double))
    assert_same(hd, wd, "host path vs oracle")
    L, R = dev(sc.left, cuda), dev(sc.right, cuda)
    for name, s0, s1 in (("list", list(L), list(R)), ("stack", L, R)):
        d, corr = pybicos.match(s0, s1, c)
        assert d.is_cuda and corr.is_cuda, name
        torch.cuda.synchronize()
        assert_same(d.cpu().numpy(), hd, name)
        assert_same(corr.cpu().numpy(), hc, name + " corrmap")


def test_cuda_array_interface_objects_and_pitch(cuda):
    sc = scenes.make_scene(40, 160, 10, seed=3)
    c = cfg()
    hd, hc = pybicos.match(list(sc.left), list(sc.right), c)
    # pitched device frames: 160 columns inside rows of 224 bytes
    pad0 = torch.zeros((10, 40, 224), dtype=torch.uint8, device=cuda)
    pad1 = torch.zeros((10, 40, 224), dtype=torch.uint8, device=cuda)
    pad0[:, :, :160] = dev(sc.left, cuda)
    pad1[:, :, :160] = dev(sc.right, cuda)
    s = torch.cuda.Stream()
    torch.cuda.synchronize()
    f0 = [CaiOnly(pad0[t, :, :160], stream=s.cuda_stream) for t in range(10)]
    f1 = [CaiOnly(pad1[t, :, :160], stream=s.cuda_stream) for t in range(10)]
    d, corr = pybicos.match(f0, f1, c)
    s.synchronize()
    assert_same(d.cpu().numpy(), hd)
    assert_same(corr.cpu().numpy(), hc)


def test_device_path_errors(cuda):
    sc = scenes.make_scene(16, 64, 6, seed=4)
    L = dev(sc.left, cuda)
    with pytest.raises(pybicos.Exception, match="mixing host and device"):
        pybicos.match(list(L), [np.asarray(a) for a in sc.right], cfg())
    with pytest.raises(pybicos.Exception, match="same number of images"):
        pybicos.match(list(L), list(L)[:5], cfg())
    with pytest.raises(pybicos.Exception, match="share size and type"):
        pybicos.match(list(L), list(L[:, :8]), cfg())
