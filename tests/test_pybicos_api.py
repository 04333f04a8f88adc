"""The pybicos surface mirrors the reference module (src/pybicos.cpp:121-177)."""
import math

import numpy as np
import pytest

from libbicos_gb300 import pybicos


def test_config_defaults_and_repr():
    c = pybicos.Config()
    assert c.nxcorr_threshold == 0.5 and c.subpixel_step is None and c.min_variance is None
    assert c.mode == pybicos.TransformMode.Limited and c.precision == pybicos.Precision.Single
    assert repr(c.variant) == "NoDuplicates"
    assert repr(c) == ("Config( nxcorr_threshold = optional(0.5), subpixel_step = none, min_variance = none, "
                       "mode = Limited, precision = Single, variant = NoDuplicates )")
    c.nxcorr_threshold = 0.9
    c.subpixel_step = 0.1
    c.variant = pybicos.Variant.Consistency(max_lr_diff=2, no_dupes=True)
    assert "nxcorr_threshold = optional(0.9)" in repr(c)
    assert "subpixel_step = optional(0.1)" in repr(c)
    assert "Consistency( max_lr_diff = 2, no_dupes = true )" in repr(c)
    assert c.nxcorr_threshold == float(np.float32(0.9))  # stored as float, as std::optional<float>


def test_enums_exported_at_module_level():
    assert pybicos.Full is pybicos.TransformMode.Full
    assert pybicos.Limited is pybicos.TransformMode.Limited
    assert pybicos.Double is pybicos.Precision.Double
    assert pybicos.Single is pybicos.Precision.Single
    assert repr(pybicos.Variant.Consistency()) == "Consistency( max_lr_diff = 1, no_dupes = false )"


def test_invalid_disparity():
    assert pybicos.invalid_disparity(np.int16) == -32768
    assert math.isnan(pybicos.invalid_disparity(np.float32))
    with pytest.raises(pybicos.Exception):
        pybicos.invalid_disparity(np.float64)


def test_match_argument_errors():
    z = np.zeros((4, 8), np.uint8)
    with pytest.raises(pybicos.Exception, match="empty stacks"):
        pybicos.match([], [z, z])
    with pytest.raises(TypeError):
        pybicos.match(None, [z, z])
    with pytest.raises(pybicos.Exception, match="need at least two images"):
        pybicos.match([z], [z])
    with pytest.raises(pybicos.Exception):
        pybicos.match([z.astype(np.float32)] * 3, [z.astype(np.float32)] * 3)


def test_too_large_is_value_error(native):
    z = np.zeros((4, 8), np.uint8)
    with pytest.raises(ValueError, match="input stacks too large, would require 257 bits"):
        pybicos.match([z] * 66, [z] * 66)
    cfg = pybicos.Config()
    cfg.mode = pybicos.Full
    with pytest.raises(ValueError, match="would require 258 bits"):
        pybicos.match([z] * 17, [z] * 17, cfg)


def test_host_images_get_a_forward_row_step():
    """Views with negative or overlapping row steps become contiguous copies
    before their pointers reach the host-buffer call."""
    import numpy as np
    from libbicos_gb300.pybicos import _as_image
    a = np.arange(6 * 8, dtype=np.uint8).reshape(6, 8)
    for v in (a[::-1], a[:, ::-1], a[::-2], np.lib.stride_tricks.as_strided(a, (6, 8), (0, 1))):
        img = _as_image(v)
        assert img.strides[1] == 1 and img.strides[0] >= 8
        assert np.array_equal(img, v)
    assert _as_image(a[:, :4]).strides[0] == 8  # a padded row step is kept (no copy)
