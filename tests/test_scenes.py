"""The seeded synthetic scene generator (stand-in for the reference's dataset)."""
import numpy as np

from libbicos_gb300 import scenes


def test_deterministic_and_typed():
    a = scenes.make_scene(40, 90, 5, seed=3)
    b = scenes.make_scene(40, 90, 5, seed=3)
    c = scenes.make_scene(40, 90, 5, seed=4)
    assert a.left.dtype == np.uint8 and a.left.shape == (5, 40, 90)
    assert np.array_equal(a.left, b.left) and np.array_equal(a.right, b.right)
    assert not np.array_equal(a.left, c.left)
    s12 = scenes.make_scene(20, 50, 3, seed=1, bits=12)
    assert s12.left.dtype == np.uint16 and s12.left.max() <= 4095


def test_disparity_range_and_flat_region():
    s = scenes.make_scene(120, 300, 4, seed=9, d_range=(20.0, 120.0))
    assert s.disparity.min() >= 20.0 - 1e-3 and s.disparity.max() <= 120.0 + 1e-3
    # the flat 40-DN rectangle is present in every frame
    flat = np.abs(s.left.astype(int) - 40) <= 8
    assert flat.all(axis=0).mean() > 0.05


def test_right_is_shifted_left():
    s = scenes.make_scene(60, 400, 3, seed=2, d_range=(40.0, 40.0), flat_fraction=0.0)
    # constant disparity 40: right(x) ~ left(x + 40)
    l, r = s.left[0].astype(float), s.right[0].astype(float)
    err = np.abs(r[:, :300] - l[:, 40:340]).mean()
    assert err < 4.0
