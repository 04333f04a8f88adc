"""bicos-cli's point-cloud step and the command-line front end on the GPU:
bicos_reproject_v1 against the oracle's FP64 reprojection (error bound of
the FP32 kernel), and the CLI end to end on a synthetic stack written as
PNG files -- its disparity bit-identical to a direct match, its .xyz the
reference's filters applied to the GPU points."""
import io
import os

import numpy as np
import pytest
import torch

import libbicos_gb300 as lbg
from gpu_util import assert_same, dev, host
from libbicos_gb300 import cli, imageio, pybicos, scenes
from oracle import pointcloud as opc

pytestmark = pytest.mark.gpu

EPS = float(np.finfo(np.float32).eps)


def _bound(disp, q):
    """Per-coordinate error bound of the FP32 kernel against the FP64
    reference: a few roundings of each Q term sum, the reciprocal of W and
    the final products (16 eps with margin)."""
    rows, cols = disp.shape
    ys, xs = np.mgrid[0:rows, 0:cols].astype(np.float64)
    d = disp.astype(np.float64)
    terms = [np.abs(q[i, 0] * xs) + np.abs(q[i, 1] * ys) + np.abs(q[i, 2] * d) + np.abs(q[i, 3]) for i in range(4)]
    w = q[3, 0] * xs + q[3, 1] * ys + q[3, 2] * d + q[3, 3]
    with np.errstate(divide="ignore", invalid="ignore"):
        ref = np.stack([(q[i, 0] * xs + q[i, 1] * ys + q[i, 2] * d + q[i, 3]) / w for i in range(3)], -1)
        b = 16 * EPS * (np.stack(terms[:3], -1) / np.abs(w)[..., None] + np.abs(ref) * (terms[3] / np.abs(w))[..., None]
                        + np.abs(ref))
    return b


@pytest.mark.parametrize("dtype", ["int16", "float32"])
def test_reproject_vs_fp64_oracle(cuda, dtype):
    rng = np.random.default_rng(5)
    rows, cols = 37, 301
    q = np.array([[1.0, 0.0, 0.0, -150.25], [0.0, 1.0, 0.0, -18.5], [0.0, 0.0, 0.0, 1200.0],
                  [0.0, 0.0, 0.0125, 0.03125]])
    q[0, 1], q[1, 0], q[3, 0] = 1e-3, -2e-3, 1e-5  # a general Q, not only the rectified form
    if dtype == "int16":
        disp = rng.integers(-40, 200, size=(rows, cols)).astype(np.int16)
        disp[rng.random((rows, cols)) < 0.1] = -32768
    else:
        disp = rng.uniform(-40, 200, size=(rows, cols)).astype(np.float32)
        disp[rng.random((rows, cols)) < 0.1] = np.nan
    got = host(lbg.reproject(dev(disp, cuda), q))
    want = opc.reproject(disp, q)
    nan = np.isnan(want)
    assert np.array_equal(np.isnan(got), nan)
    err = np.abs(got.astype(np.float64) - want.astype(np.float64))
    bound = _bound(disp, q) + np.abs(want) * EPS
    assert np.all(err[~nan] <= bound[~nan]), float(np.max((err - bound)[~nan]))


def test_reproject_w_zero_and_padding(cuda):
    q = np.array([[1.0, 0.0, 0.0, -2.0], [0.0, 1.0, 0.0, -1.0], [0.0, 0.0, 0.0, 100.0], [0.0, 0.0, 0.25, 0.0]])
    disp = np.array([[0, 4, 8], [0, -4, 2]], np.int16)
    full = torch.zeros((2, 8), dtype=torch.int16, device=cuda)
    full[:, :3] = dev(disp, cuda)
    got = host(lbg.reproject(full[:, :3], q))  # a pitched view
    assert np.array_equal(got[0, 0], [0, 0, 0]) and np.array_equal(got[1, 0], [0, 0, 0])
    assert np.allclose(got, opc.reproject(disp, q), rtol=1e-6, atol=1e-6)


def test_reproject_rejects_bad_arguments(cuda):
    d = torch.zeros((4, 5), dtype=torch.uint8, device=cuda)
    with pytest.raises(pybicos.Exception, match="int16 or float32"):
        lbg.reproject(d, np.eye(4))
    with pytest.raises(ValueError):
        lbg.reproject(torch.zeros((4, 5), dtype=torch.int16, device=cuda), np.eye(4),
                      out=torch.zeros((4, 5, 4), dtype=torch.float32, device=cuda))
    q = np.eye(4)
    q[0, 0] = np.inf
    with pytest.raises(ValueError, match="finite"):
        lbg.reproject(torch.zeros((4, 5), dtype=torch.int16, device=cuda), q)


@pytest.mark.parametrize("two_folders", [True, False])
def test_cli_end_to_end(cuda, tmp_path, two_folders):
    sc = scenes.make_scene(48, 160, 12, seed=7, bits=8)
    if two_folders:
        a, b = tmp_path / "l", tmp_path / "r"
        a.mkdir()
        b.mkdir()
        for t in range(sc.left.shape[0]):
            imageio.write_png(str(a / f"{t}.png"), sc.left[t])
            imageio.write_png(str(b / f"{t}.png"), sc.right[t])
        folders = [str(a), str(b)]
    else:
        a = tmp_path / "lr"
        a.mkdir()
        for t in range(sc.left.shape[0]):
            imageio.write_png(str(a / f"{t}_left.png"), sc.left[t])
            imageio.write_png(str(a / f"{t}_right.png"), sc.right[t])
        folders = [str(a)]
    q = np.array([[1.0, 0.0, 0.0, -80.0], [0.0, 1.0, 0.0, -24.0], [0.0, 0.0, 0.0, 900.0], [0.0, 0.0, 0.05, 0.0]])
    qfile = tmp_path / "q.yml"
    qfile.write_text("%YAML:1.0\n---\nQ: !!opencv-matrix\n   rows: 4\n   cols: 4\n   dt: d\n   data: [ "
                     + ", ".join(repr(float(v)) for v in q.ravel()) + " ]\n")
    out = tmp_path / "o" / "disp.png"
    out.parent.mkdir()
    so, se = io.StringIO(), io.StringIO()
    args = folders + ["-t", "0.9", "-s", "0.1", "-v", "2", "--limited", "-n", "10", "--corrmap", "-q", str(qfile),
                      "-o", str(out)]
    assert cli.main(args, out=so, err=se) == 0
    assert "Loaded 20 8-bit images in total" in so.getvalue()

    cfg, _ = cli.config_from_args(cli.parse_args(args))
    d, corr = lbg.match_device(dev(sc.left[:10], cuda), dev(sc.right[:10], cuda), cfg)
    d, corr = host(d), host(corr)
    assert_same(imageio.read_image(str(out.with_suffix(".tiff"))), d, "disparity")
    assert_same(imageio.read_image(str(tmp_path / "o" / "disp-corrmap.tiff")), corr, "corrmap")
    assert np.array_equal(imageio.read_image(str(out)), cli.normalized_u8(d))
    pts = host(lbg.reproject(dev(d, cuda), q))
    want, _, _ = opc.xyz_lines(pts, d, False)
    assert len(want) > 1000
    with open(str(out.with_suffix(".xyz"))) as f:
        assert f.read().splitlines() == want
