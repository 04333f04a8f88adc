"""The command-line front end's host parts, on CPU: PNG/TIFF/.npy readers
and writers (every PNG filter and bit depth, both TIFF byte orders),
cv::FileStorage matrices, the input naming conventions of libBICOS's
src/fileutils.cpp, the option -> Config mapping of src/cli.cpp and the
.xyz writer against the oracle's restatement of save_pointcloud."""
import math
import os
import struct
import zlib

import numpy as np
import pytest

from libbicos_gb300 import cli, imageio, pointcloud, pybicos
from oracle import pointcloud as opc


# ---- a test-side PNG encoder using every filter (spec section 9) --------

def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if pa <= pb and pa <= pc else (b if pb <= pc else c)


def _filter_row(ftype, cur, prev, bpp):
    out = bytearray()
    for i, x in enumerate(cur):
        a = cur[i - bpp] if i >= bpp else 0
        b = prev[i]
        c = prev[i - bpp] if i >= bpp else 0
        pred = [0, a, b, (a + b) // 2, _paeth(a, b, c)][ftype]
        out.append((x - pred) & 0xFF)
    return bytes([ftype]) + bytes(out)


def _png(path, raw_rows, width, depth, ctype, plte=None):
    bpp = max(1, ({0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype] * depth) // 8)
    stride = len(raw_rows[0])
    body, prev = b"", bytes(stride)
    for y, row in enumerate(raw_rows):
        body += _filter_row(y % 5, row, prev, bpp)
        prev = row

    def chunk(kind, data):
        return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF)

    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", width, len(raw_rows), depth, ctype, 0, 0, 0))
    if plte is not None:
        png += chunk(b"PLTE", plte.astype(np.uint8).tobytes())
    png += chunk(b"IDAT", zlib.compress(body)) + chunk(b"IEND", b"")
    with open(path, "wb") as f:
        f.write(png)


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16])
def test_png_every_filter_grey(tmp_path, dtype):
    rng = np.random.default_rng(1)
    img = rng.integers(0, np.iinfo(dtype).max + 1, size=(11, 13), dtype=dtype)
    rows = [r.astype(">u2").tobytes() if dtype == np.uint16 else r.tobytes() for r in img]
    p = str(tmp_path / "a.png")
    _png(p, rows, 13, 16 if dtype == np.uint16 else 8, 0)
    got = imageio.read_png(p)
    assert got.dtype == dtype and np.array_equal(got, img)


def test_png_colour_palette_and_low_depths(tmp_path):
    rng = np.random.default_rng(2)
    rgb = rng.integers(0, 256, size=(7, 9, 3), dtype=np.uint8)
    p = str(tmp_path / "rgb.png")
    _png(p, [r.tobytes() for r in rgb], 9, 8, 2)
    want = np.rint(rgb[..., 0] * 0.299 + rgb[..., 1] * 0.587 + rgb[..., 2] * 0.114).astype(np.uint8)
    assert np.array_equal(imageio.read_png(p), want)
    rgba = np.concatenate([rgb, np.full((7, 9, 1), 200, np.uint8)], axis=2)
    _png(p, [r.tobytes() for r in rgba], 9, 8, 6)
    assert np.array_equal(imageio.read_png(p), want)
    pal = rng.integers(0, 256, size=(16, 3), dtype=np.uint8)
    idx = rng.integers(0, 16, size=(5, 10), dtype=np.uint8)
    packed = [bytes((r[2 * i] << 4) | r[2 * i + 1] for i in range(5)) for r in idx]
    _png(p, packed, 10, 4, 3, plte=pal)
    pw = pal[idx]
    assert np.array_equal(imageio.read_png(p),
                          np.rint(pw[..., 0] * 0.299 + pw[..., 1] * 0.587 + pw[..., 2] * 0.114).astype(np.uint8))
    g1 = rng.integers(0, 2, size=(4, 12), dtype=np.uint8)
    _png(p, [np.packbits(r).tobytes() for r in g1], 12, 1, 0)
    assert np.array_equal(imageio.read_png(p), g1 * 255)


def test_png_rejects_bad_filter_and_interlace(tmp_path):
    p = str(tmp_path / "bad.png")

    def chunk(kind, data):
        return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF)

    with open(p, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", 2, 1, 8, 0, 0, 0, 0)) +
                chunk(b"IDAT", zlib.compress(b"\x07\x01\x02")) + chunk(b"IEND", b""))
    with pytest.raises(ValueError, match="unknown filter"):
        imageio.read_png(p)
    with open(p, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", 2, 1, 8, 0, 0, 0, 1)) +
                chunk(b"IEND", b""))
    with pytest.raises(ValueError, match="interlaced"):
        imageio.read_png(p)


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16, np.int16, np.float32, np.float64])
def test_tiff_and_png_round_trips(tmp_path, dtype):
    rng = np.random.default_rng(3)
    if np.issubdtype(dtype, np.floating):
        img = rng.normal(size=(6, 9)).astype(dtype)
        img[0, 0] = np.nan
    else:
        info = np.iinfo(dtype)
        img = rng.integers(info.min, info.max + 1, size=(6, 9)).astype(dtype)
    p = str(tmp_path / "x.tiff")
    imageio.write_tiff(p, img)
    got = imageio.read_image(p)
    assert got.dtype == dtype and np.array_equal(got, img, equal_nan=True)
    if dtype in (np.uint8, np.uint16):
        imageio.write_png(str(tmp_path / "x.png"), img)
        assert np.array_equal(imageio.read_image(str(tmp_path / "x.png")), img)


def test_tiff_big_endian(tmp_path):
    img = np.arange(12, dtype=np.uint16).reshape(3, 4) * 1000
    pixels = img.astype(">u2").tobytes()
    entries = [(256, 3, 1, 4), (257, 3, 1, 3), (258, 3, 1, 16), (259, 3, 1, 1), (262, 3, 1, 1),
               (273, 4, 1, 8), (277, 3, 1, 1), (278, 3, 1, 3), (279, 4, 1, len(pixels))]
    out = b"MM" + struct.pack(">HI", 42, 8 + len(pixels)) + pixels + struct.pack(">H", len(entries))
    for tag, typ, n, val in entries:
        out += struct.pack(">HHI", tag, typ, n) + (struct.pack(">HH", val, 0) if typ == 3 else struct.pack(">I", val))
    out += struct.pack(">I", 0)
    p = str(tmp_path / "be.tif")
    with open(p, "wb") as f:
        f.write(out)
    assert np.array_equal(imageio.read_image(p), img)


def test_npy_input(tmp_path):
    a = np.arange(20, dtype=np.uint16).reshape(4, 5)
    np.save(str(tmp_path / "3.npy"), a)
    assert np.array_equal(imageio.read_image(str(tmp_path / "3.npy")), a)


Q = np.array([[1.0, 0.0, 0.0, -320.5], [0.0, 1.0, 0.0, -240.25], [0.0, 0.0, 0.0, 812.5],
              [0.0, 0.0, 0.125, -0.0]])


def test_filestorage_formats(tmp_path):
    vals = ", ".join(repr(float(v)) for v in Q.ravel())
    yml = ("%YAML:1.0\n---\nQ: !!opencv-matrix\n   rows: 4\n   cols: 4\n   dt: d\n   data: [ "
           + vals.replace(", -240.25", ",\n       -240.25") + " ]\nR: !!opencv-matrix\n   rows: 1\n   cols: 1\n"
           "   dt: d\n   data: [ 7. ]\n")
    xml = ('<?xml version="1.0"?>\n<opencv_storage>\n<Q type_id="opencv-matrix">\n  <rows>4</rows>\n'
           "  <cols>4</cols>\n  <dt>d</dt>\n  <data>\n    " + vals.replace(",", " ") + "</data></Q>\n</opencv_storage>\n")
    js = '{"Q": {"type_id": "opencv-matrix", "rows": 4, "cols": 4, "dt": "d", "data": [' + vals + "]}}"
    for name, text in (("q.yml", yml), ("q.xml", xml), ("q.json", js)):
        p = str(tmp_path / name)
        with open(p, "w") as f:
            f.write(text)
        assert np.array_equal(imageio.read_matrix(p), Q), name
    with open(str(tmp_path / "q.yml")) as f:
        assert "R:" in f.read()
    assert imageio.read_matrix(str(tmp_path / "q.yml"), "R")[0, 0] == 7.0


def test_read_sequence_naming(tmp_path):
    a, b = tmp_path / "a", tmp_path / "b"
    a.mkdir()
    b.mkdir()
    for i in (10, 2, 0):
        imageio.write_png(str(a / f"{i}.png"), np.full((2, 3), i, np.uint8))
        imageio.write_png(str(b / f"{i}.png"), np.full((2, 3), 100 + i, np.uint8))
    left, right = imageio.read_sequence(str(a), str(b))
    assert [int(m[0, 0]) for m in left] == [0, 2, 10] and [int(m[0, 0]) for m in right] == [100, 102, 110]
    one = tmp_path / "one"
    one.mkdir()
    for i in (1, 0):
        imageio.write_png(str(one / f"{i}_left.png"), np.full((2, 2), i, np.uint8))
        imageio.write_png(str(one / f"{i}_right.png"), np.full((2, 2), 50 + i, np.uint8))
    left, right = imageio.read_sequence(str(one))
    assert [int(m[0, 0]) for m in left] == [0, 1] and [int(m[0, 0]) for m in right] == [50, 51]
    imageio.write_png(str(one / "x_left.png"), np.zeros((2, 2), np.uint8))
    with pytest.raises(ValueError, match="NN_"):
        imageio.read_sequence(str(one))
    os.remove(str(one / "x_left.png"))
    imageio.write_png(str(one / "7_left.png"), np.zeros((2, 2), np.uint8))
    with pytest.raises(ValueError, match="Unequal number of images"):
        imageio.read_sequence(str(one))


def test_cli_options_to_config():
    c, need = cli.config_from_args(cli.parse_args(["in"]))
    assert (c.nxcorr_threshold, c.min_variance, c.subpixel_step) == (pytest.approx(0.75), None, None)
    assert c.mode == pybicos.Full and c.precision == pybicos.Single and not need
    assert isinstance(c.variant, type(pybicos.Variant.NoDuplicates()))
    c, need = cli.config_from_args(cli.parse_args(["in", "-t", "0", "--corrmap"]))
    assert need and c.nxcorr_threshold == -1.0
    c, _ = cli.config_from_args(cli.parse_args(["in", "-t", "0"]))
    assert c.nxcorr_threshold is None
    c, _ = cli.config_from_args(cli.parse_args(["in", "b", "-v", "2", "-s", "0.25", "--limited", "--double",
                                                "-m", "3", "--no-dupes"]))
    assert c.min_variance == 2.0 and c.subpixel_step == 0.25 and c.mode == pybicos.Limited
    assert c.precision == pybicos.Double
    assert (c.variant.max_lr_diff, c.variant.no_dupes) == (3, True)
    c, _ = cli.config_from_args(cli.parse_args(["in", "-v", "0"]))
    assert c.min_variance is None


def test_normalized_png_values():
    d = np.array([[-32768, 10, 20], [30, -32768, 10]], np.int16)
    assert cli.normalized_u8(d).tolist() == [[0, 0, 128], [255, 0, 0]]
    f = np.array([[np.nan, 1.5], [2.5, 2.0]], np.float32)
    assert cli.normalized_u8(f).tolist() == [[0, 0], [255, 128]]


@pytest.mark.parametrize("dtype", [np.int16, np.float32])
def test_pointcloud_writer_matches_oracle(tmp_path, dtype):
    rng = np.random.default_rng(4)
    pts = rng.normal(scale=[1.0, 1.0, 3.0], size=(9, 11, 3)).astype(np.float32)
    pts[0, 1, 0] = np.inf
    pts[2, 3, 2] = np.nan
    pts[4, 4] = (1e-7, -2.5e9, 123456789.0)
    if dtype == np.int16:
        disp = rng.integers(-5, 60, size=(9, 11)).astype(np.int16)
        disp[rng.random((9, 11)) < 0.2] = -32768
    else:
        disp = rng.normal(size=(9, 11)).astype(np.float32)
        disp[rng.random((9, 11)) < 0.2] = np.nan
    for allow in (False, True):
        p = str(tmp_path / f"p{allow}.xyz")
        counts = pointcloud.save_pointcloud(pts, disp, allow, p)
        want, nonfinite, negative = opc.xyz_lines(pts, disp, allow)
        with open(p) as f:
            assert f.read().splitlines() == want
        assert counts == {"written": len(want), "nonfinite": nonfinite, "negative_z": negative}
    assert opc.xyz_lines(pts, disp, False)[2] > 0


def test_reproject_oracle_conventions():
    d = np.array([[0, 8], [-16, 4]], np.int16)
    pts = opc.reproject(d, Q)
    assert np.array_equal(pts[0, 0], [0.0, 0.0, 0.0])  # W = 0
    w = 0.125 * 8
    assert np.allclose(pts[0, 1], [(1 - 320.5) / w, (0 - 240.25) / w, 812.5 / w])
    f = np.array([[np.nan, 2.0]], np.float32)
    assert np.isnan(opc.reproject(f, Q)[0, 0]).all()
    assert math.isclose(float(opc.reproject(f, Q)[0, 1, 2]), 812.5 / 0.25, rel_tol=1e-7)


def test_cli_rejects_missing_qmatrix_before_any_gpu_work(tmp_path):
    import io
    with pytest.raises(ValueError, match="does not exist"):
        cli.main([str(tmp_path), "-q", str(tmp_path / "missing.yml")], out=io.StringIO(), err=io.StringIO())


def test_image_round_trips_random_shapes(tmp_path):
    rng = np.random.default_rng(11)
    for k in range(25):
        h, w = int(rng.integers(1, 40)), int(rng.integers(1, 70))
        dtype = [np.uint8, np.uint16, np.int16, np.float32, np.float64][k % 5]
        if np.issubdtype(dtype, np.floating):
            img = rng.normal(scale=100.0, size=(h, w)).astype(dtype)
        else:
            info = np.iinfo(dtype)
            img = rng.integers(info.min, info.max + 1, size=(h, w)).astype(dtype)
        p = str(tmp_path / f"r{k}.tiff")
        imageio.write_tiff(p, img)
        assert np.array_equal(imageio.read_image(p), img), (k, h, w, dtype)
        if dtype in (np.uint8, np.uint16):
            q = str(tmp_path / f"r{k}.png")
            imageio.write_png(q, img)
            assert np.array_equal(imageio.read_image(q), img), (k, h, w, dtype)
