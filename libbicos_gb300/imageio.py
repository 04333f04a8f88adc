"""Image files for the command-line front end, without OpenCV.

libBICOS's CLI reads and writes images through OpenCV (cv::imread with
IMREAD_GRAYSCALE | IMREAD_ANYDEPTH, cv::imwrite; src/fileutils.cpp:28-153)
and reads the reprojection matrix with cv::FileStorage.  OpenCV is not
available on these hosts, so this module implements what that path needs
from the file-format specifications:

* PNG (ISO/IEC 15948): greyscale, RGB, palette, grey+alpha and RGBA, 1-16
  bit, all five row filters; Adam7-interlaced files are rejected.  Colour
  images become grey with the BT.601 luma weights (0.299, 0.587, 0.114),
  rounded; OpenCV's own integer conversion can differ by 1 DN.
* TIFF 6.0 baseline, uncompressed: 8/16-bit unsigned, int16, float32 and
  float64 single-channel images (and 8/16-bit RGB, converted to grey),
  either byte order, strips.
* .npy arrays (numpy's own format), for stacks produced by other tools.
* cv::FileStorage matrices in YAML, XML or JSON (the !!opencv-matrix /
  type_id="opencv-matrix" layout: rows, cols, dt, data).
"""
from __future__ import annotations

import json
import os
import re
import struct
import zlib

import numpy as np

_PNG_SIG = b"\x89PNG\r\n\x1a\n"


# ---- PNG ---------------------------------------------------------------

def _unfilter(raw: bytes, height: int, stride: int, bpp: int) -> np.ndarray:
    """Undo the per-row filters (spec section 9) with the library's
    sequential byte loop (bicos_png_unfilter)."""
    import ctypes as C

    from . import _native as N

    if len(raw) < height * (stride + 1):
        raise ValueError("PNG: truncated image data")
    out = np.empty((height, stride), dtype=np.uint8)
    src = np.frombuffer(raw, dtype=np.uint8)
    r = N.load().bicos_png_unfilter(C.c_void_p(out.ctypes.data), C.c_void_p(src.ctypes.data), height, stride, bpp)
    if r != 0:
        raise ValueError(f"PNG: unknown filter type in row {r - 1}" if r > 0 else "PNG: bad scanline layout")
    return out


def _to_grey(rgb: np.ndarray) -> np.ndarray:
    """BT.601 luma of an (..., 3) integer image, rounded, in its dtype."""
    y = rgb[..., 0] * 0.299 + rgb[..., 1] * 0.587 + rgb[..., 2] * 0.114
    return np.rint(y).astype(rgb.dtype)


def read_png(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        data = f.read()
    if data[:8] != _PNG_SIG:
        raise ValueError(f"{path}: not a PNG file")
    pos, idat, plte = 8, [], None
    width = height = depth = ctype = None
    while pos < len(data):
        length, kind = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + length]
        pos += 12 + length
        if kind == b"IHDR":
            width, height, depth, ctype, comp, filt, interlace = struct.unpack(">IIBBBBB", body)
            if comp != 0 or filt != 0:
                raise ValueError(f"{path}: unsupported PNG compression or filter method")
            if interlace != 0:
                raise ValueError(f"{path}: interlaced PNG files are not supported")
        elif kind == b"PLTE":
            plte = np.frombuffer(body, dtype=np.uint8).reshape(-1, 3)
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
    if width is None:
        raise ValueError(f"{path}: PNG without IHDR")
    channels = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    bits_pp = channels * depth
    stride = (width * bits_pp + 7) // 8
    bpp = max(1, bits_pp // 8)
    rows = _unfilter(zlib.decompress(b"".join(idat)), height, stride, bpp)
    if depth == 16:
        px = rows.view(">u2").astype(np.uint16).reshape(height, width, channels)
    elif depth == 8:
        px = rows.reshape(height, width, channels)
    else:  # 1, 2, 4 bits: unpack MSB first
        bits = np.unpackbits(rows, axis=1)[:, :width * depth].reshape(height, width, depth)
        weights = (1 << np.arange(depth - 1, -1, -1)).astype(np.uint8)
        px = (bits * weights).sum(axis=2).astype(np.uint8)[..., None]
        if ctype == 0:  # greyscale scales to 8 bits: v * 255 / (2^depth - 1)
            px = (px.astype(np.uint32) * 255 // ((1 << depth) - 1)).astype(np.uint8)
    if ctype == 3:
        if plte is None:
            raise ValueError(f"{path}: palette PNG without PLTE")
        return _to_grey(plte[px[..., 0]].astype(np.uint8))
    if ctype in (0, 4):
        return np.ascontiguousarray(px[..., 0])
    return _to_grey(px[..., :3])


def _png_chunk(kind: bytes, body: bytes) -> bytes:
    return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)


def write_png(path: str, img: np.ndarray) -> None:
    """Greyscale (H, W) or RGB (H, W, 3) uint8/uint16 image, filter 0."""
    img = np.asarray(img)
    if img.dtype not in (np.uint8, np.uint16) or img.ndim not in (2, 3):
        raise ValueError("write_png: uint8/uint16 greyscale or RGB images only")
    h, w = img.shape[:2]
    ctype = 0 if img.ndim == 2 else 2
    depth = 8 if img.dtype == np.uint8 else 16
    rows = img.astype(">u2") if depth == 16 else img
    raw = rows.reshape(h, -1).view(np.uint8)
    body = b"".join(b"\x00" + raw[y].tobytes() for y in range(h))
    with open(path, "wb") as f:
        f.write(_PNG_SIG)
        f.write(_png_chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 0)))
        f.write(_png_chunk(b"IDAT", zlib.compress(body, 6)))
        f.write(_png_chunk(b"IEND", b""))


# ---- TIFF --------------------------------------------------------------

_TIFF_TYPES = {1: "B", 2: "c", 3: "H", 4: "I", 5: "II", 6: "b", 8: "h", 9: "i", 11: "f", 12: "d", 16: "Q"}


def read_tiff(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        data = f.read()
    order = {b"II": "<", b"MM": ">"}.get(data[:2])
    if order is None or struct.unpack(order + "H", data[2:4])[0] != 42:
        raise ValueError(f"{path}: not a TIFF file")
    ifd = struct.unpack(order + "I", data[4:8])[0]
    count = struct.unpack(order + "H", data[ifd:ifd + 2])[0]
    tags = {}
    for i in range(count):
        e = ifd + 2 + 12 * i
        tag, typ, n = struct.unpack(order + "HHI", data[e:e + 8])
        fmt = _TIFF_TYPES.get(typ)
        if fmt is None:
            continue
        size = struct.calcsize(order + fmt) * n
        off = e + 8 if size <= 4 else struct.unpack(order + "I", data[e + 8:e + 12])[0]
        vals = struct.unpack(order + fmt * n, data[off:off + size])
        tags[tag] = vals
    width, height = tags[256][0], tags[257][0]
    bits = tags.get(258, (1,))
    spp = tags.get(277, (1,))[0]
    if tags.get(259, (1,))[0] != 1:
        raise ValueError(f"{path}: compressed TIFF files are not supported")
    if tags.get(284, (1,))[0] != 1 and spp > 1:
        raise ValueError(f"{path}: planar TIFF files are not supported")
    fmt_code = tags.get(339, (1,))[0]
    b = bits[0]
    kind = {1: "u", 2: "i", 3: "f"}[fmt_code]
    dtype = np.dtype(order + kind + str(b // 8))
    buf = b"".join(data[o:o + n] for o, n in zip(tags[273], tags[279]))
    px = np.frombuffer(buf, dtype=dtype, count=width * height * spp).reshape(height, width, spp)
    px = px.astype(dtype.newbyteorder("="))
    if spp >= 3:
        return _to_grey(px[..., :3])
    return np.ascontiguousarray(px[..., 0])


def write_tiff(path: str, img: np.ndarray) -> None:
    """Single-channel uint8/uint16/int16/float32/float64 image, one
    uncompressed strip, little-endian."""
    img = np.ascontiguousarray(img)
    kinds = {np.dtype(np.uint8): 1, np.dtype(np.uint16): 1, np.dtype(np.int16): 2, np.dtype(np.float32): 3,
             np.dtype(np.float64): 3}
    if img.ndim != 2 or img.dtype not in kinds:
        raise ValueError("write_tiff: single-channel uint8/uint16/int16/float32/float64 images only")
    h, w = img.shape
    pixels = img.astype(img.dtype.newbyteorder("<")).tobytes()
    entries = [(256, 4, 1, w), (257, 4, 1, h), (258, 3, 1, img.dtype.itemsize * 8), (259, 3, 1, 1),
               (262, 3, 1, 1), (273, 4, 1, 8), (277, 3, 1, 1), (278, 4, 1, h), (279, 4, 1, len(pixels)),
               (284, 3, 1, 1), (339, 3, 1, kinds[img.dtype])]
    ifd_off = 8 + len(pixels) + (len(pixels) & 1)
    out = bytearray(b"II" + struct.pack("<HI", 42, ifd_off))
    out += pixels
    if len(pixels) & 1:
        out += b"\x00"
    out += struct.pack("<H", len(entries))
    for tag, typ, n, val in entries:
        out += struct.pack("<HHI", tag, typ, n)
        out += struct.pack("<HH", val, 0) if typ == 3 else struct.pack("<I", val)
    out += struct.pack("<I", 0)
    with open(path, "wb") as f:
        f.write(bytes(out))


# ---- any image ----------------------------------------------------------

def read_image(path: str) -> np.ndarray:
    """2-D greyscale array (uint8 / uint16 as stored) of a PNG, TIFF or .npy file."""
    ext = os.path.splitext(path)[1].lower()
    if ext == ".npy":
        a = np.load(path)
        return _to_grey(a[..., :3]) if a.ndim == 3 else a
    with open(path, "rb") as f:
        head = f.read(8)
    if head == _PNG_SIG:
        return read_png(path)
    if head[:2] in (b"II", b"MM"):
        return read_tiff(path)
    raise ValueError(f"{path}: unsupported image format (PNG, TIFF and .npy are read)")


def _index(name: str):
    m = re.match(r"\d+", name)
    return int(m.group(0)) if m else None


def read_sequence(folder0: str, folder1: str | None = None):
    """The CLI's input stacks (src/fileutils.cpp:85-133): with two folders,
    numbered files N.ext in each; with one, N_left.ext and N_right.ext.
    Returns (left, right) lists of 2-D arrays sorted by N."""
    def one_dir(d):
        seq = []
        for name in os.listdir(d):
            idx = _index(name)
            if idx is None:
                raise ValueError("Expecting numbered files with names NN.png; e.g 0.png, 1.png...")
            seq.append((idx, read_image(os.path.join(d, name))))
        return seq

    if folder1 is not None:
        lseq, rseq = one_dir(folder0), one_dir(folder1)
    else:
        lseq, rseq = [], []
        msg = "Expecting numbered files with names NN_{left,right}.png; e.g.: 5_left.png, 10_right.png..."
        for name in os.listdir(folder0):
            idx = _index(name)
            if "_" not in name or idx is None:
                raise ValueError(msg)
            (lseq if "_left" in name else rseq).append((idx, read_image(os.path.join(folder0, name))))
    if len(lseq) != len(rseq):
        raise ValueError(f"Unequal number of images; left: {len(lseq)}, right: {len(rseq)}")
    lseq.sort(key=lambda e: e[0])
    rseq.sort(key=lambda e: e[0])
    return [m for _, m in lseq], [m for _, m in rseq]


# ---- cv::FileStorage matrices ---------------------------------------------

def _matrix(rows, cols, data, name) -> np.ndarray:
    a = np.asarray(data, dtype=np.float64)
    if a.size != rows * cols:
        raise ValueError(f"matrix {name}: {a.size} values for {rows}x{cols}")
    return a.reshape(rows, cols)


def read_matrix(path: str, name: str = "Q") -> np.ndarray:
    """Matrix `name` of a cv::FileStorage file (YAML, XML or JSON)."""
    text = open(path).read()
    stripped = text.lstrip()
    if stripped.startswith("<"):
        m = re.search(r"<%s\b[^>]*>(.*?)</%s>" % (name, name), text, re.S)
        if not m:
            raise ValueError(f"{path}: no matrix {name}")
        body = m.group(1)
        get = lambda tag: re.search(r"<%s>(.*?)</%s>" % (tag, tag), body, re.S).group(1)
        return _matrix(int(get("rows")), int(get("cols")), get("data").split(), name)
    if stripped.startswith("{"):
        node = json.loads(text)[name]
        return _matrix(int(node["rows"]), int(node["cols"]), node["data"], name)
    m = re.search(r"^%s\s*:\s*(?:!!opencv-matrix)?\s*$(.*?)(?=^\S|\Z)" % re.escape(name), text, re.S | re.M)
    if not m:
        raise ValueError(f"{path}: no matrix {name}")
    body = m.group(1)
    rows = int(re.search(r"rows\s*:\s*(\d+)", body).group(1))
    cols = int(re.search(r"cols\s*:\s*(\d+)", body).group(1))
    data = re.search(r"data\s*:\s*\[(.*?)\]", body, re.S).group(1)
    return _matrix(rows, cols, [v for v in re.split(r"[,\s]+", data) if v], name)
