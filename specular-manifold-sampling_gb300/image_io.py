"""Readers for the normal-map files of the reference's scenes.

The reference loads normal maps through its Bitmap class (src/librender/
normalmap.cpp:7-24): OpenEXR (linear RGB) or 8-bit PNG / JPEG (RGB, values
taken as stored), square and power-of-two.  This module reads

  * scanline OpenEXR files with NONE, RLE, ZIPS or ZIP compression and HALF,
    FLOAT or UINT channels (the compressions the paper's normal maps use;
    PIZ, PXR24, B44 and DWA raise ValueError), following the published
    OpenEXR file layout;
  * PNG files, 8 or 16 bits per channel, grey / RGB / grey-alpha / RGBA,
    non-interlaced, following the PNG specification's filters;

and converts RGB normals to the FP16 slope maps the library takes
(normalmap.cpp:45-58: n = normalize(2 rgb - 1), slope = (-n_x / n_z, -n_y / n_z)).
"""
from __future__ import annotations

import struct
import zlib
from pathlib import Path

import numpy as np

_EXR_MAGIC = 20000630
_EXR_LINES = {0: 1, 1: 1, 2: 1, 3: 16}          # NONE, RLE, ZIPS, ZIP
_EXR_NAMES = {0: "NONE", 1: "RLE", 2: "ZIPS", 3: "ZIP", 4: "PIZ", 5: "PXR24", 6: "B44", 7: "B44A",
              8: "DWAA", 9: "DWAB"}
_EXR_TYPES = {0: (4, np.dtype("<u4")), 1: (2, np.dtype("<f2")), 2: (4, np.dtype("<f4"))}


def _cstr(b: bytes, pos: int):
    end = b.index(b"\0", pos)
    return b[pos:end].decode("latin-1"), end + 1


def _exr_header(b: bytes):
    magic, version = struct.unpack_from("<ii", b, 0)
    if magic != _EXR_MAGIC:
        raise ValueError("not an OpenEXR file")
    if version & 0x200:
        raise ValueError("tiled OpenEXR files are not supported")
    if version & 0x1800:
        raise ValueError("deep or multi-part OpenEXR files are not supported")
    pos, attrs = 8, {}
    while True:
        name, pos = _cstr(b, pos)
        if not name:
            break
        typ, pos = _cstr(b, pos)
        (size,) = struct.unpack_from("<i", b, pos)
        pos += 4
        attrs[name] = (typ, b[pos:pos + size])
        pos += size
    chans, raw, p = [], attrs["channels"][1], 0
    while raw[p] != 0:
        cname, p = _cstr(raw, p)
        ptype, _plinear, xs, ys = struct.unpack_from("<iB3xii", raw, p)
        p += 16
        if xs != 1 or ys != 1:
            raise ValueError("sub-sampled OpenEXR channels are not supported")
        chans.append((cname, ptype))
    return attrs, chans, pos


def _undo_zip_layout(t: bytes) -> bytes:
    """Inverse of the ZIP / RLE pre-pass: byte-delta predictor, then the
    split of even and odd bytes into two halves."""
    d = np.frombuffer(t, np.uint8).astype(np.int64)
    if d.size:
        d[1:] -= 128
        d = (np.cumsum(d) & 0xFF).astype(np.uint8)
    n = d.size
    out = np.empty(n, np.uint8)
    half = (n + 1) // 2
    out[0::2] = d[:half]
    out[1::2] = d[half:]
    return out.tobytes()


def _rle_decode(b: bytes, n: int) -> bytes:
    out = bytearray()
    i = 0
    while i < len(b) and len(out) < n:
        c = struct.unpack_from("b", b, i)[0]
        i += 1
        if c < 0:
            out += b[i:i - c]
            i -= c
        else:
            out += bytes([b[i]]) * (c + 1)
            i += 1
    if len(out) != n:
        raise ValueError("corrupt RLE block in OpenEXR file")
    return bytes(out)


def read_exr(path) -> dict:
    """Channel name -> float32 array (height, width) of a scanline OpenEXR file."""
    b = Path(path).read_bytes()
    attrs, chans, pos = _exr_header(b)
    comp = attrs["compression"][1][0]
    if comp not in _EXR_LINES:
        raise ValueError(f"OpenEXR compression {_EXR_NAMES.get(comp, comp)} is not supported "
                         "(NONE, RLE, ZIPS and ZIP are)")
    x0, y0, x1, y1 = struct.unpack("<iiii", attrs["dataWindow"][1])
    w, h = x1 - x0 + 1, y1 - y0 + 1
    lines = _EXR_LINES[comp]
    nchunks = (h + lines - 1) // lines
    offsets = struct.unpack_from(f"<{nchunks}Q", b, pos)
    chans = sorted(chans)   # stored in alphabetical order
    sizes = [_EXR_TYPES[t][0] for _, t in chans]
    out = {c: np.zeros((h, w), np.float32) for c, _ in chans}
    for off in offsets:
        y, dsize = struct.unpack_from("<ii", b, off)
        data = b[off + 8:off + 8 + dsize]
        nl = min(lines, y1 - y + 1)
        raw_size = nl * w * sum(sizes)
        if dsize < raw_size:
            data = _undo_zip_layout(zlib.decompress(data) if comp in (2, 3) else _rle_decode(data, raw_size))
        elif comp != 0 and dsize > raw_size:
            raise ValueError("corrupt OpenEXR chunk")
        if len(data) != raw_size:
            raise ValueError("corrupt OpenEXR chunk")
        p = 0
        for r in range(nl):
            row = y - y0 + r
            for (c, t), sz in zip(chans, sizes):
                out[c][row] = np.frombuffer(data, _EXR_TYPES[t][1], w, p).astype(np.float32)
                p += w * sz
    return out


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def read_png(path) -> np.ndarray:
    """(height, width, channels) float32 in [0, 1] of a non-interlaced PNG
    (grey, grey-alpha, RGB or RGBA at 8 or 16 bits), values as stored."""
    b = Path(path).read_bytes()
    if b[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG file")
    pos, idat, hdr = 8, bytearray(), None
    while pos < len(b):
        (n,) = struct.unpack_from(">I", b, pos)
        typ = b[pos + 4:pos + 8]
        body = b[pos + 8:pos + 8 + n]
        pos += 12 + n
        if typ == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif typ == b"IDAT":
            idat += body
        elif typ == b"IEND":
            break
    if hdr is None:
        raise ValueError("PNG without IHDR")
    w, h, depth, ctype, _, _, interlace = hdr
    nch = {0: 1, 2: 3, 4: 2, 6: 4}.get(ctype)
    if nch is None or depth not in (8, 16) or interlace:
        raise ValueError("unsupported PNG layout (palette, <8-bit or interlaced)")
    bpp = nch * depth // 8
    stride = w * bpp
    raw = zlib.decompress(bytes(idat))
    img = np.zeros((h, stride), np.uint8)
    prev = np.zeros(stride, np.int64)
    for y in range(h):
        f = raw[y * (stride + 1)]
        line = np.frombuffer(raw, np.uint8, stride, y * (stride + 1) + 1).astype(np.int64)
        if f == 0:
            cur = line
        elif f == 2:
            cur = (line + prev) & 0xFF
        elif f in (1, 3, 4):
            cur = line.copy()
            for i in range(stride):
                a = cur[i - bpp] if i >= bpp else 0
                up = prev[i]
                if f == 1:
                    cur[i] = (cur[i] + a) & 0xFF
                elif f == 3:
                    cur[i] = (cur[i] + ((a + up) >> 1)) & 0xFF
                else:
                    c = prev[i - bpp] if i >= bpp else 0
                    cur[i] = (cur[i] + _paeth(a, up, c)) & 0xFF
        else:
            raise ValueError(f"bad PNG filter type {f}")
        img[y] = cur
        prev = cur
    if depth == 16:
        v = img.view(">u2").astype(np.float32) / 65535.0
    else:
        v = img.astype(np.float32) / 255.0
    return v.reshape(h, w, nch)


def read_rgb(path) -> np.ndarray:
    """(height, width, 3) float32 RGB of an OpenEXR or PNG file."""
    path = Path(path)
    ext = path.suffix.lower()
    if ext == ".exr":
        ch = read_exr(path)
        if not all(c in ch for c in "RGB"):
            raise ValueError("OpenEXR normal map without R, G, B channels")
        return np.stack([ch["R"], ch["G"], ch["B"]], axis=-1)
    if ext == ".png":
        v = read_png(path)
        if v.shape[2] in (1, 2):
            return np.repeat(v[..., :1], 3, axis=2)
        return v[..., :3]
    raise ValueError(f"normal map format '{ext}' is not supported (.exr, .png)")


def normalmap_slopes(path) -> np.ndarray:
    """(res, res, 2) float16 slopes of an RGB normal map file, as the
    reference derives level 0 of its LEAN map (normalmap.cpp:45-58)."""
    rgb = read_rgb(path).astype(np.float32)
    h, w = rgb.shape[:2]
    if h != w or (w & (w - 1)) != 0:
        raise ValueError("expected a square power-of-two normal map")
    n = 2.0 * rgb - 1.0
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    with np.errstate(divide="ignore", invalid="ignore"):
        s = np.stack([-n[..., 0] / n[..., 2], -n[..., 1] / n[..., 2]], axis=-1)
    if not np.isfinite(s).all():
        raise ValueError("normal map has normals in the tangent plane (n_z = 0)")
    return s.astype(np.float16)
