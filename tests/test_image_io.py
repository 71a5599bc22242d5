"""Normal-map file readers (OpenEXR scanline NONE / RLE / ZIPS / ZIP, PNG) and
the normalmap BSDF of the scene XML loader.  Files are written here by small
writers that follow the published OpenEXR and PNG layouts, then read back."""
import importlib
import struct
import zlib

import numpy as np
import pytest


@pytest.fixture(scope="module")
def io(sms):
    return importlib.import_module(sms.__name__ + ".image_io")


def _exr_prepass(raw: bytes) -> bytes:
    """Even/odd byte split followed by the byte-delta predictor."""
    b = np.frombuffer(raw, np.uint8)
    t = np.concatenate([b[0::2], b[1::2]]).astype(np.int64)
    p = t.copy()
    p[1:] = (t[1:] - t[:-1] + 128) & 0xFF
    return p.astype(np.uint8).tobytes()


def _rle(b: bytes) -> bytes:
    out, i = bytearray(), 0
    while i < len(b):
        j = i
        while j + 1 < len(b) and b[j + 1] == b[i] and j - i < 126:
            j += 1
        if j - i >= 2:
            out += struct.pack("b", j - i) + b[i:i + 1]
            i = j + 1
        else:
            k = i
            while k < len(b) and k - i < 127 and not (k + 2 < len(b) and b[k] == b[k + 1] == b[k + 2]):
                k += 1
            k = max(k, i + 1)
            out += struct.pack("b", -(k - i)) + b[i:k]
            i = k
    return bytes(out)


def _write_exr(path, chans, comp, origin=(0, 0)):
    """chans: name -> (float32 array (h, w), pixel type 0 uint / 1 half / 2 float);
    origin: the data window's first pixel (x, y)."""
    names = sorted(chans)
    h, w = chans[names[0]][0].shape
    x0, y0 = origin
    hdr = bytearray(struct.pack("<ii", 20000630, 2))

    def attr(name, typ, data):
        hdr.extend(name.encode() + b"\0" + typ.encode() + b"\0" + struct.pack("<i", len(data)) + data)

    attr("channels", "chlist",
         b"".join(n.encode() + b"\0" + struct.pack("<iB3xii", chans[n][1], 0, 1, 1) for n in names) + b"\0")
    attr("compression", "compression", bytes([comp]))
    attr("dataWindow", "box2i", struct.pack("<iiii", x0, y0, x0 + w - 1, y0 + h - 1))
    attr("displayWindow", "box2i", struct.pack("<iiii", 0, 0, w - 1, h - 1))
    attr("lineOrder", "lineOrder", b"\0")
    attr("pixelAspectRatio", "float", struct.pack("<f", 1.0))
    attr("screenWindowCenter", "v2f", struct.pack("<ff", 0.0, 0.0))
    attr("screenWindowWidth", "float", struct.pack("<f", 1.0))
    hdr.extend(b"\0")
    dt = {0: "<u4", 1: "<f2", 2: "<f4"}
    lines = {0: 1, 1: 1, 2: 1, 3: 16}[comp]
    chunks = []
    for y in range(0, h, lines):
        raw = b"".join(chans[n][0][r].astype(dt[chans[n][1]]).tobytes()
                       for r in range(y, min(h, y + lines)) for n in names)
        data = raw
        if comp:
            pre = _exr_prepass(raw)
            enc = _rle(pre) if comp == 1 else zlib.compress(pre)
            if len(enc) < len(raw):
                data = enc
        chunks.append(struct.pack("<ii", y0 + y, len(data)) + data)
    pos = len(hdr) + 8 * len(chunks)
    offs = []
    for c in chunks:
        offs.append(pos)
        pos += len(c)
    path.write_bytes(bytes(hdr) + struct.pack(f"<{len(offs)}Q", *offs) + b"".join(chunks))


@pytest.mark.parametrize("comp", [0, 1, 2, 3])
@pytest.mark.parametrize("ptype", [1, 2])
def test_exr_round_trip(io, tmp_path, comp, ptype):
    rng = np.random.default_rng(comp + 4 * ptype)
    h, w = 37, 20                        # a partial last ZIP block
    R = rng.random((h, w)).astype(np.float32)
    G = np.round(rng.random((h, w)) * 4) / 4           # runs for RLE
    B = np.full((h, w), 0.75, np.float32)
    f = tmp_path / "t.exr"
    _write_exr(f, {"R": (R, ptype), "G": (G.astype(np.float32), ptype), "B": (B, ptype)}, comp)
    ch = io.read_exr(f)
    cast = (lambda a: a.astype(np.float16).astype(np.float32)) if ptype == 1 else (lambda a: a)
    for name, a in (("R", R), ("G", G), ("B", B)):
        assert np.array_equal(ch[name], cast(a.astype(np.float32))), name


def test_exr_refuses_other_compressions(io, tmp_path):
    f = tmp_path / "t.exr"
    _write_exr(f, {"R": (np.zeros((4, 4), np.float32), 2)}, 0)
    b = bytearray(f.read_bytes())
    i = b.index(b"compression\0compression\0") + len("compression\0compression\0") + 4
    b[i] = 4   # PIZ
    f.write_bytes(bytes(b))
    with pytest.raises(ValueError, match="PIZ"):
        io.read_exr(f)


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)


def _write_png(path, img, depth=8):
    """img: (h, w, 3) uint8 / uint16; rows use filter types 0..4 in turn."""
    h, w, nch = img.shape
    raw = img.astype(">u2").tobytes() if depth == 16 else img.astype(np.uint8).tobytes()
    stride = len(raw) // h
    bpp = nch * depth // 8
    out = bytearray()
    prev = bytes(stride)
    for y in range(h):
        line = raw[y * stride:(y + 1) * stride]
        f = y % 5
        enc = bytearray(stride)
        for i in range(stride):
            a = line[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            pred = (0, a, b, (a + b) >> 1, _paeth(a, b, c))[f]
            enc[i] = (line[i] - pred) & 0xFF
        out += bytes([f]) + enc
        prev = line

    def chunk(t, d):
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xFFFFFFFF)

    ihdr = struct.pack(">IIBBBBB", w, h, depth, 2, 0, 0, 0)
    path.write_bytes(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", ihdr) + chunk(b"IDAT", zlib.compress(bytes(out)))
                     + chunk(b"IEND", b""))


@pytest.mark.parametrize("depth", [8, 16])
def test_png_round_trip(io, tmp_path, depth):
    rng = np.random.default_rng(depth)
    hi = 255 if depth == 8 else 65535
    img = rng.integers(0, hi + 1, size=(11, 9, 3))
    f = tmp_path / "t.png"
    _write_png(f, img, depth)
    v = io.read_png(f)
    assert np.array_equal(np.round(v * hi).astype(np.int64), img)


def _normals_rgb(res):
    t = (np.arange(res) + 0.5) / res
    vv, uu = np.meshgrid(t, t, indexing="ij")
    n = np.stack([0.3 * np.sin(6 * uu), 0.2 * np.cos(5 * vv), np.ones_like(uu)], axis=-1)
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    return n, (0.5 * n + 0.5).astype(np.float32)


def test_normalmap_slopes_follow_the_reference(io, tmp_path):
    """slope = (-n_x / n_z, -n_y / n_z) of n = normalize(2 rgb - 1)
    (normalmap.cpp:45-58); the first scanline is the row v = 0."""
    n, rgb = _normals_rgb(16)
    f = tmp_path / "n.exr"
    _write_exr(f, {"R": (rgb[..., 0], 2), "G": (rgb[..., 1], 2), "B": (rgb[..., 2], 2)}, 3)
    s = io.normalmap_slopes(f).astype(np.float32)
    ref = np.stack([-n[..., 0] / n[..., 2], -n[..., 1] / n[..., 2]], axis=-1)
    assert s.shape == (16, 16, 2)
    assert np.allclose(s, ref, atol=2e-3)
    _write_exr(f, {"R": (rgb[:8, :16, 0], 2), "G": (rgb[:8, :16, 1], 2), "B": (rgb[:8, :16, 2], 2)}, 0)
    with pytest.raises(ValueError, match="square"):
        io.normalmap_slopes(f)


NM_XML = """<scene version="2.0.0">
  <integrator type="path_sms_ss"><boolean name="twostage" value="true"/></integrator>
  <bsdf type="normalmap" id="bumpy">
    <string name="filename" value="textures/n.exr"/>
    <float name="tiles" value="3"/>
    <bsdf type="dielectric"><float name="int_ior" value="1.5"/><float name="ext_ior" value="1.0"/></bsdf>
  </bsdf>
  <shape type="rectangle">
    <ref id="bumpy"/>
    <boolean name="caustic_caster_single" value="true"/>
  </shape>
  <emitter type="point">
    <point name="position" x="0" y="0" z="4"/>
    <spectrum name="intensity" value="10"/>
    <boolean name="caustic_emitter_single" value="true"/>
  </emitter>
</scene>"""


def test_scene_xml_normalmap_bsdf(sms, io, oracle, tmp_path):
    """<bsdf type="normalmap"> (referenced by id) on a caster: the nested
    dielectric, the slope map and its tiling reach the scene description, and
    the library and the oracle accept the scene with the twostage config."""
    (tmp_path / "textures").mkdir()
    n, rgb = _normals_rgb(32)
    _write_exr(tmp_path / "textures" / "n.exr",
               {"R": (rgb[..., 0], 1), "G": (rgb[..., 1], 1), "B": (rgb[..., 2], 1)}, 3)
    (tmp_path / "s.xml").write_text(NM_XML)
    desc, cfg, itype = sms.load_scene(tmp_path / "s.xml")
    assert itype == "path_sms_ss" and cfg.twostage
    sid, slopes, tiles = desc.normalmap
    assert sid == 0 and tiles == 3.0 and slopes.shape == (32, 32, 2) and slopes.dtype == np.float16
    b = desc.meshes[0][4]
    assert b.type == sms.BSDF_DIELECTRIC and abs(b.eta - 1.5) < 1e-6
    oracle.OracleScene(desc)
    sms.Scene(desc)
    (tmp_path / "two.xml").write_text(NM_XML.replace("</scene>", """<shape type="rectangle"><ref id="bumpy"/>
      </shape></scene>"""))
    with pytest.raises(ValueError, match="one normal map"):
        sms.load_scene(tmp_path / "two.xml")


def test_scene_xml_normalmap_lean_fallback(sms, io, oracle, tmp_path):
    """lean_fallback, lean_fallback_alpha and the fallback's eta / k of a
    normalmap BSDF (normalmap.cpp:46-55) reach the scene description; a named
    lean_fallback_material is refused."""
    (tmp_path / "textures").mkdir()
    n, rgb = _normals_rgb(32)
    _write_exr(tmp_path / "textures" / "n.exr",
               {"R": (rgb[..., 0], 1), "G": (rgb[..., 1], 1), "B": (rgb[..., 2], 1)}, 3)
    xml = NM_XML.replace('<float name="tiles" value="3"/>', '''<float name="tiles" value="3"/>
    <boolean name="lean_fallback" value="true"/>
    <float name="lean_fallback_alpha" value="0.02"/>
    <float name="eta" value="0.2"/><float name="k" value="3"/>''')
    (tmp_path / "s.xml").write_text(xml)
    desc, _, _ = sms.load_scene(tmp_path / "s.xml")
    assert desc.lean_fallback == (0.02, 0.2, 3.0)
    oracle.OracleScene(desc)
    sms.Scene(desc)
    (tmp_path / "m.xml").write_text(NM_XML.replace('<float name="tiles" value="3"/>', '''<float name="tiles" value="3"/>
    <boolean name="lean_fallback" value="true"/><string name="lean_fallback_material" value="Au"/>'''))
    with pytest.raises(ValueError, match="lean_fallback_material"):
        sms.load_scene(tmp_path / "m.xml")
    (tmp_path / "d.xml").write_text(NM_XML)
    assert sms.load_scene(tmp_path / "d.xml")[0].lean_fallback is None


def test_exr_data_window_and_uint(io, tmp_path):
    """A data window that does not start at the origin (chunks addressed by
    their absolute first scanline) and UINT channels."""
    rng = np.random.default_rng(3)
    A = rng.random((21, 7)).astype(np.float32)
    U = rng.integers(0, 1 << 20, size=(21, 7)).astype(np.float32)
    f = tmp_path / "w.exr"
    _write_exr(f, {"A": (A, 2), "U": (U, 0)}, 3, origin=(5, -4))
    ch = io.read_exr(f)
    assert np.array_equal(ch["A"], A) and np.array_equal(ch["U"], U)
