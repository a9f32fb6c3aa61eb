"""Host-side asset loaders (OBJ, PNG, EXR) on the CPU.  The PNG and EXR files
are written by small encoders in this file, which follow the published
formats independently of the decoders (forward filters, Adam7 pass split,
OpenEXR chunk layout with RLE / ZIP predictor)."""
import os
import struct
import zlib

import numpy as np
import pytest

from voidray_gb300 import assets as A
from voidray_gb300._native import VoidrayError
from voidray_gb300.scene import Mesh, Scene, ImageTexture, Environments, SampleType

# ------------------------------------------------------- OBJ restatement ---
def _obj_index(tok: str, count: int, what: str, line: int) -> int:
    try:
        i = int(tok)
    except ValueError:
        raise VoidrayError(1, f"OBJ line {line}: bad {what} index {tok!r}") from None
    j = count + i if i < 0 else i - 1
    if i == 0 or not 0 <= j < count:
        raise VoidrayError(1, f"OBJ line {line}: {what} index {i} out of range (have {count})")
    return j


def parse_obj_restated(text: str):
    """The obj-rs TexturedVertex rules written out line by line in Python (the
    library's parser is native); returns the same four arrays."""
    pos: list[tuple[float, float, float]] = []
    tex: list[tuple[float, float]] = []
    nrm: list[tuple[float, float, float]] = []
    cache: dict[tuple[int, int, int], int] = {}
    order: list[tuple[int, int, int]] = []
    indices: list[int] = []
    for ln, raw in enumerate(text.splitlines(), 1):
        line = raw.split("#", 1)[0].split()
        if not line:
            continue
        key, args = line[0], line[1:]
        try:
            if key == "v":
                if len(args) < 3:
                    raise VoidrayError(1, f"OBJ line {ln}: vertex needs 3 coordinates")
                pos.append((float(args[0]), float(args[1]), float(args[2])))
            elif key == "vt":
                if not args:
                    raise VoidrayError(1, f"OBJ line {ln}: texture coordinate needs u")
                tex.append((float(args[0]), float(args[1]) if len(args) > 1 else 0.0))
            elif key == "vn":
                if len(args) < 3:
                    raise VoidrayError(1, f"OBJ line {ln}: normal needs 3 components")
                nrm.append((float(args[0]), float(args[1]), float(args[2])))
            elif key == "f":
                if len(args) != 3:
                    raise VoidrayError(1, f"OBJ line {ln}: face with {len(args)} corners "
                                          "(the model must be triangulated)")
                for corner in args:
                    parts = corner.split("/")
                    if len(parts) != 3 or not parts[1] or not parts[2]:
                        raise VoidrayError(1, f"OBJ line {ln}: face corner {corner!r} lacks texture "
                                              "or normal indices")
                    k = (_obj_index(parts[0], len(pos), "position", ln),
                         _obj_index(parts[2], len(nrm), "normal", ln),
                         _obj_index(parts[1], len(tex), "texture", ln))
                    v = cache.get(k)
                    if v is None:
                        v = cache[k] = len(order)
                        order.append(k)
                    indices.append(v)
        except ValueError:
            raise VoidrayError(1, f"OBJ line {ln}: cannot parse {raw.strip()!r}") from None
    n = len(order)
    p = np.asarray(pos, np.float64).reshape(-1, 3)
    t = np.asarray(tex, np.float64).reshape(-1, 2)
    q = np.asarray(nrm, np.float64).reshape(-1, 3)
    ix = np.asarray(order, np.int64).reshape(-1, 3)
    positions = p[ix[:, 0]].astype(np.float32) if n else np.zeros((0, 3), np.float32)
    normals = q[ix[:, 1]].astype(np.float32) if n else np.zeros((0, 3), np.float32)
    uvs = t[ix[:, 2]].astype(np.float32) if n else np.zeros((0, 2), np.float32)
    return positions, uvs, normals, np.asarray(indices, np.uint32).reshape(-1, 3)


OBJ = """# comment line
mtllib x.mtl
o thing
v 0 0 0
v 1 0 0
v 0 1 0 1.0
v 1 1 0
vt 0 0
vt 1 0
vt 0.5
vt 1 1 0
vn 0 0 1
vn 0 0 -1
s 1
usemtl m
f 1/1/1 2/2/1 3/3/1
f 2/2/1 4/4/1 3/3/1   # shares two corners with the first face
f -3/-3/-1 -1/-1/-1 -2/-2/-2   # the last corner is (3, 3, 1) again
"""


def test_obj_numbering_follows_first_use_of_each_triple():
    pos, uv, nrm, idx = A.parse_obj(OBJ)
    assert idx.tolist() == [[0, 1, 2], [1, 3, 2], [4, 5, 2]]
    assert pos.tolist() == [[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0], [1, 0, 0], [1, 1, 0]]
    assert uv.tolist() == [[0, 0], [1, 0], [0.5, 0], [1, 1], [1, 0], [1, 1]]
    assert nrm.tolist() == [[0, 0, 1]] * 4 + [[0, 0, -1]] * 2
    assert pos.dtype == np.float32 and idx.dtype == np.uint32


@pytest.mark.parametrize("face, what", [
    ("f 1/1/1 2/1/1 3/1/1 1/1/1", "triangulated"),
    ("f 1 2 3", "lacks"),
    ("f 1//1 2//1 3//1", "lacks"),
    ("f 1/1/1 2/1/1 9/1/1", "out of range"),
    ("f 0/1/1 2/1/1 3/1/1", "out of range"),
])
def test_obj_rejects_what_texturedvertex_rejects(face, what):
    text = "v 0 0 0\nv 1 0 0\nv 0 1 0\nvt 0 0\nvn 0 0 1\n" + face + "\n"
    with pytest.raises(VoidrayError, match=what):
        A.parse_obj(text)


def test_mesh_from_file_and_scene(tmp_path):
    p = tmp_path / "m.obj"
    p.write_text(OBJ)
    m = Mesh.from_file(str(p))
    assert m.num_triangles == 3 and m.normals is not None and m.uvs is not None
    s = Scene()
    assert s.add_mesh_from_file(str(p)) == 0


# the reference checkout, when the environment names one (VOIDRAY_REFERENCE); otherwise these tests skip
REF_ROOT = os.environ.get("VOIDRAY_REFERENCE", "")
REF_ASSET = os.path.join(REF_ROOT, "assets", "mushroom.obj") if REF_ROOT else ""


@pytest.mark.skipif(not REF_ASSET or not os.path.exists(REF_ASSET), reason="VOIDRAY_REFERENCE unset or its assets absent")
def test_obj_reads_a_blender_export():
    """The reference's own demo mesh: every triangle corner carries the
    position, uv and normal of the OBJ lines it names."""
    with open(REF_ASSET) as f:
        text = f.read()
    pos, uv, nrm, idx = A.parse_obj(text)
    lines = text.splitlines()
    v = np.array([l.split()[1:4] for l in lines if l.startswith("v ")], np.float64).astype(np.float32)
    vt = np.array([l.split()[1:3] for l in lines if l.startswith("vt ")], np.float64).astype(np.float32)
    faces = [l.split()[1:] for l in lines if l.startswith("f ")]
    assert len(idx) == len(faces) == 4448
    for f, tri in zip(faces[::97], idx[::97]):
        for corner, k in zip(f, tri):
            pi, ti, _ = (int(x) - 1 for x in corner.split("/"))
            assert np.array_equal(pos[k], v[pi]) and np.array_equal(uv[k], vt[ti])
    assert len(np.unique(idx)) == len(pos)


# -------------------------------------------------------------------- PNG ---
def _png_chunk(kind: bytes, body: bytes) -> bytes:
    return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body))


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if pa <= pb and pa <= pc else (b if pb <= pc else c)


def _filter_rows(rows: np.ndarray, bpp: int) -> bytes:
    """Forward PNG filters, cycling through the five types row by row."""
    out = bytearray()
    prev = np.zeros(rows.shape[1], np.int64)
    for y, row in enumerate(rows.astype(np.int64)):
        ft = y % 5
        enc = []
        for i, x in enumerate(row):
            a = row[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            pred = [0, a, b, (a + b) >> 1, _paeth(a, b, c)][ft]
            enc.append((x - pred) & 0xFF)
        out.append(ft)
        out += bytes(enc)
        prev = row
    return bytes(out)


def _pack(samples: np.ndarray, depth: int) -> np.ndarray:
    """[h, w*ch] integer samples -> [h, stride] bytes."""
    h, n = samples.shape
    if depth == 8:
        return samples.astype(np.uint8)
    if depth == 16:
        s = samples.astype(np.uint16)
        return np.stack([s >> 8, s & 0xFF], -1).reshape(h, 2 * n).astype(np.uint8)
    bits = ((samples[..., None] >> np.arange(depth - 1, -1, -1)) & 1).reshape(h, n * depth).astype(np.uint8)
    return np.packbits(bits, axis=1)


def encode_png(samples: np.ndarray, depth: int, ctype: int, palette=None, interlace=False) -> bytes:
    h, w, ch = samples.shape
    bpp = max(1, ch * depth // 8)
    raw = b""
    passes = A._ADAM7 if interlace else [(0, 0, 1, 1)]
    for x0, y0, dx, dy in passes:
        sub = samples[y0::dy, x0::dx]
        if sub.size == 0:
            continue
        raw += _filter_rows(_pack(sub.reshape(sub.shape[0], -1), depth), bpp)
    out = A._PNG_MAGIC + _png_chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, int(interlace)))
    if palette is not None:
        out += _png_chunk(b"PLTE", palette.astype(np.uint8).tobytes())
    z = zlib.compress(raw)
    out += _png_chunk(b"IDAT", z[:len(z) // 2]) + _png_chunk(b"IDAT", z[len(z) // 2:])
    return out + _png_chunk(b"IEND", b"")


@pytest.mark.parametrize("depth, ctype, interlace", [
    (8, 2, False), (8, 6, False), (16, 2, False), (16, 6, True), (8, 0, True), (1, 0, False),
    (2, 0, False), (4, 0, True), (16, 0, False), (8, 4, False), (16, 4, True), (8, 3, False), (4, 3, True),
])
def test_png_decodes_like_to_rgb32f(depth, ctype, interlace):
    rng = np.random.default_rng(depth * 10 + ctype)
    h, w = 11, 13
    ch = A._PNG_CHANNELS[ctype]
    maxv = (1 << depth) - 1
    samples = rng.integers(0, maxv + 1, (h, w, ch))
    palette = rng.integers(0, 256, (1 << depth, 3)) if ctype == 3 else None
    img = A.decode_png(encode_png(samples, depth, ctype, palette, interlace))
    assert img.shape == (h, w, 3) and img.dtype == np.float32
    if ctype == 3:
        want = palette[samples[..., 0]].astype(np.float32) / np.float32(255)
    else:
        s = samples if depth >= 8 else samples * (255 // maxv)
        full = np.float32(65535 if depth == 16 else 255)
        col = s[..., :3] if ch >= 3 else np.repeat(s[..., :1], 3, -1)
        want = col.astype(np.float32) / full
    assert np.array_equal(img, want)


def test_png_rejects_corruption():
    data = bytearray(encode_png(np.zeros((2, 2, 3), int), 8, 2))
    data[20] ^= 1  # inside IHDR: CRC no longer matches
    with pytest.raises(VoidrayError, match="CRC"):
        A.decode_png(bytes(data))


# -------------------------------------------------------------------- EXR ---
def _exr_attr(name, typ, value: bytes) -> bytes:
    return name.encode() + b"\0" + typ.encode() + b"\0" + struct.pack("<i", len(value)) + value


def _rle(b: bytes) -> bytes:
    out, i = bytearray(), 0
    while i < len(b):
        j = i
        while j + 1 < len(b) and b[j + 1] == b[i] and j - i < 126:
            j += 1
        if j > i:  # run of j-i+1 equal bytes
            out += struct.pack("b", j - i) + b[i:i + 1]
            i = j + 1
        else:
            k = i
            while k < len(b) and k - i < 127 and not (k + 1 < len(b) and b[k + 1] == b[k]):
                k += 1
            k = max(k, i + 1)
            out += struct.pack("b", -(k - i)) + b[i:k]
            i = k
    return bytes(out)


def _predict(raw: bytes) -> bytes:
    d = np.frombuffer(raw, np.uint8)
    t = np.concatenate([d[0::2], d[1::2]]).astype(np.int64)
    p = t.copy()
    p[1:] = (t[1:] - t[:-1] + 128) & 0xFF
    return p.astype(np.uint8).tobytes()


def encode_exr(planes: dict, types: dict, comp: int, y_origin: int = 5) -> bytes:
    names = sorted(planes)
    h, w = planes[names[0]].shape
    dts = {0: "<u4", 1: "<f2", 2: "<f4"}
    ch = b"".join(n.encode() + b"\0" + struct.pack("<iB3xii", types[n], 0, 1, 1) for n in names) + b"\0"
    box = struct.pack("<iiii", 2, y_origin, 2 + w - 1, y_origin + h - 1)
    hdr = (_exr_attr("channels", "chlist", ch) + _exr_attr("compression", "compression", bytes([comp]))
           + _exr_attr("dataWindow", "box2i", box) + _exr_attr("displayWindow", "box2i", box)
           + _exr_attr("lineOrder", "lineOrder", b"\0") + _exr_attr("pixelAspectRatio", "float", struct.pack("<f", 1))
           + b"\0")
    lines = A._EXR_LINES[comp]
    chunks = []
    for y0 in range(0, h, lines):
        raw = b"".join(planes[n][y].astype(dts[types[n]]).tobytes()
                       for y in range(y0, min(h, y0 + lines)) for n in names)
        if comp == 1:
            data = _rle(_predict(raw))
        elif comp in (2, 3):
            data = zlib.compress(_predict(raw))
        else:
            data = raw
        if len(data) >= len(raw):
            data = raw
        chunks.append(struct.pack("<ii", y_origin + y0, len(data)) + data)
    head = struct.pack("<ii", A._EXR_MAGIC, 2) + hdr
    table_end = len(head) + 8 * len(chunks)
    offs, o = [], table_end
    for c in chunks:
        offs.append(o)
        o += len(c)
    return head + struct.pack(f"<{len(chunks)}Q", *offs) + b"".join(chunks)


@pytest.mark.parametrize("comp", [0, 1, 2, 3])
@pytest.mark.parametrize("ptype", [1, 2])
def test_exr_scanline_round_trip(comp, ptype):
    rng = np.random.default_rng(comp * 7 + ptype)
    h, w = 37, 21
    planes = {}
    for c in "RGBA":
        x = rng.gamma(0.7, 3.0, (h, w)).astype(np.float32)
        x[:4] = 1.5  # flat rows: runs for RLE and chunks that compress
        planes[c] = x.astype(np.float16).astype(np.float32) if ptype == 1 else x
    types = {c: ptype for c in planes}
    types["A"] = 1
    img = A.decode_exr(encode_exr(planes, types, comp))
    want = np.stack([planes["R"], planes["G"], planes["B"]], -1)
    assert img.shape == (h, w, 3) and np.array_equal(img, want)


def test_exr_rejects_unsupported():
    p = {c: np.zeros((4, 4), np.float32) for c in "RGB"}
    data = bytearray(encode_exr(p, {c: 2 for c in p}, 0))
    i = data.index(b"compression\0compression\0") + len(b"compression\0compression\0") + 4
    data[i] = 4  # PIZ
    with pytest.raises(VoidrayError, match="not supported"):
        A.decode_exr(bytes(data))
    with pytest.raises(VoidrayError, match="needs R, G and B"):
        A.decode_exr(encode_exr({"Y": np.zeros((2, 2), np.float32)}, {"Y": 2}, 0))


def test_files_reach_textures_and_environments(tmp_path):
    rgb = np.random.default_rng(3).integers(0, 256, (5, 6, 3))
    (tmp_path / "t.png").write_bytes(encode_png(rgb, 8, 2))
    (tmp_path / "e.exr").write_bytes(encode_exr({c: np.full((3, 4), i + 1.0, np.float32) for i, c in enumerate("RGB")},
                                                {c: 2 for c in "RGB"}, 3))
    (tmp_path / "x.gif").write_bytes(b"GIF89a\x01\x00\x01\x00")
    t = ImageTexture.from_file(str(tmp_path / "t.png"), SampleType.Nearest)
    assert np.array_equal(t.image, rgb.astype(np.float32) / np.float32(255))
    s = Scene()
    assert s.add_image_texture(str(tmp_path / "t.png")) == 0
    env = Environments.hdri(str(tmp_path / "e.exr"))
    assert env.image.shape == (3, 4, 3) and env.image[0, 0].tolist() == [1.0, 2.0, 3.0]
    with pytest.raises(VoidrayError, match="not decoded here"):
        A.load_image_rgb32f(str(tmp_path / "x.gif"))


REF_PNGS = [os.path.join(REF_ROOT, "assets", f) if REF_ROOT else "" for f in ("test.png", "uv_test.png")]


@pytest.mark.skipif(not all(p and os.path.exists(p) for p in REF_PNGS), reason="VOIDRAY_REFERENCE unset or its assets absent")
def test_png_reads_the_reference_assets():
    """The reference's own PNGs (written by another encoder, RGBA 8-bit): every
    chunk CRC and the zlib checksum verify, the size is the header's, and the
    values lie on the u8 / 255 grid to_rgb32f produces."""
    shapes = []
    for p in REF_PNGS:
        img = A.load_image_rgb32f(p)
        shapes.append(img.shape)
        q = img * np.float32(255)
        assert np.all(np.abs(q - np.round(q)) < 1e-4) and img.min() >= 0 and img.max() <= 1
    assert shapes == [(2, 2, 3), (256, 256, 3)]


def _fix_png_crcs(b: bytes) -> bytes:
    """Recomputes every chunk CRC so that a mutation reaches the decoder's logic."""
    b = bytearray(b)
    pos = 8
    while pos + 8 <= len(b):
        (length,) = struct.unpack(">I", b[pos:pos + 4])
        if pos + 12 + length > len(b):
            break
        b[pos + 8 + length:pos + 12 + length] = struct.pack(">I", zlib.crc32(bytes(b[pos + 4:pos + 8 + length])))
        pos += 12 + length
    return bytes(b)


def test_corrupt_files_raise_voidray_errors_only():
    """Mutated PNG / EXR / OBJ inputs either decode or raise VoidrayError with
    VR_ERR_INVALID or VR_ERR_UNSUPPORTED: no zlib, struct, index or memory
    errors escape, and no header asks for an unbounded allocation."""
    rng = np.random.default_rng(9)
    pngs = [encode_png(rng.integers(0, 256, (7, 9, 3)), 8, 2),
            encode_png(rng.integers(0, 4, (5, 11, 1)), 2, 0, interlace=True),
            encode_png(rng.integers(0, 65536, (6, 6, 4)), 16, 6),
            encode_png(rng.integers(0, 16, (8, 8, 1)), 4, 3, palette=rng.integers(0, 256, (16, 3)))]
    exrs = [encode_exr({c: rng.normal(0, 1, (6, 5)).astype(np.float32) for c in "RGB"}, {c: 2 for c in "RGB"}, comp)
            for comp in (0, 1, 2, 3)]
    obj = b"v 0 0 0\nv 1 0 0\nv 0 1 0\nvt 0 0\nvt 1 0\nvt 0 1\nvn 0 0 1\nf 1/1/1 2/2/1 3/3/1\nf -1/-1/-1 -2/-2/-1 -3/-3/-1\n"
    cases = [(pngs, lambda b: A.decode_png(_fix_png_crcs(b)), 8, None),
             (exrs, A.decode_exr, 8, None),
             ([obj], lambda b: A.parse_obj(b.decode("latin-1")), 0, list(b"0123456789-/ \nvftn.e"))]
    for seeds, decode, start, alphabet in cases:
        for it in range(1200):
            b = bytearray(seeds[it % len(seeds)])
            for _ in range(rng.integers(1, 5)):
                b[int(rng.integers(start, len(b)))] = int(rng.choice(alphabet) if alphabet else rng.integers(0, 256))
            try:
                decode(bytes(b))
            except VoidrayError as e:
                assert e.status in (1, 2)


def _random_obj(rng, n_faces, bad=False):
    """OBJ text with comments, ignored statements, w components, 1- and
    3-component vt, negative indices, CRLF / CR line ends and shared corners."""
    lines = ["# generated", "mtllib a.mtl", "o part"]
    counts = [0, 0, 0]  # v, vt, vn
    for _ in range(rng.integers(3, 9)):
        lines.append("v " + " ".join(f"{x:.6g}" for x in rng.normal(0, 3, rng.integers(3, 5))))
        counts[0] += 1
    for _ in range(rng.integers(1, 6)):
        lines.append("vt " + " ".join(f"{x:.5f}" for x in rng.random(rng.integers(1, 4))))
        counts[1] += 1
    for _ in range(rng.integers(1, 5)):
        lines.append("vn " + " ".join(f"{x:.4e}" for x in rng.normal(0, 1, 3)))
        counts[2] += 1
    for f in range(n_faces):
        if rng.random() < 0.15:
            kind = rng.integers(0, 3)
            lines.append(["v", "vt", "vn"][kind] + " " + " ".join(f"{x:.3f}" for x in rng.random(3)))
            counts[kind] += 1
        corners = []
        for _ in range(3):
            ix = []
            for c in (0, 1, 2):
                k = int(rng.integers(1, counts[c] + 1))
                ix.append(str(k - counts[c] - 1) if rng.random() < 0.3 else str(k))
            corners.append("/".join(ix))
        line = "f " + " ".join(corners)
        if rng.random() < 0.1:
            line += "  # trailing comment"
        if rng.random() < 0.05:
            lines.append("s off")
        lines.append(line)
    if bad:
        j = int(rng.integers(3, len(lines)))
        lines[j] = rng.choice(["f 1/1/1 2/1/1", "f 1//1 2//1 3//1", "v 1 2", "vt", "vn 1 x 2",
                               f"f 1/1/1 2/1/1 {counts[0] + 7}/1/1", "f 0/1/1 1/1/1 1/1/1", "f a/1/1 1/1/1 1/1/1",
                               "v 1.5 2..5 3"])
    sep = rng.choice(["\n", "\r\n", "\r"])
    return sep.join(lines) + sep


def test_native_obj_parser_matches_the_restatement():
    """The native parser against the Python restatement of the obj-rs rules on
    random OBJ texts: identical arrays, and the same error message for the
    same first bad line."""
    rng = np.random.default_rng(21)
    for it in range(400):
        bad = it % 4 == 3
        text = _random_obj(rng, int(rng.integers(0, 40)), bad)
        try:
            want = parse_obj_restated(text)
        except VoidrayError as e:
            with pytest.raises(VoidrayError) as got:
                A.parse_obj(text)
            assert got.value.status == 1 and str(got.value) == str(e), (str(got.value), str(e))
            continue
        got = A.parse_obj(text)
        for a, b in zip(got, want):
            assert a.dtype == b.dtype and np.array_equal(a, b)


@pytest.mark.skipif(not REF_ASSET or not os.path.exists(REF_ASSET), reason="VOIDRAY_REFERENCE unset or its assets absent")
def test_native_obj_parser_on_the_reference_meshes():
    folder = os.path.dirname(REF_ASSET)
    for name in ("mushroom.obj", "mossy_ground.obj", "material_testing_stand.obj"):
        path = os.path.join(folder, name)
        if not os.path.exists(path):
            continue
        with open(path, "r", encoding="utf-8", errors="replace") as f:
            want = parse_obj_restated(f.read())
        got = A.load_obj(path)
        for a, b in zip(got, want):
            assert np.array_equal(a, b)


def test_obj_errors_quoting_undecodable_bytes():
    """An error message that quotes bytes of the input which are not UTF-8
    still reaches Python as a VoidrayError."""
    with pytest.raises(VoidrayError, match="cannot parse"):
        A.parse_obj(b"v 0 0 \xff\xfe\n")
    with pytest.raises(VoidrayError, match="bad position index"):
        A.parse_obj("v 0 0 0\nvt 0 0\nvn 0 0 1\nf \ud800/1/1 1/1/1 1/1/1\n")


def _paeth_restated(a: int, b: int, c: int) -> int:
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def png_unfilter_restated(data: bytes, pos: int, rows: int, stride: int, bpp: int):
    """The five PNG scanline filters undone byte by byte in Python (the
    library does it natively); returns (uint8 [rows, stride], new pos)."""
    out = np.zeros((rows, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    for y in range(rows):
        ftype = data[pos]
        line = np.frombuffer(data, np.uint8, stride, pos + 1).astype(np.int32)
        pos += 1 + stride
        if ftype == 0:
            cur = line
        elif ftype == 2:
            cur = (line + prev) & 0xFF
        elif ftype == 1:  # Sub: a running sum per byte lane of the pixel
            cur = line.copy()
            for k in range(min(bpp, stride)):
                cur[k::bpp] = np.cumsum(line[k::bpp]) & 0xFF
        elif ftype in (3, 4):  # Average and Paeth depend on the byte just decoded
            lst = line.tolist()
            up = prev.tolist()
            for i in range(stride):
                a = lst[i - bpp] if i >= bpp else 0
                if ftype == 3:
                    lst[i] = (lst[i] + ((a + up[i]) >> 1)) & 0xFF
                else:
                    lst[i] = (lst[i] + _paeth_restated(a, up[i], up[i - bpp] if i >= bpp else 0)) & 0xFF
            cur = np.asarray(lst, np.int32)
        else:
            raise VoidrayError(1, f"PNG: unknown filter type {ftype}")
        out[y] = cur
        prev = cur
    return out, pos


@pytest.mark.parametrize("rows,stride,bpp", [(1, 1, 1), (7, 13, 3), (16, 64, 4), (5, 96, 8), (33, 7, 1), (4, 24, 6)])
def test_png_unfilter_matches_the_restatement(rows, stride, bpp):
    """vr_png_unfilter against the byte-by-byte Python restatement on random
    scanlines with every filter type (and a random mix per row)."""
    rng = np.random.default_rng(rows * stride + bpp)
    for types in ([0], [1], [2], [3], [4], [0, 1, 2, 3, 4]):
        body = rng.integers(0, 256, (rows, stride + 1), dtype=np.uint8)
        body[:, 0] = rng.choice(types, rows)
        data = b"xyz" + body.tobytes()
        got, gpos = A._png_unfilter(data, 3, rows, stride, bpp)
        want, wpos = png_unfilter_restated(data, 3, rows, stride, bpp)
        assert gpos == wpos and np.array_equal(got, want)
    bad = bytearray(data)
    bad[3 + (stride + 1) * (rows - 1)] = 5
    with pytest.raises(VoidrayError, match="unknown filter type 5"):
        A._png_unfilter(bytes(bad), 3, rows, stride, bpp)
    with pytest.raises(VoidrayError, match="shorter"):
        A._png_unfilter(data[:-1], 3, rows, stride, bpp)
