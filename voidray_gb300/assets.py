"""Host-side asset loaders: the file formats voidray reads before a scene
reaches the renderer.

- `load_obj` follows `Mesh::from_file` (voidray_renderer/src/core/mesh.rs:46-74),
  which calls `obj::load_obj::<TexturedVertex, u32>` of the obj-rs crate
  (version 0.7.0 in the reference's Cargo.lock; not vendored).  The crate's
  published behaviour for that vertex type is restated here: `v x y z [w]`,
  `vt u [v [w]]` (missing components 0), `vn x y z`; face corners `p/t/n`
  with 1-based indices, negative indices counting back from the current end
  of their list; every face must be a triangle with all three of position,
  texture and normal indices, else the load fails (the crate's
  `UntriangulatedModel` / `InsufficientData` errors); each distinct
  (position, normal, texture) index triple becomes one vertex, numbered in
  order of first use; other statements (`o`, `g`, `s`, `usemtl`, `mtllib`,
  `l`, `p`) do not change the mesh.  Numbers are parsed as f64 and rounded
  to f32, which equals a direct decimal-to-f32 conversion for the short
  decimals OBJ writers emit.  The parsing runs in the native library
  (`vr_obj_parse`, one pass, hundreds of MB/s).
- `load_image_rgb32f` follows `image::open(path).to_rgb32f()` as
  `ImageTexture::new` (voidray_renderer/src/core/texture.rs:36-50) and
  `HDRIEnvironment::new` (voidray_common/src/environments.rs:42-55) call it
  (image 0.24): row 0 at the top, RGB f32, alpha dropped, grey replicated,
  integer samples divided by their maximum (255 or 65535).  Formats read
  here: PNG (every colour type and bit depth, Adam7 interlacing); OpenEXR
  scanline files with NONE, RLE, ZIPS or ZIP compression and HALF, FLOAT or
  UINT channels; JPEG (baseline, extended and progressive Huffman DCT, 8-bit;
  decoded by the native library, `include/voidray_assets.h`); TIFF (the first
  image of the file: strips or tiles, chunky or planar, no / LZW / Deflate /
  PackBits compression, horizontal and floating-point predictors, grey,
  palette and RGB(A), 1-32-bit integer and 16/32/64-bit float samples).
  JPEG-in-TIFF, CMYK and YCbCr TIFF and the other EXR compressions are not
  restated; decode those elsewhere and pass float RGB arrays
  (`Scene.add_texture`, `Environments.hdri`).
"""
from __future__ import annotations

import ctypes
import functools
import os
import struct
import zlib

import numpy as np

from ._native import VoidrayError


def _corrupt_is_invalid(fmt: str):
    """Decoders read untrusted bytes: whatever a corrupt file makes the parsing
    raise (short buffers, bad zlib streams, out-of-range indices, undecodable
    names) is reported as VR_ERR_INVALID, like the native decoder's errors."""
    def wrap(fn):
        @functools.wraps(fn)
        def inner(*args, **kwargs):
            try:
                return fn(*args, **kwargs)
            except VoidrayError:
                raise
            except (zlib.error, struct.error, IndexError, KeyError, ValueError, TypeError, OverflowError) as e:
                raise VoidrayError(1, f"{fmt}: corrupt data ({type(e).__name__}: {e})") from None
        return inner
    return wrap


# -------------------------------------------------------------------- OBJ ---
def parse_obj(text):
    """Returns (positions f32 [V,3], uvs f32 [V,2], normals f32 [V,3],
    indices u32 [F,3]) with the obj-rs TexturedVertex numbering, parsed by the
    native library (vr_obj_parse, include/voidray_assets.h)."""
    from . import _native as N

    data = text.encode("utf-8", "surrogatepass") if isinstance(text, str) else bytes(text)
    mesh = N.vr_obj_mesh()
    N.check(N.lib().vr_obj_parse(data, len(data), ctypes.byref(mesh)))
    try:
        nv, nt = mesh.num_vertices, mesh.num_triangles

        def take(ptr, count, dtype, width):
            if count == 0:
                return np.zeros((0, width), dtype)
            return np.ctypeslib.as_array(ptr, shape=(count * width,)).copy().reshape(count, width)

        return (take(mesh.positions, nv, np.float32, 3), take(mesh.uvs, nv, np.float32, 2),
                take(mesh.normals, nv, np.float32, 3), take(mesh.indices, nt, np.uint32, 3))
    finally:
        N.lib().vr_obj_free(ctypes.byref(mesh))


def load_obj(path: str):
    with open(path, "rb") as f:
        return parse_obj(f.read())


# -------------------------------------------------------------------- PNG ---
# decoders refuse images above this many pixels (the native JPEG decoder's limit too)
MAX_IMAGE_PIXELS = 1 << 28

_PNG_MAGIC = b"\x89PNG\r\n\x1a\n"
_ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]
_PNG_CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}


def _png_unfilter(data: bytes, pos: int, rows: int, stride: int, bpp: int):
    """Undoes the five PNG scanline filters (native vr_png_unfilter); returns
    (uint8 [rows, stride], new pos)."""
    from . import _native as N

    need = rows * (stride + 1)
    src = np.frombuffer(data, np.uint8, min(need, max(0, len(data) - pos)), pos)
    out = np.empty((rows, stride), np.uint8)
    N.check(N.lib().vr_png_unfilter(src.ctypes.data, src.size, rows, stride, bpp, out.ctypes.data))
    return out, pos + need


def _png_samples(rows: np.ndarray, width: int, depth: int, channels: int) -> np.ndarray:
    """Unpacks filtered-out scanlines into integer samples [h, w, channels]."""
    h = rows.shape[0]
    if depth == 8:
        return rows[:, :width * channels].reshape(h, width, channels).astype(np.uint16)
    if depth == 16:
        s = rows[:, :width * channels * 2].reshape(h, width * channels, 2).astype(np.uint16)
        return ((s[..., 0] << 8) | s[..., 1]).reshape(h, width, channels)
    bits = np.unpackbits(rows, axis=1)[:, :width * channels * depth].reshape(h, width * channels, depth)
    weights = (1 << np.arange(depth - 1, -1, -1)).astype(np.uint16)
    return (bits.astype(np.uint16) * weights).sum(-1).astype(np.uint16).reshape(h, width, channels)


@_corrupt_is_invalid("PNG")
def decode_png(data: bytes) -> np.ndarray:
    if data[:8] != _PNG_MAGIC:
        raise VoidrayError(1, "PNG: bad signature")
    pos, ihdr, idat, plte, trns = 8, None, [], None, None
    while pos + 8 <= len(data):
        length, ctype = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + length]
        if len(body) != length:
            raise VoidrayError(1, "PNG: truncated chunk")
        if zlib.crc32(ctype + body) != struct.unpack(">I", data[pos + 8 + length:pos + 12 + length])[0]:
            raise VoidrayError(1, f"PNG: CRC mismatch in {ctype!r}")
        pos += 12 + length
        if ctype == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body)
        elif ctype == b"PLTE":
            plte = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif ctype == b"tRNS":
            trns = body
        elif ctype == b"IDAT":
            idat.append(body)
        elif ctype == b"IEND":
            break
    if ihdr is None:
        raise VoidrayError(1, "PNG: no IHDR")
    width, height, depth, ctype, comp, filt, interlace = ihdr
    if ctype not in _PNG_CHANNELS or comp != 0 or filt != 0 or interlace not in (0, 1):
        raise VoidrayError(1, f"PNG: unsupported header {ihdr}")
    if ctype == 3 and plte is None:
        raise VoidrayError(1, "PNG: palette image without PLTE")
    if width == 0 or height == 0:
        raise VoidrayError(1, "PNG: zero width or height")
    if width * height > MAX_IMAGE_PIXELS:
        raise VoidrayError(2, f"PNG: {width}x{height} is above {MAX_IMAGE_PIXELS} pixels")
    ch = _PNG_CHANNELS[ctype]
    raw = zlib.decompress(b"".join(idat))
    bpp = max(1, ch * depth // 8)
    img = np.zeros((height, width, ch), np.uint16)
    passes = _ADAM7 if interlace else [(0, 0, 1, 1)]
    p = 0
    for x0, y0, dx, dy in passes:
        pw = (width - x0 + dx - 1) // dx if width > x0 else 0
        ph = (height - y0 + dy - 1) // dy if height > y0 else 0
        if pw == 0 or ph == 0:
            continue
        stride = (pw * ch * depth + 7) // 8
        rows, p = _png_unfilter(raw, p, ph, stride, bpp)
        img[y0::dy, x0::dx] = _png_samples(rows, pw, depth, ch)
    if ctype == 3:
        return plte[img[..., 0]].astype(np.float32) / np.float32(255.0)
    maxv = 65535 if depth == 16 else 255
    if depth < 8:
        img = img * (255 // ((1 << depth) - 1))  # low bit depths expand to 8 bits
    f = img.astype(np.float32) / np.float32(maxv)
    if ch in (1, 2):
        return np.repeat(f[..., :1], 3, axis=-1)
    return np.ascontiguousarray(f[..., :3])


# -------------------------------------------------------------------- EXR ---
_EXR_MAGIC = 20000630
_EXR_LINES = {0: 1, 1: 1, 2: 1, 3: 16}  # compression -> scanlines per chunk (NONE, RLE, ZIPS, ZIP)
_EXR_TYPES = {0: (np.dtype("<u4"), 4), 1: (np.dtype("<f2"), 2), 2: (np.dtype("<f4"), 4)}


def _exr_header(data: bytes):
    magic, version = struct.unpack("<ii", data[:8])
    if magic != _EXR_MAGIC:
        raise VoidrayError(1, "EXR: bad magic number")
    if version & 0x200 or version & 0x800 or version & 0x1000:
        raise VoidrayError(2, "EXR: tiled, deep or multi-part files are not supported")
    pos, attrs = 8, {}
    while data[pos] != 0:
        end = data.index(b"\0", pos)
        name = data[pos:end].decode()
        tend = data.index(b"\0", end + 1)
        typ = data[end + 1:tend].decode()
        size = struct.unpack("<i", data[tend + 1:tend + 5])[0]
        attrs[name] = (typ, data[tend + 5:tend + 5 + size])
        pos = tend + 5 + size
    return attrs, pos + 1


def _exr_channels(value: bytes):
    chans, pos = [], 0
    while value[pos] != 0:
        end = value.index(b"\0", pos)
        name = value[pos:end].decode()
        ptype, _linear, xs, ys = struct.unpack("<iB3xii", value[end + 1:end + 17])
        if ptype not in _EXR_TYPES or xs != 1 or ys != 1:
            raise VoidrayError(2, f"EXR: channel {name!r} type {ptype} sampling {xs}x{ys} not supported")
        chans.append((name, ptype))
        pos = end + 17
    return chans


def _exr_rle_decode(src: bytes, size: int) -> bytes:
    out, i = bytearray(), 0
    while i < len(src) and len(out) < size:
        n = struct.unpack("b", src[i:i + 1])[0]
        i += 1
        if n < 0:
            out += src[i:i - n]
            i -= n
        else:
            out += src[i:i + 1] * (n + 1)
            i += 1
    if len(out) != size:
        raise VoidrayError(1, "EXR: RLE chunk has the wrong size")
    return bytes(out)


def _exr_unpredict(t: bytes) -> bytes:
    """The ZIP/RLE post-pass: undo the byte delta, then re-interleave the two
    halves (even bytes were stored first, odd bytes second)."""
    d = np.frombuffer(t, np.uint8).astype(np.int64)
    if d.size:
        d[1:] -= 128
        d = np.cumsum(d) & 0xFF
    d = d.astype(np.uint8)
    out = np.empty_like(d)
    half = (d.size + 1) // 2
    out[0::2] = d[:half]
    out[1::2] = d[half:]
    return out.tobytes()


@_corrupt_is_invalid("EXR")
def decode_exr(data: bytes) -> np.ndarray:
    attrs, pos = _exr_header(data)
    for req in ("channels", "compression", "dataWindow"):
        if req not in attrs:
            raise VoidrayError(1, f"EXR: header lacks {req!r}")
    chans = _exr_channels(attrs["channels"][1])
    comp = attrs["compression"][1][0]
    if comp not in _EXR_LINES:
        raise VoidrayError(2, f"EXR: compression {comp} not supported (NONE, RLE, ZIPS, ZIP are)")
    xmin, ymin, xmax, ymax = struct.unpack("<iiii", attrs["dataWindow"][1])
    w, h = xmax - xmin + 1, ymax - ymin + 1
    if w <= 0 or h <= 0:
        raise VoidrayError(1, "EXR: empty data window")
    if w * h > MAX_IMAGE_PIXELS:
        raise VoidrayError(2, f"EXR: {w}x{h} is above {MAX_IMAGE_PIXELS} pixels")
    lines = _EXR_LINES[comp]
    nchunks = (h + lines - 1) // lines
    offsets = struct.unpack(f"<{nchunks}Q", data[pos:pos + 8 * nchunks])
    planes = {name: np.zeros((h, w), np.float32) for name, _ in chans}
    row_bytes = sum(_EXR_TYPES[t][1] for _, t in chans) * w
    for off in offsets:
        y, size = struct.unpack("<ii", data[off:off + 8])
        blob = data[off + 8:off + 8 + size]
        y0 = y - ymin
        if not 0 <= y0 < h:
            raise VoidrayError(1, f"EXR: chunk for line {y} outside the data window")
        n = min(lines, h - y0)
        want = row_bytes * n
        if size < want and comp == 1:
            blob = _exr_unpredict(_exr_rle_decode(blob, want))
        elif size < want and comp in (2, 3):
            blob = _exr_unpredict(zlib.decompress(blob))
        if len(blob) != want:
            raise VoidrayError(1, "EXR: chunk has the wrong size")
        p = 0
        for r in range(n):
            for name, t in chans:
                dt, sz = _EXR_TYPES[t]
                planes[name][y0 + r] = np.frombuffer(blob, dt, w, p).astype(np.float32)
                p += sz * w
    if not all(c in planes for c in "RGB"):
        raise VoidrayError(2, "EXR: needs R, G and B channels")
    return np.ascontiguousarray(np.stack([planes["R"], planes["G"], planes["B"]], axis=-1))


# ------------------------------------------------------------------- JPEG ---
_JPEG_MAGIC = b"\xff\xd8\xff"


def jpeg_info(data: bytes) -> dict:
    """Frame-header facts of a JPEG stream (no pixels decoded)."""
    from . import _native as N

    buf = np.frombuffer(data, np.uint8)
    info = N.vr_image_info()
    N.check(N.lib().vr_image_info_get(buf.ctypes.data, buf.size, ctypes.byref(info)))
    return {"width": info.width, "height": info.height, "components": info.components,
            "progressive": bool(info.progressive)}


def decode_jpeg_rgb8(data: bytes) -> np.ndarray:
    """Decodes a JPEG stream with the native decoder: uint8 RGB [height, width, 3]."""
    from . import _native as N

    info = jpeg_info(data)
    buf = np.frombuffer(data, np.uint8)
    out = np.empty((info["height"], info["width"], 3), np.uint8)
    N.check(N.lib().vr_image_decode_rgb8(buf.ctypes.data, buf.size, out.ctypes.data, out.nbytes))
    return out


def decode_jpeg(data: bytes) -> np.ndarray:
    return decode_jpeg_rgb8(data).astype(np.float32) / np.float32(255.0)


# ------------------------------------------------------------------- TIFF ---
_TIFF_TYPES = {1: "B", 2: "c", 3: "H", 4: "I", 5: "II", 6: "b", 7: "B", 8: "h", 9: "i", 10: "ii", 11: "f",
               12: "d", 16: "Q", 17: "q", 18: "Q"}
_TIFF_SIZES = {1: 1, 2: 1, 3: 2, 4: 4, 5: 8, 6: 1, 7: 1, 8: 2, 9: 4, 10: 8, 11: 4, 12: 8, 16: 8, 17: 8, 18: 8}


def _tiff_ifd(data: bytes, bo: str):
    """Tags of the first image file directory: {tag: tuple of values}."""
    if len(data) < 8:
        raise VoidrayError(1, "TIFF: truncated header")
    magic, off = struct.unpack(bo + "HI", data[2:8])
    if magic == 43:
        raise VoidrayError(2, "TIFF: BigTIFF is not decoded here")
    if magic != 42 or off + 2 > len(data):
        raise VoidrayError(1, "TIFF: bad header")
    (n,) = struct.unpack(bo + "H", data[off:off + 2])
    if off + 2 + 12 * n > len(data):
        raise VoidrayError(1, "TIFF: truncated directory")
    tags = {}
    for i in range(n):
        tag, typ, cnt = struct.unpack(bo + "HHI", data[off + 2 + 12 * i:off + 10 + 12 * i])
        if typ not in _TIFF_SIZES:
            continue
        size = _TIFF_SIZES[typ] * cnt
        if size <= 4:
            raw = data[off + 10 + 12 * i:off + 10 + 12 * i + size]
        else:
            (voff,) = struct.unpack(bo + "I", data[off + 10 + 12 * i:off + 14 + 12 * i])
            raw = data[voff:voff + size]
            if len(raw) != size:
                raise VoidrayError(1, f"TIFF: tag {tag} points past the end of the file")
        if typ == 2:
            tags[tag] = (raw.split(b"\0")[0].decode("latin-1"),)
            continue
        fmt = _TIFF_TYPES[typ]
        vals = struct.unpack(bo + fmt * cnt, raw)
        if typ in (5, 10):
            vals = tuple(vals[2 * k] / vals[2 * k + 1] if vals[2 * k + 1] else 0.0 for k in range(cnt))
        tags[tag] = vals
    return tags


def _tiff_lzw_decode(src: bytes, size: int) -> bytes:
    """TIFF 6.0 LZW (native vr_tiff_lzw_decode): the first `size` bytes of the
    decoded stream, fewer when the stream is shorter."""
    from . import _native as N

    buf = np.frombuffer(src, np.uint8)
    length = ctypes.c_size_t(0)
    # the decoded length first, so that a header's claimed size allocates nothing
    N.check(N.lib().vr_tiff_lzw_decode(buf.ctypes.data, buf.size, None, 0, ctypes.byref(length)))
    out = np.empty(min(size, length.value), np.uint8)
    N.check(N.lib().vr_tiff_lzw_decode(buf.ctypes.data, buf.size, out.ctypes.data, out.size, ctypes.byref(length)))
    return out.tobytes()


def _tiff_packbits_decode(src: bytes, size: int) -> bytes:
    out = bytearray()
    i, n = 0, len(src)
    while i < n and len(out) < size:
        h = src[i]
        i += 1
        if h < 128:
            out += src[i:i + h + 1]
            i += h + 1
        elif h > 128:
            if i >= n:
                break
            out += bytes((src[i],)) * (257 - h)
            i += 1
    return bytes(out)


def _tiff_chunk(raw: bytes, compression: int, size: int) -> bytes:
    if compression == 1:
        out = raw
    elif compression == 5:
        out = _tiff_lzw_decode(raw, size)
    elif compression in (8, 32946):
        try:
            out = zlib.decompress(raw)
        except zlib.error as e:
            raise VoidrayError(1, f"TIFF: corrupt Deflate data ({e})") from None
    elif compression == 32773:
        out = _tiff_packbits_decode(raw, size)
    else:
        raise VoidrayError(2, f"TIFF: compression {compression} is not decoded here")
    if len(out) < size:
        raise VoidrayError(1, f"TIFF: chunk holds {len(out)} bytes, {size} expected")
    return out[:size]


def _tiff_samples(buf: bytes, rows: int, cols: int, spp: int, bps: int, fmt: int, bo: str,
                  predictor: int) -> np.ndarray:
    """One decompressed strip or tile -> samples [rows, cols, spp] (integers or floats)."""
    row_bytes = (cols * spp * bps + 7) // 8
    a = np.frombuffer(buf, np.uint8, rows * row_bytes).reshape(rows, row_bytes)
    if predictor == 3:  # floating-point predictor: byte differences, then byte planes MSB first
        if fmt != 3 or bps not in (16, 32, 64):
            raise VoidrayError(1, "TIFF: floating-point predictor on non-float samples")
        a = np.cumsum(a.reshape(rows, row_bytes), axis=1, dtype=np.uint8)
        nb = bps // 8
        planes = a.reshape(rows, nb, cols * spp).transpose(0, 2, 1)
        return np.ascontiguousarray(planes).view(np.dtype(f">f{nb}")).reshape(rows, cols, spp)
    if bps < 8:
        bits = np.unpackbits(a, axis=1)[:, :cols * spp * bps].reshape(rows, cols * spp, bps)
        weights = (1 << np.arange(bps - 1, -1, -1)).astype(np.uint32)
        v = (bits.astype(np.uint32) * weights).sum(-1).reshape(rows, cols, spp)
        if predictor == 2:
            v = np.cumsum(v, axis=1) % (1 << bps)
        return v.astype(np.uint32)
    if bps % 8:
        raise VoidrayError(2, f"TIFF: {bps}-bit samples are not decoded here")
    kind = {1: "u", 2: "i", 3: "f"}.get(fmt)
    if kind is None or (kind == "f" and bps not in (16, 32, 64)) or (kind != "f" and bps > 32):
        raise VoidrayError(2, f"TIFF: sample format {fmt} with {bps} bits is not decoded here")
    dt = np.dtype(f"{bo}{kind}{bps // 8}")
    v = a.view(dt).reshape(rows, cols, spp)
    if predictor == 2:
        if kind == "f":
            raise VoidrayError(1, "TIFF: horizontal predictor on float samples")
        v = np.cumsum(v, axis=1, dtype=dt.newbyteorder("="))
    return v


@_corrupt_is_invalid("TIFF")
def decode_tiff(data: bytes) -> np.ndarray:
    bo = {b"II": "<", b"MM": ">"}.get(data[:2])
    if bo is None:
        raise VoidrayError(1, "TIFF: bad byte-order mark")
    t = _tiff_ifd(data, bo)

    def ints(tag):
        v = t.get(tag)
        if v is not None and not all(isinstance(x, int) and x >= 0 for x in v):
            raise VoidrayError(1, f"TIFF: tag {tag} holds {v[:4]!r}, not unsigned integers")
        return v

    def one(tag, default=None):
        v = ints(tag)
        if not v:
            if default is None:
                raise VoidrayError(1, f"TIFF: required tag {tag} missing")
            return default
        return v[0]

    width, height = int(one(256)), int(one(257))
    spp = int(one(277, 1))
    bps_all = ints(258) or (1,) * spp
    if len(set(bps_all)) != 1:
        raise VoidrayError(2, f"TIFF: mixed bit depths {bps_all}")
    bps = int(bps_all[0])
    fmt = int(one(339, 1))
    compression = int(one(259, 1))
    photometric = int(one(262))
    planar = int(one(284, 1))
    predictor = int(one(317, 1))
    if width <= 0 or height <= 0 or width * height > MAX_IMAGE_PIXELS:
        raise VoidrayError(2 if width * height > MAX_IMAGE_PIXELS else 1, f"TIFF: image size {width}x{height}")
    if not 1 <= spp <= 16:
        raise VoidrayError(1, f"TIFF: {spp} samples per pixel")
    if photometric not in (0, 1, 2, 3):
        raise VoidrayError(2, f"TIFF: photometric interpretation {photometric} is not decoded here")
    if photometric == 2 and spp < 3 or photometric != 2 and spp < 1:
        raise VoidrayError(1, f"TIFF: {spp} samples per pixel for photometric {photometric}")
    if predictor not in (1, 2, 3):
        raise VoidrayError(2, f"TIFF: predictor {predictor}")
    planes = spp if planar == 2 else 1
    chunk_spp = 1 if planar == 2 else spp
    if 322 in t:
        cw, chh = int(one(322)), int(one(323))
        offsets, counts = ints(324), ints(325)
        across, down = -(-width // cw), -(-height // chh)
        layout = [(p, ty * chh, tx * cw, chh, cw) for p in range(planes) for ty in range(down) for tx in range(across)]
    else:
        rps = min(int(one(278, height)), height)
        offsets, counts = ints(273), ints(279)
        per_plane = -(-height // rps)
        layout = [(p, s * rps, 0, min(rps, height - s * rps), width) for p in range(planes) for s in range(per_plane)]
    if offsets is None or counts is None or len(offsets) < len(layout) or len(counts) < len(layout):
        raise VoidrayError(1, "TIFF: chunk offsets or byte counts missing")
    img = None
    for k, (p, y0, x0, rows, cols) in enumerate(layout):
        raw = data[offsets[k]:offsets[k] + counts[k]]
        if len(raw) != counts[k]:
            raise VoidrayError(1, "TIFF: chunk points past the end of the file")
        size = rows * ((cols * chunk_spp * bps + 7) // 8)
        v = _tiff_samples(_tiff_chunk(raw, compression, size), rows, cols, chunk_spp, bps, fmt, bo, predictor)
        if img is None:
            img = np.zeros((height, width, spp), v.dtype.newbyteorder("="))
        h, w = min(rows, height - y0), min(cols, width - x0)
        img[y0:y0 + h, x0:x0 + w, p:p + chunk_spp] = v[:h, :w]
    if photometric == 3:
        cmap = ints(320)
        if cmap is None or len(cmap) != 3 * (1 << bps):
            raise VoidrayError(1, "TIFF: palette image without a colour map of 3 * 2^bits entries")
        cm = np.asarray(cmap, np.float32).reshape(3, -1).T / np.float32(65535.0)
        return np.ascontiguousarray(cm[img[..., 0].astype(np.int64)])
    if img.dtype.kind == "f":
        f = img.astype(np.float32)
        if photometric == 0:
            f = np.float32(1.0) - f
    else:
        if img.dtype.kind == "i":
            raise VoidrayError(2, "TIFF: signed integer samples are not decoded here")
        if bps < 8:  # low bit depths expand to 8 bits, as for PNG
            img = img * (255 // ((1 << bps) - 1))
            maxv = 255
        else:
            maxv = (1 << bps) - 1
        if photometric == 0:
            img = maxv - img
        f = img.astype(np.float32) / np.float32(maxv)
    if photometric in (0, 1):
        return np.ascontiguousarray(np.repeat(f[..., :1], 3, axis=-1))
    return np.ascontiguousarray(f[..., :3])


def load_image_rgb32f(path: str) -> np.ndarray:
    """Decodes an image file to float32 RGB [height, width, 3], row 0 at the top."""
    with open(path, "rb") as f:
        data = f.read()
    if data[:8] == _PNG_MAGIC:
        return decode_png(data)
    if len(data) >= 4 and struct.unpack("<i", data[:4])[0] == _EXR_MAGIC:
        return decode_exr(data)
    if data[:3] == _JPEG_MAGIC:
        return decode_jpeg(data)
    if data[:4] in (b"II*\0", b"MM\0*", b"II+\0", b"MM\0+"):
        return decode_tiff(data)
    ext = os.path.splitext(path)[1].lower()
    raise VoidrayError(2, f"image format of {os.path.basename(path)!r} ({ext or 'unknown'}) is not "
                          "decoded here: pass float RGB arrays instead")
