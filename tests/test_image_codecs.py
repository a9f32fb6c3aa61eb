"""JPEG (native decoder, include/voidray_assets.h) and TIFF (voidray_gb300.assets)
decoding against independent encoders written here.

The JPEG encoder follows ITU-T T.81: JFIF colour conversion, forward DCT,
quantisation, Huffman tables built from the symbol counts with the Annex K.2
length limit, sequential interleaved and single-component scans, restart
intervals, and progressive scans (DC first / refinement, AC bands with EOB runs,
AC refinement with correction bits).  The decoder's output is compared with a
float64 numpy decode of the same quantised coefficients (inverse DCT, IJG
triangle upsampling, JFIF matrix); a progressive stream must decode to exactly
the bytes of the sequential stream with the same coefficients.  No GPU.
"""
import heapq
import os
import struct
import zlib
from pathlib import Path

import numpy as np
import pytest

from voidray_gb300 import assets as A
from voidray_gb300._native import VoidrayError

ZZ = np.array([0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5, 12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6,
               7, 14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51, 58, 59, 52, 45, 38, 31,
               39, 46, 53, 60, 61, 54, 47, 55, 62, 63])
_U = np.arange(8)
DCT = np.array([[(np.sqrt(0.5) if u == 0 else 1.0) * 0.5 * np.cos((2 * x + 1) * u * np.pi / 16) for x in _U]
                for u in _U])  # DCT[u, x]
# the reference checkout, when the environment names one (VOIDRAY_REFERENCE); otherwise these tests skip
_REF_ROOT = os.environ.get("VOIDRAY_REFERENCE", "")
ASSETS = Path(_REF_ROOT) / "assets" if _REF_ROOT else Path("/nonexistent-voidray-assets")


# ------------------------------------------------------------ JPEG encoder ---
def huffman_table(freq):
    """(bits[1..16], symbols) from symbol counts: Huffman code sizes, Annex K.2
    limit to 16 bits, one reserved code so that no code is all ones."""
    f = {s: c for s, c in freq.items() if c}
    f[256] = 1
    size = dict.fromkeys(f, 0)
    heap = [(c, i, [s]) for i, (s, c) in enumerate(sorted(f.items()))]
    heapq.heapify(heap)
    uid = len(heap)
    while len(heap) > 1:
        c1, _, s1 = heapq.heappop(heap)
        c2, _, s2 = heapq.heappop(heap)
        for s in s1 + s2:
            size[s] += 1
        heapq.heappush(heap, (c1 + c2, uid, s1 + s2))
        uid += 1
    bits = [0] * 40
    for s in f:
        bits[size[s]] += 1
    for i in range(39, 16, -1):
        while bits[i] > 0:
            j = i - 2
            while bits[j] == 0:
                j -= 1
            bits[i] -= 2
            bits[i - 1] += 1
            bits[j + 1] += 2
            bits[j] -= 1
    i = 16
    while bits[i] == 0:
        i -= 1
    bits[i] -= 1
    syms = [s for _, s in sorted((size[s], s) for s in f if s != 256)]
    return bits[1:17], syms


def canonical_codes(bits, syms):
    codes, code, k = {}, 0, 0
    for ln in range(1, 17):
        for _ in range(bits[ln - 1]):
            codes[syms[k]] = (code, ln)
            code += 1
            k += 1
        code <<= 1
    return codes


class BitWriter:
    def __init__(self):
        self.out = bytearray()
        self.acc = 0
        self.n = 0

    def put(self, v, n):
        for i in range(n - 1, -1, -1):
            self.acc = (self.acc << 1) | ((v >> i) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                if self.acc == 0xFF:
                    self.out.append(0)
                self.acc = self.n = 0

    def flush(self):
        if self.n:
            self.put((1 << (8 - self.n)) - 1, 8 - self.n)


def category(v):
    return int(abs(int(v))).bit_length()


def magnitude_bits(v, s):
    v = int(v)
    return v if v >= 0 else v + (1 << s) - 1


class Emitter:
    """Pass 1 counts symbols per table; pass 2 writes them with the built codes."""

    def __init__(self, codes=None):
        self.codes = codes
        self.freq = {}
        self.bw = BitWriter()

    def sym(self, table, s):
        if self.codes is None:
            self.freq.setdefault(table, {}).setdefault(s, 0)
            self.freq[table][s] += 1
        else:
            code, ln = self.codes[table][s]
            self.bw.put(code, ln)

    def bits(self, v, n):
        if self.codes is not None and n:
            self.bw.put(v, n)


def rgb_to_ycc(img):
    r, g, b = (img[..., i].astype(np.float64) for i in range(3))
    y = 0.299 * r + 0.587 * g + 0.114 * b
    cb = -0.168736 * r - 0.331264 * g + 0.5 * b + 128
    cr = 0.5 * r - 0.418688 * g - 0.081312 * b + 128
    return [np.clip(np.floor(p + 0.5), 0, 255) for p in (y, cb, cr)]


def forward_blocks(plane, bw, bh, q):
    """Quantised coefficients [bh, bw, 64] (natural order) of a plane padded by edge replication."""
    h, w = plane.shape
    p = np.pad(plane, ((0, bh * 8 - h), (0, bw * 8 - w)), mode="edge") - 128.0
    blk = p.reshape(bh, 8, bw, 8).transpose(0, 2, 1, 3)
    coef = np.einsum("ux,vy,abyx->abvu", DCT, DCT, blk)
    return np.round(coef.reshape(bh, bw, 64) / q.reshape(64)).astype(np.int64)


class Jpeg:
    """Quantised coefficients of an image and the ways to code them."""

    def __init__(self, img, sampling=((1, 1), (1, 1), (1, 1)), quality_q=None, colour="ycc", seed=0):
        rng = np.random.default_rng(seed)
        self.h, self.w = img.shape[:2]
        if img.ndim == 2:
            planes = [img.astype(np.float64)]
            sampling = ((1, 1),)
        elif colour == "ycc":
            planes = rgb_to_ycc(img)
        else:
            planes = [img[..., i].astype(np.float64) for i in range(img.shape[2])]
        self.samp = sampling
        self.hmax = max(s[0] for s in sampling)
        self.vmax = max(s[1] for s in sampling)
        self.mcux = -(-self.w // (8 * self.hmax))
        self.mcuy = -(-self.h // (8 * self.vmax))
        if quality_q is None:
            quality_q = [rng.integers(1, 24, 64) for _ in range(min(2, len(planes)))]
        self.q = [np.asarray(t, np.int64) for t in quality_q]
        self.tq = [0] + [len(self.q) - 1] * (len(planes) - 1)
        self.comps = []
        for i, p in enumerate(planes):
            hs, vs = sampling[i]
            cw, ch = -(-self.w * hs // self.hmax), -(-self.h * vs // self.vmax)
            fy, fx = self.vmax // vs, self.hmax // hs
            # box-filtered chroma at the component's size
            ph, pw = ch * fy, cw * fx
            pp = np.pad(p, ((0, max(0, ph - self.h)), (0, max(0, pw - self.w))), mode="edge")[:ph, :pw]
            sub = pp.reshape(ch, fy, cw, fx).mean(axis=(1, 3))
            bw, bh = self.mcux * hs, self.mcuy * vs
            self.comps.append(dict(h=hs, v=vs, cw=cw, ch=ch, bw=bw, bh=bh,
                                   coef=forward_blocks(sub, bw, bh, self.q[self.tq[i]])))

    # ---- markers
    def _header(self, sof, adobe=None, jfif=True, ids=None):
        out = bytearray(b"\xff\xd8")
        if jfif:
            body = b"JFIF\x00\x01\x01\x00\x00\x01\x00\x01\x00\x00"
            out += b"\xff\xe0" + struct.pack(">H", len(body) + 2) + body
        if adobe is not None:
            body = b"Adobe" + struct.pack(">HHHB", 100, 0, 0, adobe)
            out += b"\xff\xee" + struct.pack(">H", len(body) + 2) + body
        for t, q in enumerate(self.q):
            body = bytes([t]) + bytes(int(x) for x in q[ZZ])
            out += b"\xff\xdb" + struct.pack(">H", len(body) + 2) + body
        ids = ids or list(range(1, len(self.comps) + 1))
        self.ids = ids
        body = struct.pack(">BHHB", 8, self.h, self.w, len(self.comps))
        for i, c in enumerate(self.comps):
            body += bytes([ids[i], (c["h"] << 4) | c["v"], self.tq[i]])
        out += bytes([0xFF, sof]) + struct.pack(">H", len(body) + 2) + body
        return out

    @staticmethod
    def _dht(tables):
        out = bytearray()
        for (cls, tid), (bits, syms) in tables.items():
            body = bytes([(cls << 4) | tid]) + bytes(bits) + bytes(syms)
            out += b"\xff\xc4" + struct.pack(">H", len(body) + 2) + body
        return out

    def _units(self, comp_idx):
        """Blocks in scan order: per MCU for interleaved scans, raster for single-component ones."""
        if len(comp_idx) == 1:
            c = self.comps[comp_idx[0]]
            for by in range(-(-c["ch"] // 8)):
                for bx in range(-(-c["cw"] // 8)):
                    yield [(comp_idx[0], by, bx)]
        else:
            for my in range(self.mcuy):
                for mx in range(self.mcux):
                    u = []
                    for ci in comp_idx:
                        c = self.comps[ci]
                        for v in range(c["v"]):
                            for h in range(c["h"]):
                                u.append((ci, my * c["v"] + v, mx * c["h"] + h))
                    yield u

    def _scan(self, comp_idx, kind, ss, se, ah, al, restart, tables_of):
        """Codes one scan twice (counting, then writing); returns DHT + SOS + data."""
        def run(em):
            pred = dict.fromkeys(comp_idx, 0)
            state = {"eobrun": 0, "be": []}

            def flush_eob():
                n = state["eobrun"]
                if n:
                    nb = n.bit_length() - 1
                    em.sym(tables_of(comp_idx[0])[1], nb << 4)
                    em.bits(n - (1 << nb), nb)
                    state["eobrun"] = 0
                for b in state["be"]:
                    em.bits(b, 1)
                state["be"] = []

            for ui, unit in enumerate(self._units(comp_idx)):
                if restart and ui and ui % restart == 0:
                    flush_eob()
                    if em.codes is not None:
                        em.bw.flush()
                        em.bw.out += bytes([0xFF, 0xD0 + ((ui // restart - 1) & 7)])
                    pred = dict.fromkeys(comp_idx, 0)
                for ci, by, bx in unit:
                    coef = self.comps[ci]["coef"][by, bx]
                    dct, act = tables_of(ci)
                    if kind == "seq":
                        d = int(coef[0]) - pred[ci]
                        pred[ci] = int(coef[0])
                        s = category(d)
                        em.sym(dct, s)
                        em.bits(magnitude_bits(d, s), s)
                        r = 0
                        for k in range(1, 64):
                            v = int(coef[ZZ[k]])
                            if v == 0:
                                r += 1
                                continue
                            while r > 15:
                                em.sym(act, 0xF0)
                                r -= 16
                            s = category(v)
                            em.sym(act, (r << 4) | s)
                            em.bits(magnitude_bits(v, s), s)
                            r = 0
                        if r:
                            em.sym(act, 0x00)
                    elif kind == "dc_first":
                        v = int(coef[0]) >> al
                        d = v - pred[ci]
                        pred[ci] = v
                        s = category(d)
                        em.sym(dct, s)
                        em.bits(magnitude_bits(d, s), s)
                    elif kind == "dc_refine":
                        em.bits((int(coef[0]) >> al) & 1, 1)
                    elif kind == "ac_first":
                        r = 0
                        for k in range(ss, se + 1):
                            c = int(coef[ZZ[k]])
                            v = (abs(c) >> al) * (1 if c >= 0 else -1)
                            if v == 0:
                                r += 1
                                continue
                            flush_eob()
                            while r > 15:
                                em.sym(act, 0xF0)
                                r -= 16
                            s = category(v)
                            em.sym(act, (r << 4) | s)
                            em.bits(magnitude_bits(v, s), s)
                            r = 0
                        if r:
                            state["eobrun"] += 1
                            if state["eobrun"] == 0x7FFF:
                                flush_eob()
                    else:  # ac_refine
                        absv = [abs(int(coef[ZZ[k]])) >> al for k in range(64)]
                        eob = max([k for k in range(ss, se + 1) if absv[k] == 1], default=0)
                        r, br = 0, []
                        for k in range(ss, se + 1):
                            t = absv[k]
                            if t == 0:
                                r += 1
                                continue
                            while r > 15 and k <= eob:
                                flush_eob()
                                em.sym(act, 0xF0)
                                r -= 16
                                for b in br:
                                    em.bits(b, 1)
                                br = []
                            if t > 1:
                                br.append(t & 1)
                                continue
                            flush_eob()
                            em.sym(act, (r << 4) | 1)
                            em.bits(1 if int(coef[ZZ[k]]) > 0 else 0, 1)
                            for b in br:
                                em.bits(b, 1)
                            br, r = [], 0
                        if r > 0 or br:
                            state["eobrun"] += 1
                            state["be"] += br
                            if state["eobrun"] == 0x7FFF or len(state["be"]) > 937:
                                flush_eob()
            flush_eob()

        counter = Emitter()
        run(counter)
        tables = {key: huffman_table(fr) for key, fr in counter.freq.items()}
        writer = Emitter({key: canonical_codes(*t) for key, t in tables.items()})
        run(writer)
        writer.bw.flush()
        dht = self._dht({(1 if key[0] == "ac" else 0, key[1]): t for key, t in tables.items()})
        body = bytes([len(comp_idx)])
        for ci in comp_idx:
            d, a = tables_of(ci)
            body += bytes([self.ids[ci], (d[1] << 4) | a[1]])
        body += bytes([ss, se, (ah << 4) | al])
        return dht + b"\xff\xda" + struct.pack(">H", len(body) + 2) + body + bytes(writer.bw.out)

    @staticmethod
    def _tables(ci):
        t = 0 if ci == 0 else 1
        return ("dc", t), ("ac", t)

    def _dri(self, restart):
        return b"\xff\xdd\x00\x04" + struct.pack(">H", restart) if restart else b""

    def sequential(self, restart=0, interleaved=True, adobe=None, jfif=True, ids=None, sof=0xC0):
        out = self._header(sof, adobe, jfif, ids) + self._dri(restart)
        groups = [list(range(len(self.comps)))] if interleaved else [[i] for i in range(len(self.comps))]
        for g in groups:
            out += self._scan(g, "seq", 0, 63, 0, 0, restart, self._tables)
        return bytes(out + b"\xff\xd9")

    def progressive(self, restart=0, script=None):
        out = self._header(0xC2) + self._dri(restart)
        n = len(self.comps)
        if script is None:
            script = [(list(range(n)), 0, 0, 0, 1)]
            for ci in range(n):
                script += [([ci], 1, 5, 0, 2), ([ci], 6, 63, 0, 2)]
            script += [(list(range(n)), 0, 0, 1, 0)]
            for ci in range(n):
                script += [([ci], 1, 63, 2, 1), ([ci], 1, 63, 1, 0)]
        for comps, ss, se, ah, al in script:
            if ss == 0:
                kind = "dc_first" if ah == 0 else "dc_refine"
            else:
                kind = "ac_first" if ah == 0 else "ac_refine"
            out += self._scan(comps, kind, ss, se, ah, al, restart, self._tables)
        return bytes(out + b"\xff\xd9")

    # ---- float64 reference decode of the same coefficients
    def reference_rgb8(self, colour="ycc"):
        planes = []
        for i, c in enumerate(self.comps):
            f = (c["coef"] * self.q[self.tq[i]]).reshape(c["bh"], c["bw"], 8, 8).astype(np.float64)
            pix = np.einsum("vy,ux,abvu->abyx", DCT, DCT, f)
            pix = np.clip(np.floor(pix + 128.5), 0, 255)
            plane = pix.transpose(0, 2, 1, 3).reshape(c["bh"] * 8, c["bw"] * 8)[:c["ch"], :c["cw"]]
            planes.append(upsample_ref(plane.astype(np.int64), self.hmax // c["h"], self.vmax // c["v"], self.w,
                                       self.h))
        if len(planes) == 1:
            return np.repeat(planes[0][..., None], 3, axis=-1).astype(np.uint8)
        if colour == "rgb":
            return np.stack(planes, -1).astype(np.uint8)
        y, cb, cr = (p.astype(np.float64) for p in planes)
        rgb = np.stack([y + 1.402 * (cr - 128), y - 0.344136 * (cb - 128) - 0.714136 * (cr - 128),
                        y + 1.772 * (cb - 128)], -1)
        return np.clip(np.floor(rgb + 0.5), 0, 255).astype(np.uint8)


def upsample_ref(p, fx, fy, w, h):
    """IJG triangle upsampling for 2x1 / 2x2, replication otherwise (numpy restatement)."""
    ch, cw = p.shape
    if fx == 1 and fy == 1:
        return p[:h, :w]
    if fx == 2 and fy in (1, 2):
        if fy == 1:
            rows = p
            left = np.concatenate([p[:, :1], p[:, :-1]], 1)
            right = np.concatenate([p[:, 1:], p[:, -1:]], 1)
            even = (3 * rows + left + 1) >> 2
            odd = (3 * rows + right + 2) >> 2
            even[:, 0] = p[:, 0]
            odd[:, -1] = p[:, -1]
            out = np.stack([even, odd], -1).reshape(ch, 2 * cw)
            return out[:h, :w]
        up = np.concatenate([p[:1], p[:-1]], 0)
        down = np.concatenate([p[1:], p[-1:]], 0)
        res = []
        for near in (up, down):
            col = 3 * p + near
            left = np.concatenate([col[:, :1], col[:, :-1]], 1)
            right = np.concatenate([col[:, 1:], col[:, -1:]], 1)
            even = (3 * col + left + 8) >> 4
            odd = (3 * col + right + 7) >> 4
            even[:, 0] = (4 * col[:, 0] + 8) >> 4
            odd[:, -1] = (4 * col[:, -1] + 7) >> 4
            res.append(np.stack([even, odd], -1).reshape(ch, 2 * cw))
        out = np.stack(res, 1).reshape(2 * ch, 2 * cw)
        return out[:h, :w]
    ys = np.minimum(np.arange(h) // fy, ch - 1)
    xs = np.minimum(np.arange(w) // fx, cw - 1)
    return p[ys][:, xs]


def test_image(h, w, seed=0, smooth=True):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w]
    base = np.stack([128 + 100 * np.sin(x / 7.0 + k) * np.cos(y / 5.0 - k) for k in range(3)], -1)
    noise = rng.normal(0, 12 if smooth else 60, (h, w, 3))
    return np.clip(base + noise, 0, 255).astype(np.uint8)


test_image.__test__ = False


def ac_symbols(stream):
    """Symbols of the AC Huffman tables a stream defines."""
    out, i = set(), 0
    while (i := stream.find(b"\xff\xc4", i)) >= 0:
        bits = stream[i + 5:i + 21]
        if stream[i + 4] >> 4 == 1:
            out |= set(stream[i + 21:i + 21 + sum(bits)])
        i += 2
    return out


def check_close(got, ref, tol):
    d = np.abs(got.astype(np.int64) - ref.astype(np.int64))
    assert got.shape == ref.shape
    assert d.max() <= tol, (d.max(), np.argwhere(d == d.max())[:3])
    assert d.mean() < 0.05, d.mean()


# ------------------------------------------------------------------- tests ---
@pytest.mark.parametrize("h,w,samp", [
    (16, 16, ((1, 1), (1, 1), (1, 1))),
    (37, 23, ((1, 1), (1, 1), (1, 1))),
    (40, 48, ((2, 1), (1, 1), (1, 1))),
    (33, 47, ((2, 2), (1, 1), (1, 1))),
    (1, 1, ((2, 2), (1, 1), (1, 1))),
    (29, 61, ((1, 2), (1, 1), (1, 1))),
    (24, 40, ((2, 2), (1, 2), (2, 1))),
])
def test_jpeg_sequential_matches_float64_decode(native, h, w, samp):
    j = Jpeg(test_image(h, w, seed=h * w), samp)
    data = j.sequential()
    info = A.jpeg_info(data)
    assert (info["width"], info["height"], info["components"], info["progressive"]) == (w, h, 3, False)
    got = A.decode_jpeg_rgb8(data)
    check_close(got, j.reference_rgb8(), 3)
    # the encoder round trip itself stays near the source image
    assert np.abs(got.astype(float) - test_image(h, w, seed=h * w)).mean() < 25


def test_jpeg_quality_one_tables_long_codes(native):
    # quantisation by 1 everywhere: DC/AC categories up to 11, Huffman codes up to 16 bits
    img = test_image(64, 72, seed=3, smooth=False)
    j = Jpeg(img, quality_q=[np.ones(64, np.int64), np.ones(64, np.int64)])
    data = j.sequential(restart=5)
    lengths, i = [], 0
    while (i := data.find(b"\xff\xc4", i)) >= 0:
        lengths += [k + 1 for k in range(16) if data[i + 5 + k]]
        i += 2
    assert max(lengths) > 9  # codes beyond the decoder's 9-bit lookup
    got = A.decode_jpeg_rgb8(data)
    check_close(got, j.reference_rgb8(), 3)
    assert np.abs(got.astype(float) - img).max() <= 4


@pytest.mark.parametrize("restart", [1, 3, 7, 200])
@pytest.mark.parametrize("interleaved", [True, False])
def test_jpeg_restart_intervals_and_single_component_scans(native, restart, interleaved):
    j = Jpeg(test_image(43, 57, seed=restart), ((2, 2), (1, 1), (1, 1)))
    plain = A.decode_jpeg_rgb8(j.sequential())
    got = A.decode_jpeg_rgb8(j.sequential(restart=restart, interleaved=interleaved))
    assert np.array_equal(got, plain)


def test_jpeg_grey_and_rgb_and_extended_sof(native):
    g = test_image(21, 34, seed=5)[..., 1]
    j = Jpeg(g)
    data = j.sequential(sof=0xC1)
    assert A.jpeg_info(data)["components"] == 1
    check_close(A.decode_jpeg_rgb8(data), j.reference_rgb8(), 1)
    img = test_image(26, 30, seed=6)
    j = Jpeg(img, colour="rgb")
    # Adobe transform 0 = RGB; component ids R, G, B without JFIF or Adobe = RGB as well
    for data in (j.sequential(adobe=0), j.sequential(jfif=False, ids=[ord("R"), ord("G"), ord("B")])):
        check_close(A.decode_jpeg_rgb8(data), j.reference_rgb8("rgb"), 1)
    jy = Jpeg(img)
    check_close(A.decode_jpeg_rgb8(jy.sequential(adobe=1)), jy.reference_rgb8(), 3)


@pytest.mark.parametrize("h,w,samp", [(32, 32, ((1, 1), (1, 1), (1, 1))), (45, 70, ((2, 2), (1, 1), (1, 1))),
                                      (17, 9, ((2, 1), (1, 1), (1, 1))),
                                      (120, 200, ((2, 2), (1, 1), (1, 1)))])  # 26 restart intervals: decoded in parallel
@pytest.mark.parametrize("restart", [0, 4])
def test_jpeg_progressive_equals_sequential(native, h, w, samp, restart):
    img = test_image(h, w, seed=w, smooth=False)
    j = Jpeg(img, samp, quality_q=[np.full(64, 2), np.full(64, 3)])
    seq = A.decode_jpeg_rgb8(j.sequential())
    prog = j.progressive(restart=restart)
    assert A.jpeg_info(prog)["progressive"]
    assert np.array_equal(A.decode_jpeg_rgb8(prog), seq)


def test_jpeg_progressive_scan_scripts(native):
    img = test_image(40, 56, seed=9, smooth=False)
    j = Jpeg(img, ((2, 2), (1, 1), (1, 1)), quality_q=[np.ones(64), np.full(64, 2)])
    seq = A.decode_jpeg_rgb8(j.sequential())
    scripts = [
        # spectral selection only, DC interleaved
        [([0, 1, 2], 0, 0, 0, 0), ([0], 1, 63, 0, 0), ([1], 1, 63, 0, 0), ([2], 1, 63, 0, 0)],
        # DC per component, three refinement levels of the luma AC band
        [([0], 0, 0, 0, 0), ([1], 0, 0, 0, 0), ([2], 0, 0, 0, 0), ([0], 1, 9, 0, 3), ([0], 10, 63, 0, 3),
         ([0], 1, 63, 3, 2), ([0], 1, 63, 2, 1), ([0], 1, 63, 1, 0), ([1], 1, 63, 0, 0), ([2], 1, 63, 0, 1),
         ([2], 1, 63, 1, 0)],
        # refinement of DC in two steps
        [([0, 1, 2], 0, 0, 0, 2), ([0, 1, 2], 0, 0, 2, 1), ([0, 1, 2], 0, 0, 1, 0), ([0], 1, 63, 0, 0),
         ([1], 1, 63, 0, 0), ([2], 1, 63, 0, 0)],
    ]
    for script in scripts:
        assert np.array_equal(A.decode_jpeg_rgb8(j.progressive(script=script)), seq)
    # long EOB runs: a flat image whose AC bands are empty in almost every block
    flat = np.full((64, 256, 3), 90, np.uint8)
    flat[5, 7] = 250
    jf = Jpeg(flat, quality_q=[np.ones(64), np.ones(64)])
    prog = jf.progressive()
    assert max(s for s in ac_symbols(prog) if s & 15 == 0 and s != 0xF0) >= 0x70  # runs of 128+ blocks
    assert np.array_equal(A.decode_jpeg_rgb8(prog), A.decode_jpeg_rgb8(jf.sequential()))


def test_jpeg_errors(native):
    j = Jpeg(test_image(24, 24, seed=1))
    good = j.sequential()
    with pytest.raises(VoidrayError) as e:
        A.decode_jpeg_rgb8(b"\xff\xd8\xff\xd9")
    assert e.value.status == 1 and "frame" in str(e.value)
    with pytest.raises(VoidrayError):
        A.decode_jpeg_rgb8(b"not a jpeg at all")
    for cut in (len(good) // 2, len(good) - 3):
        with pytest.raises(VoidrayError) as e:
            A.decode_jpeg_rgb8(good[:cut])
        assert e.value.status == 1
    # lossless (SOF3) and 12-bit frames are reported as unsupported
    lossless = good.replace(b"\xff\xc0", b"\xff\xc3", 1)
    with pytest.raises(VoidrayError) as e:
        A.decode_jpeg_rgb8(lossless)
    assert e.value.status == 2
    sof = good.index(b"\xff\xc0")
    twelve = good[:sof + 4] + b"\x0c" + good[sof + 5:]
    with pytest.raises(VoidrayError) as e:
        A.decode_jpeg_rgb8(twelve)
    assert e.value.status == 2
    # an output buffer that is too small is an error, not an overflow
    buf = np.frombuffer(good, np.uint8)
    out = np.zeros(24 * 24 * 3 - 1, np.uint8)
    assert native.lib().vr_image_decode_rgb8(buf.ctypes.data, buf.size, out.ctypes.data, out.nbytes) == 1
    # a Huffman table that refers to undefined codes
    i = good.index(b"\xff\xc4")
    bad = bytearray(good)
    bad[i + 5:i + 21] = bytes([0] * 15 + [1])  # one 16-bit code only
    with pytest.raises(VoidrayError):
        A.decode_jpeg_rgb8(bytes(bad))


def test_jpeg_fuzzed_streams_never_crash(native):
    rng = np.random.default_rng(11)
    good = Jpeg(test_image(32, 40, seed=2), ((2, 2), (1, 1), (1, 1))).sequential(restart=2)
    for _ in range(300):
        b = bytearray(good)
        for _ in range(rng.integers(1, 8)):
            b[rng.integers(2, len(b))] = rng.integers(0, 256)
        try:
            out = A.decode_jpeg_rgb8(bytes(b))
            assert out.shape[2] == 3
        except VoidrayError as e:
            assert e.status in (1, 2)


@pytest.mark.skipif(not (ASSETS / "mushroom_albedo.jpg").exists(), reason="the reference's assets are not here")
def test_jpeg_reference_assets(native):
    for name in ("mushroom_albedo.jpg", "mossy_ground_albedo.jpg"):
        data = (ASSETS / name).read_bytes()
        assert A.jpeg_info(data) == {"width": 2048, "height": 2048, "components": 3, "progressive": False}
        img = A.load_image_rgb32f(str(ASSETS / name))
        assert img.shape == (2048, 2048, 3) and img.dtype == np.float32
        assert 0.0 <= img.min() and img.max() <= 1.0 and 0.1 < img.mean() < 0.9


def test_jpeg_and_tiff_files_reach_textures(native, tmp_path):
    from voidray_gb300.scene import ImageTexture, SampleType, Scene

    img = test_image(20, 28, seed=12)
    j = Jpeg(img)
    (tmp_path / "a.jpg").write_bytes(j.sequential())
    (tmp_path / "b.tif").write_bytes(write_tiff(img, compression=5, predictor=2))
    t = ImageTexture.from_file(str(tmp_path / "a.jpg"), SampleType.Bilinear)
    assert np.array_equal(t.image, A.decode_jpeg_rgb8(j.sequential()).astype(np.float32) / np.float32(255.0))
    s = Scene()
    assert s.add_image_texture(str(tmp_path / "b.tif")) == 0
    assert np.array_equal(ImageTexture.from_file(str(tmp_path / "b.tif")).image,
                          img.astype(np.float32) / np.float32(255.0))


@pytest.mark.skipif(not (ASSETS / "mushroom.obj").exists(), reason="the reference's assets are not here")
def test_mushroom_demo_scene_from_reference_assets(native):
    from voidray_gb300 import workloads as W

    scene, settings, dims = W.mushroom_scene(str(ASSETS))
    info = scene.validate()  # host BVH build and structural checks
    assert dims == (1000, 1000) and info.num_triangles > 10_000
    texel_bytes = sum(t.image.nbytes for t in scene.textures)
    assert texel_bytes == 2 * 2048 * 2048 * 3 * 4
    assert info.device_bytes > texel_bytes  # the estimate counts the textures it uploads
    assert int(settings.color_management.tonemap) == 1 and settings.color_management.gamma == 1.0


# ------------------------------------------------------------ TIFF writer ---
def lzw_encode(data: bytes) -> bytes:
    """TIFF LZW with the early code-width change and a Clear before the table fills."""
    out = bytearray()
    acc = [0, 0]

    def put(code, n):
        acc[0] = (acc[0] << n) | code
        acc[1] += n
        while acc[1] >= 8:
            acc[1] -= 8
            out.append((acc[0] >> acc[1]) & 0xFF)

    def width(nxt):
        return 9 if nxt < 512 else 10 if nxt < 1024 else 11 if nxt < 2048 else 12

    table = {bytes((i,)): i for i in range(256)}
    nxt = 258
    put(256, 9)
    w = b""
    for byte in data:
        wc = w + bytes((byte,))
        if wc in table:
            w = wc
            continue
        put(table[w], width(nxt))
        table[wc] = nxt
        nxt += 1
        w = bytes((byte,))
        if nxt == 4094:
            put(256, width(nxt))
            table = {bytes((i,)): i for i in range(256)}
            nxt = 258
    if w:
        put(table[w], width(nxt))
        nxt += 1
    put(257, width(nxt))
    if acc[1]:
        out.append((acc[0] << (8 - acc[1])) & 0xFF)
    return bytes(out)


def packbits_encode(data: bytes) -> bytes:
    out, i, n = bytearray(), 0, len(data)
    while i < n:
        j = i
        while j + 1 < n and data[j + 1] == data[i] and j - i < 127:
            j += 1
        if j > i:
            out += bytes((257 - (j - i + 1),)) + data[i:i + 1]
            i = j + 1
            continue
        j = i
        while j + 1 < n and data[j + 1] != data[j] and j - i < 127:
            j += 1
        out += bytes((j - i,)) + data[i:j + 1]
        i = j + 1
    return bytes(out)


def write_tiff(arr, bo="<", compression=1, predictor=1, planar=1, tile=None, rows_per_strip=None,
               photometric=None, colormap=None, bps=None, fmt=1):
    """arr: [h, w, spp] integers or floats -> TIFF bytes (one image)."""
    h, w, spp = arr.shape
    bps = bps or arr.dtype.itemsize * 8
    if photometric is None:
        photometric = 2 if spp >= 3 else 1

    def encode_rows(block):  # block [rows, cols, nspp] -> raw chunk bytes
        rows, cols, ns = block.shape
        if predictor == 2:
            block = block.astype(np.int64)
            d = np.diff(block, axis=1, prepend=0)
            d[:, 0] = block[:, 0]
            block = (d % (1 << bps)).astype(block.dtype)
        if bps < 8:
            bits = ((block.reshape(rows, cols * ns)[..., None] >> np.arange(bps - 1, -1, -1)) & 1).astype(np.uint8)
            raw = np.packbits(bits.reshape(rows, -1), axis=1).tobytes()
        elif predictor == 3:
            nb = bps // 8
            be = block.astype(np.dtype(f">f{nb}")).reshape(rows, cols * ns).view(np.uint8).reshape(rows, cols * ns, nb)
            planes = be.transpose(0, 2, 1).reshape(rows, -1).astype(np.int64)
            d = np.diff(planes, axis=1, prepend=0)
            d[:, 0] = planes[:, 0]
            raw = (d % 256).astype(np.uint8).tobytes()
        else:
            raw = block.astype(arr.dtype.newbyteorder(bo)).tobytes()
        if compression == 5:
            return lzw_encode(raw)
        if compression == 8:
            return zlib.compress(raw)
        if compression == 32773:
            row_bytes = len(raw) // rows
            return b"".join(packbits_encode(raw[r * row_bytes:(r + 1) * row_bytes]) for r in range(rows))
        return raw

    planes = [arr[..., p:p + 1] for p in range(spp)] if planar == 2 else [arr]
    chunks = []
    if tile:
        tw, th = tile
        for pl in planes:
            for ty in range(0, h, th):
                for tx in range(0, w, tw):
                    blk = np.zeros((th, tw, pl.shape[2]), arr.dtype)
                    part = pl[ty:ty + th, tx:tx + tw]
                    blk[:part.shape[0], :part.shape[1]] = part
                    chunks.append(encode_rows(blk))
    else:
        rps = rows_per_strip or h
        for pl in planes:
            for y0 in range(0, h, rps):
                chunks.append(encode_rows(pl[y0:y0 + rps]))
    body = bytearray(b"II*\0" if bo == "<" else b"MM\0*") + b"\0\0\0\0"
    offsets = []
    for c in chunks:
        offsets.append(len(body))
        body += c
        if len(body) % 2:
            body += b"\0"
    extra = bytearray()
    entries = []

    def tag(t, typ, vals):
        fmt_c = {3: "H", 4: "I"}[typ]
        raw = struct.pack(bo + fmt_c * len(vals), *vals)
        entries.append((t, typ, len(vals), raw))

    tag(256, 4, [w])
    tag(257, 4, [h])
    tag(258, 3, [bps] * spp)
    tag(259, 3, [compression])
    tag(262, 3, [photometric])
    if tile:
        tag(322, 4, [tile[0]])
        tag(323, 4, [tile[1]])
        tag(324, 4, offsets)
        tag(325, 4, [len(c) for c in chunks])
    else:
        tag(273, 4, offsets)
        tag(278, 4, [rows_per_strip or h])
        tag(279, 4, [len(c) for c in chunks])
    tag(277, 3, [spp])
    tag(284, 3, [planar])
    if predictor != 1:
        tag(317, 3, [predictor])
    if colormap is not None:
        tag(320, 3, list(colormap.T.reshape(-1)))
    if spp in (2, 4):
        tag(338, 3, [2])
    tag(339, 3, [fmt] * spp)
    entries.sort()
    ifd_off = len(body)
    data_off = ifd_off + 2 + 12 * len(entries) + 4
    ifd = bytearray(struct.pack(bo + "H", len(entries)))
    for t, typ, cnt, raw in entries:
        if len(raw) <= 4:
            ifd += struct.pack(bo + "HHI", t, typ, cnt) + raw.ljust(4, b"\0")
        else:
            ifd += struct.pack(bo + "HHII", t, typ, cnt, data_off + len(extra))
            extra += raw
            if len(extra) % 2:
                extra += b"\0"
    ifd += b"\0\0\0\0"
    body += ifd + extra
    body[4:8] = struct.pack(bo + "I", ifd_off)
    return bytes(body)


@pytest.mark.parametrize("compression", [1, 5, 8, 32773])
@pytest.mark.parametrize("predictor", [1, 2])
@pytest.mark.parametrize("bo", ["<", ">"])
def test_tiff_rgb8_compressions(compression, predictor, bo):
    rng = np.random.default_rng(compression + predictor)
    img = np.clip(test_image(37, 53, seed=4).astype(int) + rng.integers(-3, 4, (37, 53, 3)), 0, 255).astype(np.uint8)
    data = write_tiff(img, bo, compression, predictor, rows_per_strip=8)
    got = A.decode_tiff(data)
    assert got.dtype == np.float32
    assert np.array_equal(got, img.astype(np.float32) / np.float32(255.0))


def test_tiff_lzw_table_resets():
    rng = np.random.default_rng(2)
    img = rng.integers(0, 256, (64, 96, 3), dtype=np.uint8)  # incompressible: the table fills and clears
    data = write_tiff(img, compression=5)
    assert np.array_equal(A.decode_tiff(data), img.astype(np.float32) / np.float32(255.0))


@pytest.mark.parametrize("layout", ["strips", "tiles", "planar", "planar_tiles"])
def test_tiff_layouts_rgba16(layout):
    rng = np.random.default_rng(7)
    img = rng.integers(0, 65536, (45, 50, 4), dtype=np.uint16)
    kw = {"strips": dict(rows_per_strip=7), "tiles": dict(tile=(16, 16)), "planar": dict(planar=2, rows_per_strip=9),
          "planar_tiles": dict(planar=2, tile=(32, 16))}[layout]
    for compression, predictor in ((1, 1), (5, 2), (8, 2)):
        data = write_tiff(img, ">", compression, predictor, **kw)
        got = A.decode_tiff(data)
        assert np.array_equal(got, img[..., :3].astype(np.float32) / np.float32(65535.0))


def test_tiff_grey_palette_bilevel_float():
    rng = np.random.default_rng(8)
    g = rng.integers(0, 256, (19, 23, 1), dtype=np.uint8)
    assert np.array_equal(A.decode_tiff(write_tiff(g, compression=5, predictor=2)),
                          np.repeat(g.astype(np.float32) / np.float32(255.0), 3, -1))
    # WhiteIsZero inverts
    assert np.array_equal(A.decode_tiff(write_tiff(g, photometric=0)),
                          np.repeat((255 - g).astype(np.float32) / np.float32(255.0), 3, -1))
    # 4-bit palette
    idx = rng.integers(0, 16, (11, 13, 1), dtype=np.uint8)
    cmap = rng.integers(0, 65536, (16, 3), dtype=np.uint16)
    got = A.decode_tiff(write_tiff(idx, photometric=3, colormap=cmap, bps=4, compression=32773))
    assert np.array_equal(got, cmap[idx[..., 0]].astype(np.float32) / np.float32(65535.0))
    # 1-bit grey expands to 0 / 255 like the PNG path
    bl = rng.integers(0, 2, (9, 21, 1), dtype=np.uint8)
    got = A.decode_tiff(write_tiff(bl, bps=1))
    assert np.array_equal(got, np.repeat(bl.astype(np.float32) * 255 / np.float32(255.0), 3, -1))
    # float32 RGB, plain and with the floating-point predictor
    f = rng.normal(1.0, 3.0, (14, 17, 3)).astype(np.float32)
    for predictor, compression in ((1, 1), (3, 8), (3, 5)):
        got = A.decode_tiff(write_tiff(f, ">", compression, predictor, fmt=3))
        assert np.array_equal(got, f)


def test_tiff_errors():
    img = np.zeros((4, 4, 3), np.uint8)
    good = write_tiff(img)
    with pytest.raises(VoidrayError):
        A.decode_tiff(b"II*\0" + b"\xff\xff\xff\x7f")
    with pytest.raises(VoidrayError) as e:
        A.decode_tiff(write_tiff(img, compression=7))  # JPEG-in-TIFF
    assert e.value.status == 2
    with pytest.raises(VoidrayError) as e:
        A.decode_tiff(write_tiff(img, photometric=5))  # CMYK
    assert e.value.status == 2
    with pytest.raises(VoidrayError):
        A.decode_tiff(good[:20])
    with pytest.raises(VoidrayError):
        A.decode_tiff(write_tiff(img, compression=5)[:12] + b"\xff" * 40)


def test_tiff_corrupt_files_raise_voidray_errors_only():
    rng = np.random.default_rng(6)
    img = rng.integers(0, 256, (20, 24, 3), dtype=np.uint8)
    seeds = [write_tiff(img, compression=c, predictor=p, rows_per_strip=5) for c in (1, 5, 8, 32773) for p in (1, 2)]
    seeds.append(write_tiff(rng.integers(0, 65536, (13, 17, 4), dtype=np.uint16), ">", 5, 2, tile=(16, 16), planar=2))
    seeds.append(write_tiff(rng.normal(0, 1, (9, 10, 3)).astype(np.float32), ">", 8, 3, fmt=3))
    for it in range(1500):
        b = bytearray(seeds[it % len(seeds)])
        for _ in range(rng.integers(1, 6)):
            b[int(rng.integers(4, len(b)))] = int(rng.integers(0, 256))
        try:
            A.decode_tiff(bytes(b))
        except VoidrayError as e:
            assert e.status in (1, 2)


@pytest.mark.skipif(not (ASSETS / "wood_albedo.tif").exists(), reason="the reference's assets are not here")
def test_tiff_reference_assets():
    alb = A.load_image_rgb32f(str(ASSETS / "wood_albedo.tif"))
    nrm = A.load_image_rgb32f(str(ASSETS / "wood_normal.tif"))
    hgt = A.load_image_rgb32f(str(ASSETS / "wood_height.tif"))
    for img in (alb, nrm, hgt):
        assert img.shape == (512, 512, 3) and img.dtype == np.float32
    # a tangent-space normal map points along +z on average; the height map is grey
    m = nrm.reshape(-1, 3).mean(0)
    assert abs(m[0] - 0.5) < 0.02 and abs(m[1] - 0.5) < 0.02 and m[2] > 0.95
    assert np.array_equal(hgt[..., 0], hgt[..., 2])
    # LZW + horizontal predictor decode to whole 8-bit levels
    assert np.array_equal(np.round(alb * 255), alb * np.float32(255.0))


def tiff_lzw_decode_restated(src: bytes) -> bytes:
    """TIFF 6.0 LZW decoded code by code in Python (the library's decoder is
    native): MSB-first codes of 9-12 bits, Clear = 256, EOI = 257, the code
    width growing one code early (at 511, 1023 and 2047 table entries)."""
    out = bytearray()
    table = [bytes((i,)) for i in range(256)] + [b"", b""]
    total = len(src) * 8
    padded = src + b"\0\0\0"
    nbits, pos, prev = 9, 0, b""
    while pos + nbits <= total:
        b = pos >> 3
        word = (padded[b] << 16) | (padded[b + 1] << 8) | padded[b + 2]
        code = (word >> (24 - (pos & 7) - nbits)) & ((1 << nbits) - 1)
        pos += nbits
        if code == 257:
            break
        if code == 256:
            del table[258:]
            nbits, prev = 9, b""
            continue
        if code < len(table) and code < 256 or code >= 258 and code < len(table):
            entry = table[code]
            if prev:
                table.append(prev + entry[:1])
        elif code == len(table) and prev:
            entry = prev + prev[:1]
            table.append(entry)
        else:
            raise VoidrayError(1, f"TIFF: corrupt LZW data (code {code} with {len(table)} table entries)")
        out += entry
        prev = entry
        if len(table) >= (1 << nbits) - 1 and nbits < 12:
            nbits += 1
    return bytes(out)


def test_native_lzw_matches_the_restatement():
    """vr_tiff_lzw_decode against the Python restatement: streams from the
    encoder here (table resets included), truncated streams, and mutated
    ones, which both decode to the same bytes or both reject."""
    rng = np.random.default_rng(31)
    streams = []
    for n in (1, 100, 5000, 40000):
        raw = bytes(rng.integers(0, 256, n, dtype=np.uint8)) if n % 2 else bytes(
            np.cumsum(rng.integers(0, 3, n)).astype(np.uint8))
        enc = lzw_encode(raw)
        assert A._tiff_lzw_decode(enc, len(raw)) == raw == tiff_lzw_decode_restated(enc)
        streams += [enc, enc[:len(enc) // 2]]
    for it in range(600):
        b = bytearray(streams[it % len(streams)])
        for _ in range(rng.integers(0, 4)):
            b[int(rng.integers(0, len(b)))] = int(rng.integers(0, 256))
        b = bytes(b)
        try:
            want = tiff_lzw_decode_restated(b)
        except VoidrayError:
            with pytest.raises(VoidrayError, match="corrupt LZW"):
                A._tiff_lzw_decode(b, 1 << 16)
            continue
        assert A._tiff_lzw_decode(b, len(want) + 5) == want
        assert A._tiff_lzw_decode(b, len(want) // 2) == want[:len(want) // 2]
