// vr_image.cpp — host-side JPEG decoding for textures and environments.
//
// voidray loads textures with `image::open(path).to_rgb32f()`
// (voidray_renderer/src/core/texture.rs:36-37; image 0.24, whose JPEG support
// is the jpeg-decoder crate).  The reference's demo scenes ship their albedo
// maps as JPEG (voidray_app/src/examples/mushroom.rs:9-17, assets/*.jpg).
// This file decodes ITU-T T.81 Huffman-coded DCT JPEG — baseline, extended
// sequential and progressive, 8-bit samples, 1/3/4 components, any sampling
// factors, restart intervals — to interleaved RGB8; the Python layer divides
// by 255 as to_rgb32f does.
//
// The steps follow the standard: marker parsing (B.2), canonical Huffman
// tables (C, F.2.2.3), sequential decoding (F.2.2), progressive DC/AC first
// and refinement scans (G.1.2), dequantisation and the 8x8 inverse DCT (A.3.3,
// computed in float from its definition), then the JFIF YCbCr -> RGB matrix.
// Chroma upsampling is IJG's "fancy" triangle filter for 2x1 and 2x2 factors
// and replication otherwise; Adobe APP14 transform flags select RGB, YCbCr,
// CMYK and YCCK.  The float IDCT and the upsampling filter can differ from
// jpeg-decoder's fixed-point ones by about one level out of 255.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <future>
#include <new>
#include <stdexcept>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "../../include/voidray_assets.h"

namespace vr {
// The C ABI's thread-local error message (vr_capi.cu); returns s.
vr_status set_error(vr_status s, const std::string& message);
}  // namespace vr

namespace {

constexpr uint8_t kZigzag[64] = {
    0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,  12, 19, 26, 33, 40, 48,
    41, 34, 27, 20, 13, 6,  7,  14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23,
    30, 37, 44, 51, 58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

constexpr uint64_t kMaxPixels = 1ull << 28;
constexpr int kFastBits = 9;

struct JpegError {
    vr_status status;
    std::string message;
};

[[noreturn]] void fail(vr_status s, const std::string& m) { throw JpegError{s, m}; }

// Canonical Huffman table (T.81 C.2 / F.2.2.3) with a 9-bit lookup.
struct Huffman {
    bool defined = false;
    uint16_t fast[1 << kFastBits];  // (length << 8) | symbol, 0 = longer than kFastBits
    int32_t maxcode[18];            // largest code of each length, -1 if none
    int32_t valptr[17];             // index of the first symbol of each length
    int32_t mincode[17];
    uint8_t vals[256];

    void build(const uint8_t counts[16], const uint8_t* symbols, int total) {
        std::memcpy(vals, symbols, total);
        std::memset(fast, 0, sizeof(fast));
        int code = 0, k = 0;
        for (int len = 1; len <= 16; ++len) {
            valptr[len] = k;
            mincode[len] = code;
            for (int i = 0; i < counts[len - 1]; ++i, ++k, ++code) {
                // checked before the code is used: an over-subscribed table has no valid codes
                if (code >= (1 << len)) fail(VR_ERR_INVALID, "JPEG: Huffman table over-subscribed");
                if (len <= kFastBits) {
                    const int shift = kFastBits - len;
                    for (int j = 0; j < (1 << shift); ++j)
                        fast[(code << shift) | j] = uint16_t((len << 8) | symbols[k]);
                }
            }
            maxcode[len] = counts[len - 1] ? code - 1 : -1;
            code <<= 1;
        }
        maxcode[17] = 0x7fffffff;  // sentinel: lengths above 16 are corrupt data
        defined = true;
    }
};

// Entropy-coded segment reader: removes stuffed zero bytes, stops at markers
// and feeds zero bits after them (or after the end of the data).
struct BitReader {
    const uint8_t* p = nullptr;
    const uint8_t* end = nullptr;
    uint64_t acc = 0;
    int bits = 0;      // bits in acc
    int real = 0;      // of those, bits that came from the data
    bool at_marker = false;
    bool overrun = false;

    void reset(const uint8_t* start, const uint8_t* stop) {
        p = start;
        end = stop;
        acc = 0;
        bits = real = 0;
        at_marker = false;
    }
    void fill() {
        while (bits <= 56) {
            uint64_t b = 0;
            if (!at_marker && p < end) {
                if (*p == 0xFF) {
                    if (p + 1 < end && p[1] == 0x00) {
                        b = 0xFF;
                        p += 2;
                        real += 8;
                    } else {
                        at_marker = true;
                    }
                } else {
                    b = *p++;
                    real += 8;
                }
            }
            acc |= b << (56 - bits);
            bits += 8;
        }
    }
    void consume(int n) {
        acc <<= n;
        bits -= n;
        if (n > real) overrun = true;
        real = n > real ? 0 : real - n;
    }
    uint32_t get(int n) {  // n in 0..16
        if (n == 0) return 0;
        fill();
        const uint32_t v = uint32_t(acc >> (64 - n));
        consume(n);
        return v;
    }
    int bit() { return int(get(1)); }
    int decode(const Huffman& h) {
        fill();
        const uint16_t f = h.fast[acc >> (64 - kFastBits)];
        if (f) {
            consume(f >> 8);
            return f & 0xff;
        }
        int len = kFastBits + 1;
        int32_t code = int32_t(acc >> (64 - len));
        while (code > h.maxcode[len]) {
            ++len;
            if (len > 16) fail(VR_ERR_INVALID, "JPEG: invalid Huffman code");
            code = int32_t(acc >> (64 - len));
        }
        consume(len);
        return h.vals[h.valptr[len] + code - h.mincode[len]];
    }
    // T.81 F.2.2.1 EXTEND of an s-bit magnitude category.
    int receive_extend(int s) {
        if (s == 0) return 0;
        if (s > 16) fail(VR_ERR_INVALID, "JPEG: coefficient category above 16");
        const int v = int(get(s));
        return v < (1 << (s - 1)) ? v - (1 << s) + 1 : v;
    }
};

struct Component {
    int id = 0, h = 1, v = 1, tq = 0;
    int bw = 0, bh = 0;        // blocks per line / column, padded to whole MCUs
    int cw = 0, ch = 0;        // component size in samples
    std::vector<int16_t> coef;  // bw * bh * 64, natural order
    uint16_t q[64] = {};        // latched at the component's first scan
    bool scanned = false;
};

// Runs body(begin, end) over [0, n) in pieces on the host's threads (one
// piece below `grain` items).  The bodies write disjoint outputs.
template <class F>
void parallel_for(size_t n, size_t grain, F&& body) {
    unsigned hw = std::thread::hardware_concurrency();
    const size_t pieces = std::max<size_t>(1, std::min<size_t>(hw ? hw : 1, n / std::max<size_t>(grain, 1)));
    std::vector<std::future<void>> tasks;
    for (size_t k = 1; k < pieces; ++k) {
        const size_t lo = n * k / pieces, hi = n * (k + 1) / pieces;
        try {
            tasks.push_back(std::async(std::launch::async, [&body, lo, hi] { body(lo, hi); }));
        } catch (const std::system_error&) {
            body(lo, hi);
        }
    }
    body(0, n / pieces);
    for (auto& t : tasks) t.get();
}

// Entropy-decoding state that a restart marker resets: the DC predictions of
// the scan's components and the end-of-band run.
struct ScanState {
    int eobrun = 0;
    int dc_pred[4] = {0, 0, 0, 0};
};

struct Decoder {
    const uint8_t* data;
    size_t size;
    size_t pos = 0;

    uint16_t qt[4][64] = {};
    bool qt_defined[4] = {};
    Huffman dc[4], ac[4];
    std::vector<Component> comps;
    int width = 0, height = 0, precision = 8;
    bool frame = false, progressive = false;
    int hmax = 1, vmax = 1, mcux = 0, mcuy = 0;
    int restart_interval = 0;
    bool jfif = false, adobe = false;
    int adobe_transform = -1;
    bool header_only = false;

    Decoder(const uint8_t* d, size_t n) : data(d), size(n) {}

    uint8_t u8() {
        if (pos >= size) fail(VR_ERR_INVALID, "JPEG: unexpected end of data");
        return data[pos++];
    }
    uint16_t u16() {
        const int a = u8();
        return uint16_t((a << 8) | u8());
    }

    void run() {
        if (size < 4 || data[0] != 0xFF || data[1] != 0xD8) fail(VR_ERR_INVALID, "not a JPEG stream (no SOI)");
        pos = 2;
        for (;;) {
            // markers may be preceded by any number of 0xFF fill bytes
            uint8_t b = u8();
            if (b != 0xFF) fail(VR_ERR_INVALID, "JPEG: marker expected");
            uint8_t m = u8();
            while (m == 0xFF) m = u8();
            if (m == 0xD9) break;  // EOI
            if (m >= 0xD0 && m <= 0xD7) continue;
            if (m == 0x01) continue;  // TEM
            const size_t seg_start = pos;
            const int len = u16();
            if (len < 2 || seg_start + len > size) fail(VR_ERR_INVALID, "JPEG: segment length out of range");
            const size_t seg_end = seg_start + len;
            switch (m) {
                case 0xC0: case 0xC1: case 0xC2:
                    sof(m, seg_end);
                    if (header_only) return;
                    break;
                case 0xC3: case 0xC5: case 0xC6: case 0xC7:
                case 0xC9: case 0xCA: case 0xCB: case 0xCD: case 0xCE: case 0xCF:
                    fail(VR_ERR_UNSUPPORTED, "JPEG: lossless, hierarchical and arithmetic-coded frames are not decoded");
                case 0xC4: dht(seg_end); break;
                case 0xDB: dqt(seg_end); break;
                case 0xDD:
                    if (len != 4) fail(VR_ERR_INVALID, "JPEG: DRI length");
                    restart_interval = u16();
                    break;
                case 0xDA: sos(seg_end); break;
                case 0xDC: fail(VR_ERR_UNSUPPORTED, "JPEG: DNL marker (height defined after the first scan)");
                case 0xE0:
                    if (len >= 7 && std::memcmp(data + pos, "JFIF\0", 5) == 0) jfif = true;
                    break;
                case 0xEE:
                    if (len >= 14 && std::memcmp(data + pos, "Adobe", 5) == 0) {
                        adobe = true;
                        adobe_transform = data[pos + 11];
                    }
                    break;
                default: break;  // APPn, COM and others carry nothing the pixels need
            }
            if (m != 0xDA) pos = seg_end;
        }
        if (!frame) fail(VR_ERR_INVALID, "JPEG: no frame header");
        for (const Component& c : comps)
            if (!c.scanned) fail(VR_ERR_INVALID, "JPEG: a component has no scan");
    }

    void sof(uint8_t m, size_t seg_end) {
        if (frame) fail(VR_ERR_UNSUPPORTED, "JPEG: more than one frame");
        frame = true;
        progressive = m == 0xC2;
        precision = u8();
        height = u16();
        width = u16();
        const int nf = u8();
        if (precision != 8) fail(VR_ERR_UNSUPPORTED, "JPEG: only 8-bit samples are decoded");
        if (height == 0) fail(VR_ERR_UNSUPPORTED, "JPEG: height defined by a DNL marker");
        if (width == 0) fail(VR_ERR_INVALID, "JPEG: zero width");
        if (uint64_t(width) * height > kMaxPixels) fail(VR_ERR_UNSUPPORTED, "JPEG: image larger than 2^28 pixels");
        if (nf != 1 && nf != 3 && nf != 4) fail(VR_ERR_UNSUPPORTED, "JPEG: only 1, 3 or 4 components are decoded");
        if (pos + 3 * size_t(nf) > seg_end) fail(VR_ERR_INVALID, "JPEG: SOF segment too short");
        comps.resize(nf);
        for (Component& c : comps) {
            c.id = u8();
            const int hv = u8();
            c.h = hv >> 4;
            c.v = hv & 15;
            c.tq = u8();
            if (c.h < 1 || c.h > 4 || c.v < 1 || c.v > 4 || c.tq > 3)
                fail(VR_ERR_INVALID, "JPEG: sampling factor or quantisation table out of range");
            hmax = std::max(hmax, c.h);
            vmax = std::max(vmax, c.v);
        }
        for (int i = 0; i < nf; ++i)
            for (int j = 0; j < i; ++j)
                if (comps[i].id == comps[j].id) fail(VR_ERR_INVALID, "JPEG: duplicate component id");
        mcux = (width + 8 * hmax - 1) / (8 * hmax);
        mcuy = (height + 8 * vmax - 1) / (8 * vmax);
        if (header_only) return;
        for (Component& c : comps) {
            c.bw = mcux * c.h;
            c.bh = mcuy * c.v;
            c.cw = (width * c.h + hmax - 1) / hmax;
            c.ch = (height * c.v + vmax - 1) / vmax;
            c.coef.assign(size_t(c.bw) * c.bh * 64, 0);
        }
    }

    void dht(size_t seg_end) {
        while (pos < seg_end) {
            const int tc_th = u8();
            const int tc = tc_th >> 4, th = tc_th & 15;
            if (tc > 1 || th > 3) fail(VR_ERR_INVALID, "JPEG: Huffman table class or id out of range");
            uint8_t counts[16];
            int total = 0;
            for (int i = 0; i < 16; ++i) total += counts[i] = u8();
            if (total > 256 || pos + total > seg_end) fail(VR_ERR_INVALID, "JPEG: Huffman table too long");
            (tc ? ac : dc)[th].build(counts, data + pos, total);
            pos += total;
        }
    }

    void dqt(size_t seg_end) {
        while (pos < seg_end) {
            const int pq_tq = u8();
            const int pq = pq_tq >> 4, tq = pq_tq & 15;
            if (pq > 1 || tq > 3) fail(VR_ERR_INVALID, "JPEG: quantisation table precision or id out of range");
            for (int i = 0; i < 64; ++i) qt[tq][kZigzag[i]] = pq ? u16() : u8();
            qt_defined[tq] = true;
        }
    }

    void sos(size_t seg_end) {
        if (!frame) fail(VR_ERR_INVALID, "JPEG: scan before the frame header");
        const int ns = u8();
        if (ns < 1 || ns > 4 || pos + 2 * size_t(ns) + 3 != seg_end) fail(VR_ERR_INVALID, "JPEG: SOS segment length");
        Component* sc[4];
        int td[4], ta[4];
        for (int i = 0; i < ns; ++i) {
            const int cs = u8(), t = u8();
            sc[i] = nullptr;
            for (Component& c : comps)
                if (c.id == cs) sc[i] = &c;
            if (!sc[i]) fail(VR_ERR_INVALID, "JPEG: scan names an unknown component");
            for (int j = 0; j < i; ++j)
                if (sc[j] == sc[i]) fail(VR_ERR_INVALID, "JPEG: scan names a component twice");
            td[i] = t >> 4;
            ta[i] = t & 15;
            if (td[i] > 3 || ta[i] > 3) fail(VR_ERR_INVALID, "JPEG: scan table id out of range");
        }
        const int ss = u8(), se = u8(), a = u8();
        const int ah = a >> 4, al = a & 15;
        if (progressive) {
            if (ss > se || se > 63 || (ss == 0 && se != 0) || ah > 13 || al > 13)
                fail(VR_ERR_INVALID, "JPEG: progressive scan parameters out of range");
            if (ss > 0 && ns != 1) fail(VR_ERR_INVALID, "JPEG: AC scan with more than one component");
        } else if (ss != 0 || se != 63 || a != 0) {
            fail(VR_ERR_INVALID, "JPEG: sequential scan parameters out of range");
        }
        if (ns > 1) {
            int blocks = 0;
            for (int i = 0; i < ns; ++i) blocks += sc[i]->h * sc[i]->v;
            if (blocks > 10) fail(VR_ERR_INVALID, "JPEG: more than 10 blocks per MCU");
        }
        for (int i = 0; i < ns; ++i) {
            Component& c = *sc[i];
            if (!c.scanned) {
                if (!qt_defined[c.tq]) fail(VR_ERR_INVALID, "JPEG: quantisation table not defined");
                std::memcpy(c.q, qt[c.tq], sizeof(c.q));
                c.scanned = true;
            }
            // sequential scans code DC and AC; progressive scans DC first, DC
            // refinement (raw bits) or AC bands
            const bool need_dc = ss == 0 && ah == 0;
            const bool need_ac = !progressive || ss > 0;
            if (need_dc && !dc[td[i]].defined) fail(VR_ERR_INVALID, "JPEG: DC Huffman table not defined");
            if (need_ac && !ac[ta[i]].defined) fail(VR_ERR_INVALID, "JPEG: AC Huffman table not defined");
        }
        pos = seg_end;
        decode_scan(ns, sc, td, ta, ss, se, ah, al);
    }

    // One block of one scan, by scan kind.
    void block(BitReader& br, ScanState& st, int slot, int16_t* blk, const Huffman& hd, const Huffman& ha, int ss,
               int se, int ah, int al) const {
        int& dc_pred = st.dc_pred[slot];
        int& eobrun = st.eobrun;
        if (!progressive) {
            const int t = br.decode(hd);
            dc_pred += br.receive_extend(t);
            blk[0] = int16_t(dc_pred);
            for (int k = 1; k < 64;) {
                const int rs = br.decode(ha);
                const int r = rs >> 4, s = rs & 15;
                if (s == 0) {
                    if (r != 15) break;
                    k += 16;
                    continue;
                }
                k += r;
                if (k > 63) fail(VR_ERR_INVALID, "JPEG: AC coefficient index past 63");
                blk[kZigzag[k]] = int16_t(br.receive_extend(s));
                ++k;
            }
            return;
        }
        if (ss == 0) {  // DC scans (G.1.2.1)
            if (ah == 0) {
                const int t = br.decode(hd);
                dc_pred += br.receive_extend(t);
                blk[0] = int16_t(dc_pred * (1 << al));
            } else if (br.bit()) {
                blk[0] = int16_t(blk[0] | (1 << al));
            }
            return;
        }
        if (ah == 0) {  // AC first scan (G.1.2.2)
            if (eobrun > 0) {
                --eobrun;
                return;
            }
            for (int k = ss; k <= se; ++k) {
                const int rs = br.decode(ha);
                const int r = rs >> 4, s = rs & 15;
                if (s == 0) {
                    if (r < 15) {
                        eobrun = (1 << r) - 1;
                        if (r) eobrun += int(br.get(r));
                        break;
                    }
                    k += 15;
                    continue;
                }
                k += r;
                if (k > 63) fail(VR_ERR_INVALID, "JPEG: AC coefficient index past 63");
                blk[kZigzag[k]] = int16_t(br.receive_extend(s) * (1 << al));
            }
            return;
        }
        // AC refinement scan (G.1.2.3): a correction bit for every coefficient
        // already non-zero, new coefficients of magnitude 1 << al.
        const int p1 = 1 << al, m1 = -(1 << al);
        int k = ss;
        if (eobrun == 0) {
            for (; k <= se; ++k) {
                const int rs = br.decode(ha);
                int r = rs >> 4;
                const int s = rs & 15;
                int val = 0;
                if (s) {
                    if (s != 1) fail(VR_ERR_INVALID, "JPEG: refinement coefficient of magnitude above 1");
                    val = br.bit() ? p1 : m1;
                } else if (r != 15) {
                    eobrun = 1 << r;
                    if (r) eobrun += int(br.get(r));
                    break;
                }
                for (; k <= se; ++k) {
                    int16_t& co = blk[kZigzag[k]];
                    if (co != 0) {
                        if (br.bit() && (co & p1) == 0) co = int16_t(co + (co >= 0 ? p1 : m1));
                    } else {
                        if (r == 0) {
                            if (val) co = int16_t(val);
                            break;
                        }
                        --r;
                    }
                }
            }
        }
        if (eobrun > 0) {
            for (; k <= se; ++k) {
                int16_t& co = blk[kZigzag[k]];
                if (co != 0 && br.bit() && (co & p1) == 0) co = int16_t(co + (co >= 0 ? p1 : m1));
            }
            --eobrun;
        }
    }

    // Decodes units [u0, u1) of a scan (MCUs of an interleaved scan, blocks of
    // a single-component one) from `br`; restart markers are not handled here.
    void decode_units(BitReader& br, ScanState& st, long u0, long u1, int ns, Component** sc, const int* td,
                      const int* ta, int ss, int se, int ah, int al) const {
        const int ux = (sc[0]->cw + 7) / 8;
        for (long u = u0; u < u1; ++u) {
            if (ns == 1) {
                Component& c = *sc[0];
                const long by = u / ux, bx = u % ux;
                block(br, st, 0, c.coef.data() + (size_t(by) * c.bw + bx) * 64, dc[td[0]], ac[ta[0]], ss, se, ah, al);
            } else {
                const long my = u / mcux, mx = u % mcux;
                for (int i = 0; i < ns; ++i) {
                    Component& c = *sc[i];
                    for (int v = 0; v < c.v; ++v)
                        for (int h = 0; h < c.h; ++h) {
                            const size_t by = size_t(my) * c.v + v, bx = size_t(mx) * c.h + h;
                            block(br, st, i, c.coef.data() + (by * c.bw + bx) * 64, dc[td[i]], ac[ta[i]], ss, se,
                                  ah, al);
                        }
                }
            }
            if (br.overrun) fail(VR_ERR_INVALID, "JPEG: entropy-coded data truncated");
        }
    }

    // With many restart intervals the intervals decode on separate threads:
    // each starts after its RST marker with fresh predictions, and writes its
    // own blocks.  Returns false, having decoded nothing, when the markers do
    // not split the scan into the expected intervals (the serial path then
    // reports what is wrong).
    bool decode_intervals_parallel(long units, int ns, Component** sc, const int* td, const int* ta, int ss, int se,
                                   int ah, int al) {
        const long R = restart_interval;
        const long intervals = (units + R - 1) / R;
        std::vector<const uint8_t*> seg{data + pos};
        const uint8_t* q = data + pos;
        const uint8_t* end = data + size;
        while (q + 1 < end) {
            if (q[0] != 0xFF) {
                ++q;
                continue;
            }
            const uint8_t m = q[1];
            if (m == 0x00) {
                q += 2;
            } else if (m == 0xFF) {
                ++q;  // fill byte
            } else if (m >= 0xD0 && m <= 0xD7) {
                seg.push_back(q + 2);
                q += 2;
            } else {
                break;  // the marker after the scan
            }
        }
        if (q + 1 >= end || (long)seg.size() < intervals) return false;
        std::vector<std::string> err(intervals);
        std::vector<vr_status> code(intervals, VR_OK);
        parallel_for(size_t(intervals), 4, [&](size_t k0, size_t k1) {
            for (size_t k = k0; k < k1; ++k) {
                try {
                    BitReader br;
                    br.reset(seg[k], end);
                    ScanState st;
                    decode_units(br, st, long(k) * R, std::min(units, long(k + 1) * R), ns, sc, td, ta, ss, se, ah,
                                 al);
                    // every byte of the interval consumed: its RST marker is next
                    br.fill();
                    if (long(k) + 1 < intervals && !br.at_marker) fail(VR_ERR_INVALID, "JPEG: restart marker missing");
                } catch (const JpegError& e) {
                    code[k] = e.status;
                    err[k] = e.message;
                }
            }
        });
        for (long k = 0; k < intervals; ++k)
            if (code[k] != VR_OK) fail(code[k], err[k]);
        pos = size_t(q - data);
        return true;
    }

    void decode_scan(int ns, Component** sc, const int* td, const int* ta, int ss, int se, int ah, int al) {
        long units;  // MCUs of an interleaved scan, blocks of a single-component one
        if (ns == 1) {
            units = long((sc[0]->cw + 7) / 8) * ((sc[0]->ch + 7) / 8);
        } else {
            units = long(mcux) * mcuy;
        }
        if (restart_interval && (units + restart_interval - 1) / restart_interval >= 8 &&
            decode_intervals_parallel(units, ns, sc, td, ta, ss, se, ah, al))
            return;
        BitReader br;
        br.reset(data + pos, data + size);
        ScanState st;
        for (long u = 0; u < units;) {
            if (restart_interval && u > 0 && u % restart_interval == 0) {
                // byte-align, expect RSTn, reset predictions and the EOB run
                br.fill();
                const uint8_t* mp = br.p;
                while (br.at_marker && mp + 2 < br.end && mp[1] == 0xFF) ++mp;  // fill bytes
                if (!br.at_marker || mp + 1 >= br.end || mp[1] < 0xD0 || mp[1] > 0xD7)
                    fail(VR_ERR_INVALID, "JPEG: restart marker missing");
                br.reset(mp + 2, data + size);
                st = ScanState();
            }
            const long u1 = restart_interval ? std::min(units, (u / restart_interval + 1) * restart_interval) : units;
            decode_units(br, st, u, u1, ns, sc, td, ta, ss, se, ah, al);
            u = u1;
        }
        // continue at the next marker after the scan's data
        const uint8_t* q = br.p;
        while (q + 1 < data + size && !(q[0] == 0xFF && q[1] != 0x00 && !(q[1] >= 0xD0 && q[1] <= 0xD7))) ++q;
        if (q + 1 >= data + size) fail(VR_ERR_INVALID, "JPEG: no marker after the scan (missing EOI)");
        pos = size_t(q - data);
    }
};

// Inverse DCT of one dequantised block (A.3.3), float, level shift, rounding.
struct Idct {
    float c[8][8];  // c[u][x] = C(u)/2 cos((2x+1)u pi/16)
    Idct() {
        for (int u = 0; u < 8; ++u)
            for (int x = 0; x < 8; ++x)
                c[u][x] = float((u == 0 ? std::sqrt(0.5) : 1.0) * 0.5 * std::cos((2 * x + 1) * u * M_PI / 16.0));
    }
    static uint8_t clamp_round(float v) {
        const float r = std::floor(v + 128.5f);
        return uint8_t(r < 0.f ? 0.f : (r > 255.f ? 255.f : r));
    }
    void run(const int16_t* co, const uint16_t* q, uint8_t* out, int stride) const {
        float f[64];
        bool ac = false;
        for (int i = 0; i < 64; ++i) {
            f[i] = float(int32_t(co[i]) * int32_t(q[i]));
            if (i && co[i]) ac = true;
        }
        if (!ac) {
            const uint8_t v = clamp_round(f[0] * c[0][0] * c[0][0]);
            for (int y = 0; y < 8; ++y) std::memset(out + size_t(y) * stride, v, 8);
            return;
        }
        float t[64];  // rows: t[v][x] = sum_u c[u][x] f[v][u]
        for (int v = 0; v < 8; ++v)
            for (int x = 0; x < 8; ++x) {
                float s = 0.f;
                for (int u = 0; u < 8; ++u) s += c[u][x] * f[v * 8 + u];
                t[v * 8 + x] = s;
            }
        for (int y = 0; y < 8; ++y)
            for (int x = 0; x < 8; ++x) {
                float s = 0.f;
                for (int v = 0; v < 8; ++v) s += c[v][y] * t[v * 8 + x];
                out[size_t(y) * stride + x] = clamp_round(s);
            }
    }
};

// Component plane -> full-resolution plane (row-major, width x height).
void upsample(const Component& c, const std::vector<uint8_t>& plane, int hmax, int vmax, int width, int height,
              std::vector<uint8_t>& out) {
    const int pw = c.bw * 8;
    out.resize(size_t(width) * height);
    const int fx = hmax / c.h, fy = vmax / c.v;
    const bool integral = hmax % c.h == 0 && vmax % c.v == 0;
    if (fx == 1 && fy == 1 && integral) {
        for (int y = 0; y < height; ++y) std::memcpy(&out[size_t(y) * width], &plane[size_t(y) * pw], width);
        return;
    }
    const int cw = c.cw, ch = c.ch;
    if (integral && fx == 2 && (fy == 1 || fy == 2)) {
        // IJG fancy upsampling: a triangle filter, 3/4 nearer sample + 1/4 farther one.
        std::vector<int> col(cw);
        std::vector<uint8_t> row(size_t(2) * cw);
        for (int y = 0; y < height; ++y) {
            const int sy = y / fy;
            if (fy == 1) {
                const uint8_t* in = &plane[size_t(sy) * pw];
                if (cw == 1) {
                    row[0] = row[1] = in[0];
                } else {
                    row[0] = in[0];
                    row[1] = uint8_t((in[0] * 3 + in[1] + 2) >> 2);
                    for (int i = 1; i < cw - 1; ++i) {
                        row[2 * i] = uint8_t((in[i] * 3 + in[i - 1] + 1) >> 2);
                        row[2 * i + 1] = uint8_t((in[i] * 3 + in[i + 1] + 2) >> 2);
                    }
                    row[2 * cw - 2] = uint8_t((in[cw - 1] * 3 + in[cw - 2] + 1) >> 2);
                    row[2 * cw - 1] = in[cw - 1];
                }
            } else {
                // the nearer neighbouring row: above for even output rows, below for odd
                const int ny = (y & 1) ? std::min(sy + 1, ch - 1) : std::max(sy - 1, 0);
                const uint8_t* in0 = &plane[size_t(sy) * pw];
                const uint8_t* in1 = &plane[size_t(ny) * pw];
                for (int i = 0; i < cw; ++i) col[i] = in0[i] * 3 + in1[i];
                if (cw == 1) {
                    row[0] = row[1] = uint8_t((col[0] * 4 + 8) >> 4);
                } else {
                    row[0] = uint8_t((col[0] * 4 + 8) >> 4);
                    row[1] = uint8_t((col[0] * 3 + col[1] + 7) >> 4);
                    for (int i = 1; i < cw - 1; ++i) {
                        row[2 * i] = uint8_t((col[i] * 3 + col[i - 1] + 8) >> 4);
                        row[2 * i + 1] = uint8_t((col[i] * 3 + col[i + 1] + 7) >> 4);
                    }
                    row[2 * cw - 2] = uint8_t((col[cw - 1] * 3 + col[cw - 2] + 8) >> 4);
                    row[2 * cw - 1] = uint8_t((col[cw - 1] * 4 + 7) >> 4);
                }
            }
            std::memcpy(&out[size_t(y) * width], row.data(), width);
        }
        return;
    }
    // any other ratio: replicate the sample covering each output pixel
    for (int y = 0; y < height; ++y) {
        const int sy = std::min(int(int64_t(y) * c.v / vmax), ch - 1);
        for (int x = 0; x < width; ++x) {
            const int sx = std::min(int(int64_t(x) * c.h / hmax), cw - 1);
            out[size_t(y) * width + x] = plane[size_t(sy) * pw + sx];
        }
    }
}

uint8_t clamp_u8(float v) {
    const float r = std::floor(v + 0.5f);
    return uint8_t(r < 0.f ? 0.f : (r > 255.f ? 255.f : r));
}

// JFIF YCbCr -> RGB (CCIR 601 matrix as JFIF 1.02 states it).
void ycc_to_rgb(uint8_t y, uint8_t cb, uint8_t cr, uint8_t* rgb) {
    const float Y = y, Cb = float(cb) - 128.f, Cr = float(cr) - 128.f;
    rgb[0] = clamp_u8(Y + 1.402f * Cr);
    rgb[1] = clamp_u8(Y - 0.344136f * Cb - 0.714136f * Cr);
    rgb[2] = clamp_u8(Y + 1.772f * Cb);
}

void decode_pixels(Decoder& d, uint8_t* rgb) {
    static const Idct idct;
    const size_t n = size_t(d.width) * d.height;
    std::vector<std::vector<uint8_t>> full(d.comps.size());
    std::vector<uint8_t> plane;
    for (size_t ci = 0; ci < d.comps.size(); ++ci) {
        const Component& c = d.comps[ci];
        const int pw = c.bw * 8;
        // only the blocks that cover the component's samples are transformed
        const int bw_used = std::min(c.bw, (c.cw + 7) / 8), bh_used = std::min(c.bh, (c.ch + 7) / 8);
        plane.assign(size_t(pw) * c.bh * 8, 0);
        parallel_for(size_t(bh_used), 16, [&](size_t by0, size_t by1) {
            for (size_t by = by0; by < by1; ++by)
                for (int bx = 0; bx < bw_used; ++bx)
                    idct.run(&c.coef[(by * c.bw + bx) * 64], c.q, &plane[by * 8 * pw + size_t(bx) * 8], pw);
        });
        upsample(c, plane, d.hmax, d.vmax, d.width, d.height, full[ci]);
    }
    const size_t nc = d.comps.size();
    if (nc == 1) {
        for (size_t i = 0; i < n; ++i) rgb[3 * i] = rgb[3 * i + 1] = rgb[3 * i + 2] = full[0][i];
        return;
    }
    if (nc == 3) {
        bool is_rgb;
        if (d.adobe) is_rgb = d.adobe_transform == 0;
        else is_rgb = !d.jfif && d.comps[0].id == 'R' && d.comps[1].id == 'G' && d.comps[2].id == 'B';
        parallel_for(n, 1 << 16, [&](size_t i0, size_t i1) {
            for (size_t i = i0; i < i1; ++i) {
                if (is_rgb) {
                    rgb[3 * i] = full[0][i];
                    rgb[3 * i + 1] = full[1][i];
                    rgb[3 * i + 2] = full[2][i];
                } else {
                    ycc_to_rgb(full[0][i], full[1][i], full[2][i], rgb + 3 * i);
                }
            }
        });
        return;
    }
    // four components: Adobe CMYK (transform 0) or YCCK (transform 2), stored
    // inverted as Adobe writes them; R = C * K / 255 and so on.
    const bool ycck = d.adobe && d.adobe_transform == 2;
    for (size_t i = 0; i < n; ++i) {
        uint8_t cmy[3] = {full[0][i], full[1][i], full[2][i]};
        if (ycck) {
            uint8_t t[3];
            ycc_to_rgb(cmy[0], cmy[1], cmy[2], t);
            for (int k = 0; k < 3; ++k) cmy[k] = uint8_t(255 - t[k]);
        }
        const int k = full[3][i];
        for (int j = 0; j < 3; ++j) rgb[3 * i + j] = uint8_t((cmy[j] * k + 127) / 255);
    }
}

vr_status guarded(const char* what, const std::function<void()>& body) {
    try {
        body();
        return VR_OK;
    } catch (const JpegError& e) {
        return vr::set_error(e.status, e.message);
    } catch (const std::bad_alloc&) {
        return vr::set_error(VR_ERR_OOM, std::string(what) + ": host allocation failed");
    } catch (const std::exception& e) {
        return vr::set_error(VR_ERR_INVALID, std::string(what) + ": " + e.what());
    }
}
}  // namespace

extern "C" {

vr_status vr_png_unfilter(const uint8_t* data, size_t size, uint32_t rows, uint32_t stride, uint32_t bpp,
                          uint8_t* out) {
    if ((!data && size) || (!out && rows && stride) || bpp == 0)
        return vr::set_error(VR_ERR_INVALID, "vr_png_unfilter: null argument or zero byte distance");
    if ((uint64_t)rows * ((uint64_t)stride + 1) > size)
        return vr::set_error(VR_ERR_INVALID, "PNG: image data shorter than its scanlines");
    const uint8_t* in = data;
    const uint8_t* up = nullptr;  // previous output row, none above the first
    for (uint32_t y = 0; y < rows; ++y, in += stride + 1) {
        const uint8_t type = in[0];
        const uint8_t* line = in + 1;
        uint8_t* cur = out + (size_t)y * stride;
        for (uint32_t i = 0; i < stride; ++i) {
            const int a = i >= bpp ? cur[i - bpp] : 0;
            const int b = up ? up[i] : 0;
            const int c = (up && i >= bpp) ? up[i - bpp] : 0;
            int pred;
            switch (type) {
                case 0: pred = 0; break;
                case 1: pred = a; break;
                case 2: pred = b; break;
                case 3: pred = (a + b) >> 1; break;
                case 4: {  // Paeth: the neighbour nearest to a + b - c, ties to a then b
                    const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
                    pred = (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
                    break;
                }
                default:
                    return vr::set_error(VR_ERR_INVALID, "PNG: unknown filter type " + std::to_string(type));
            }
            cur[i] = (uint8_t)(line[i] + pred);
        }
        up = cur;
    }
    return VR_OK;
}

vr_status vr_tiff_lzw_decode(const uint8_t* src, size_t size, uint8_t* out, size_t capacity, size_t* length) {
    if ((!src && size) || (!out && capacity) || !length)
        return vr::set_error(VR_ERR_INVALID, "vr_tiff_lzw_decode: null argument");
    // table entries as (prefix code, last byte, first byte, length); codes
    // below 256 are single bytes, 256 and 257 are the control codes
    constexpr int kMax = 4096;
    static thread_local int16_t prefix[kMax];
    static thread_local uint8_t last[kMax], first[kMax];
    static thread_local uint16_t len[kMax];
    for (int c = 0; c < 256; ++c) {
        prefix[c] = -1;
        last[c] = first[c] = (uint8_t)c;
        len[c] = 1;
    }
    const uint64_t total = (uint64_t)size * 8;
    uint64_t pos = 0;
    int nbits = 9, next = 258, prev = -1;
    size_t w = 0;
    auto emit = [&](int code) {
        const size_t n = len[code];
        if (w < capacity) {
            // the entry's bytes from its end back along the prefix chain
            size_t k = n;
            for (int c = code; c >= 0; c = prefix[c]) {
                --k;
                if (w + k < capacity) out[w + k] = last[c];
            }
        }
        w += n;
    };
    while (pos + (uint64_t)nbits <= total) {
        // nbits (9-12) from the bit position, most significant bit first
        uint32_t word = 0;
        const size_t byte = (size_t)(pos >> 3);
        for (int k = 0; k < 3; ++k) word = (word << 8) | (byte + k < size ? src[byte + k] : 0u);
        const int code = (int)((word >> (24 - (int)(pos & 7) - nbits)) & ((1u << nbits) - 1));
        pos += (uint64_t)nbits;
        if (code == 257) break;
        if (code == 256) {
            next = 258;
            nbits = 9;
            prev = -1;
            continue;
        }
        if (code < next && (code < 256 || code >= 258)) {
            if (prev >= 0 && next < kMax) {
                prefix[next] = (int16_t)prev;
                last[next] = first[code];
                first[next] = first[prev];
                len[next] = (uint16_t)(len[prev] + 1);
                ++next;
            }
            emit(code);
            prev = code;
        } else if (code == next && prev >= 0 && next < kMax) {
            prefix[next] = (int16_t)prev;
            last[next] = first[prev];
            first[next] = first[prev];
            len[next] = (uint16_t)(len[prev] + 1);
            ++next;
            emit(code);
            prev = code;
        } else {
            return vr::set_error(VR_ERR_INVALID, "TIFF: corrupt LZW data (code " + std::to_string(code) + " with " +
                                                     std::to_string(next) + " table entries)");
        }
        if (next >= (1 << nbits) - 1 && nbits < 12) ++nbits;
    }
    *length = w;
    return VR_OK;
}

vr_status vr_image_info_get(const uint8_t* data, size_t size, vr_image_info* info) {
    if (!data || !info) return vr::set_error(VR_ERR_INVALID, "vr_image_info_get: null argument");
    return guarded("vr_image_info_get", [&] {
        Decoder d(data, size);
        d.header_only = true;
        d.run();
        if (!d.frame) fail(VR_ERR_INVALID, "JPEG: no frame header");
        info->width = uint32_t(d.width);
        info->height = uint32_t(d.height);
        info->components = uint32_t(d.comps.size());
        info->format = VR_IMAGE_JPEG;
        info->progressive = d.progressive ? 1u : 0u;
        info->reserved = 0;
    });
}

vr_status vr_image_decode_rgb8(const uint8_t* data, size_t size, uint8_t* rgb, size_t capacity) {
    if (!data || !rgb) return vr::set_error(VR_ERR_INVALID, "vr_image_decode_rgb8: null argument");
    return guarded("vr_image_decode_rgb8", [&] {
        Decoder d(data, size);
        d.run();
        const size_t need = size_t(d.width) * d.height * 3;
        if (capacity < need)
            fail(VR_ERR_INVALID, "vr_image_decode_rgb8: output holds " + std::to_string(capacity) + " bytes, the image needs " +
                                     std::to_string(need));
        decode_pixels(d, rgb);
    });
}

}  // extern "C"
