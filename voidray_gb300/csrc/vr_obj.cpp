// vr_obj.cpp — OBJ mesh parsing on the host (Mesh::from_file,
// voidray_renderer/src/core/mesh.rs:46-74, which loads with obj-rs 0.7.0 as
// `load_obj::<TexturedVertex, u32>`).  One pass over the text: positions,
// texture coordinates and normals collect as doubles, every face corner
// resolves its (position, normal, texture) triple to a vertex numbered in
// order of first use, and the vertex arrays are gathered at the end.
#include <charconv>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <new>
#include <stdexcept>
#include <string>
#include <system_error>
#include <vector>

#include "../../include/voidray_assets.h"

namespace vr {
// The C ABI's thread-local error message (vr_capi.cu); returns s.
vr_status set_error(vr_status s, const std::string& message);
}  // namespace vr

namespace {

struct ObjError {
    std::string message;
};

struct Token {
    const char* p;
    size_t n;
    std::string str() const { return std::string(p, n); }
};

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\v' || c == '\f' || c == '\r'; }

// A token quoted for messages: 'text'.
std::string quoted(const Token& t) { return "'" + t.str() + "'"; }

[[noreturn]] void fail(uint64_t line, const std::string& what) {
    throw ObjError{"OBJ line " + std::to_string(line) + ": " + what};
}

// Decimal (or inf / nan) to the nearest double; an optional leading '+'.
bool parse_double(const Token& t, double& out) {
    const char* b = t.p;
    const char* e = t.p + t.n;
    if (b < e && *b == '+' && b + 1 < e && *(b + 1) != '-' && *(b + 1) != '+') ++b;
    if (b == e) return false;
    auto r = std::from_chars(b, e, out);
    return r.ec == std::errc() && r.ptr == e;
}

// Resolves a 1-based or negative OBJ index against `count` entries.
uint32_t resolve(const Token& t, size_t count, const char* what, uint64_t line) {
    const char* b = t.p;
    const char* e = t.p + t.n;
    if (b < e && *b == '+') ++b;
    long long i = 0;
    auto r = std::from_chars(b, e, i);
    if (b == e || r.ptr != e || (r.ec != std::errc() && r.ec != std::errc::result_out_of_range))
        fail(line, std::string("bad ") + what + " index " + quoted(t));
    if (r.ec == std::errc::result_out_of_range)
        fail(line, std::string(what) + " index " + t.str() + " out of range (have " + std::to_string(count) + ")");
    const long long j = i < 0 ? (long long)count + i : i - 1;
    if (i == 0 || j < 0 || j >= (long long)count)
        fail(line, std::string(what) + " index " + std::to_string(i) + " out of range (have " + std::to_string(count) +
                       ")");
    return (uint32_t)j;
}

// Vertex numbering: an open-addressing table from (p, n, t) to the vertex
// id, linear probing, kept at most half full.
class TripleTable {
  public:
    TripleTable() : slots_(1024) {}
    // The id of (p, n, t), inserting `fresh` when the triple is new.
    uint32_t find_or_insert(uint32_t p, uint32_t n, uint32_t t, uint32_t fresh) {
        if (2 * (used_ + 1) > slots_.size()) grow();
        Slot* s = probe(p, n, t);
        if (s->id == kEmpty) {
            *s = Slot{p, n, t, fresh};
            ++used_;
        }
        return s->id;
    }

  private:
    static constexpr uint32_t kEmpty = UINT32_MAX;
    struct Slot {
        uint32_t p = 0, n = 0, t = 0, id = kEmpty;
    };
    static uint64_t mix(uint32_t p, uint32_t n, uint32_t t) {
        uint64_t h = (uint64_t)p * 0x9E3779B97F4A7C15ull;
        h ^= ((uint64_t)n + 0x632BE59BD9B4E019ull) * 0xC2B2AE3D27D4EB4Full;
        h ^= ((uint64_t)t + 0x165667B19E3779F9ull) * 0x27D4EB2F165667C5ull;
        return h ^ (h >> 31);
    }
    Slot* probe(uint32_t p, uint32_t n, uint32_t t) {
        const size_t mask = slots_.size() - 1;
        for (size_t i = mix(p, n, t) & mask;; i = (i + 1) & mask) {
            Slot& s = slots_[i];
            if (s.id == kEmpty || (s.p == p && s.n == n && s.t == t)) return &s;
        }
    }
    void grow() {
        std::vector<Slot> old(slots_.size() * 2);
        old.swap(slots_);
        for (const Slot& s : old)
            if (s.id != kEmpty) *probe(s.p, s.n, s.t) = s;
    }
    std::vector<Slot> slots_;
    size_t used_ = 0;
};

struct Parsed {
    std::vector<double> pos, tex, nrm;                // 3, 2, 3 per entry
    std::vector<uint32_t> order;                       // 3 per vertex: p, n, t
    std::vector<uint32_t> indices;
};

void parse(const char* text, size_t size, Parsed& out) {
    TripleTable vertices;
    std::vector<Token> tok;
    tok.reserve(8);
    uint64_t line = 0;
    size_t i = 0;
    while (i < size) {
        // one line: [i, end), then skip its terminator (\n, \r\n or \r)
        size_t end = i;
        while (end < size && text[end] != '\n' && text[end] != '\r') ++end;
        ++line;
        size_t next = end;
        if (next < size) next += (text[next] == '\r' && next + 1 < size && text[next + 1] == '\n') ? 2 : 1;
        // text after '#' is a comment
        size_t stop = i;
        while (stop < end && text[stop] != '#') ++stop;
        tok.clear();
        for (size_t k = i; k < stop;) {
            while (k < stop && is_space(text[k])) ++k;
            const size_t s0 = k;
            while (k < stop && !is_space(text[k])) ++k;
            if (k > s0) tok.push_back(Token{text + s0, k - s0});
        }
        const Token raw{text + i, end - i};
        i = next;
        if (tok.empty()) continue;
        const Token& key = tok[0];
        const size_t nargs = tok.size() - 1;
        auto number = [&](size_t a) {
            double v;
            if (!parse_double(tok[a], v)) {
                // the whole line, stripped, as the message shows it
                size_t b = 0, e = raw.n;
                while (b < e && (is_space(raw.p[b]))) ++b;
                while (e > b && (is_space(raw.p[e - 1]))) --e;
                fail(line, "cannot parse " + quoted(Token{raw.p + b, e - b}));
            }
            return v;
        };
        auto is = [&](const char* k) { return key.n == std::strlen(k) && std::memcmp(key.p, k, key.n) == 0; };
        if (is("v")) {
            if (nargs < 3) fail(line, "vertex needs 3 coordinates");
            for (int a = 1; a <= 3; ++a) out.pos.push_back(number(a));
        } else if (is("vt")) {
            if (nargs < 1) fail(line, "texture coordinate needs u");
            const double u = number(1);
            const double v = nargs > 1 ? number(2) : 0.0;
            out.tex.push_back(u);
            out.tex.push_back(v);
        } else if (is("vn")) {
            if (nargs < 3) fail(line, "normal needs 3 components");
            for (int a = 1; a <= 3; ++a) out.nrm.push_back(number(a));
        } else if (is("f")) {
            if (nargs != 3)
                fail(line, "face with " + std::to_string(nargs) + " corners (the model must be triangulated)");
            for (size_t c = 1; c <= 3; ++c) {
                const Token& t = tok[c];
                // p/t/n: exactly three parts, texture and normal present
                const char* s1 = (const char*)std::memchr(t.p, '/', t.n);
                const char* s2 = s1 ? (const char*)std::memchr(s1 + 1, '/', t.p + t.n - (s1 + 1)) : nullptr;
                const bool three = s2 && !std::memchr(s2 + 1, '/', t.p + t.n - (s2 + 1));
                if (!three || s2 == s1 + 1 || s2 + 1 == t.p + t.n)
                    fail(line, "face corner " + quoted(t) + " lacks texture or normal indices");
                const Token tp{t.p, (size_t)(s1 - t.p)}, tt{s1 + 1, (size_t)(s2 - s1 - 1)},
                    tn{s2 + 1, (size_t)(t.p + t.n - s2 - 1)};
                const uint32_t p = resolve(tp, out.pos.size() / 3, "position", line);
                const uint32_t n = resolve(tn, out.nrm.size() / 3, "normal", line);
                const uint32_t x = resolve(tt, out.tex.size() / 2, "texture", line);
                const uint32_t next_id = (uint32_t)(out.order.size() / 3);
                if (next_id == UINT32_MAX) fail(line, "more than 2^32 - 2 vertices");
                const uint32_t id = vertices.find_or_insert(p, n, x, next_id);
                if (id == next_id) {
                    out.order.push_back(p);
                    out.order.push_back(n);
                    out.order.push_back(x);
                }
                out.indices.push_back(id);
            }
            if (out.indices.size() / 3 >= UINT32_MAX) fail(line, "more than 2^32 - 1 triangles");
        }
        // other statements do not change the mesh
    }
}

template <class T>
T* alloc_array(size_t n) {
    if (n == 0) return nullptr;
    T* p = static_cast<T*>(std::malloc(n * sizeof(T)));
    if (!p) throw std::bad_alloc();
    return p;
}

}  // namespace

extern "C" {

vr_status vr_obj_free(vr_obj_mesh* mesh) {
    if (!mesh) return vr::set_error(VR_ERR_INVALID, "vr_obj_free: null mesh");
    std::free(mesh->positions);
    std::free(mesh->uvs);
    std::free(mesh->normals);
    std::free(mesh->indices);
    *mesh = vr_obj_mesh{};
    return VR_OK;
}

vr_status vr_obj_parse(const char* text, size_t size, vr_obj_mesh* mesh) {
    if (!mesh || (!text && size)) return vr::set_error(VR_ERR_INVALID, "vr_obj_parse: null argument");
    *mesh = vr_obj_mesh{};
    try {
        Parsed P;
        parse(text, size, P);
        const size_t nv = P.order.size() / 3, nt = P.indices.size() / 3;
        vr_obj_mesh m{};
        m.num_vertices = (uint32_t)nv;
        m.num_triangles = (uint32_t)nt;
        try {
            m.positions = alloc_array<float>(3 * nv);
            m.uvs = alloc_array<float>(2 * nv);
            m.normals = alloc_array<float>(3 * nv);
            m.indices = alloc_array<uint32_t>(3 * nt);
        } catch (...) {
            vr_obj_free(&m);
            throw;
        }
        for (size_t v = 0; v < nv; ++v) {
            const uint32_t p = P.order[3 * v], n = P.order[3 * v + 1], x = P.order[3 * v + 2];
            for (int a = 0; a < 3; ++a) {
                m.positions[3 * v + a] = (float)P.pos[3 * (size_t)p + a];
                m.normals[3 * v + a] = (float)P.nrm[3 * (size_t)n + a];
            }
            m.uvs[2 * v] = (float)P.tex[2 * (size_t)x];
            m.uvs[2 * v + 1] = (float)P.tex[2 * (size_t)x + 1];
        }
        if (nt) std::memcpy(m.indices, P.indices.data(), 3 * nt * sizeof(uint32_t));
        *mesh = m;
        return VR_OK;
    } catch (const ObjError& e) {
        return vr::set_error(VR_ERR_INVALID, e.message);
    } catch (const std::bad_alloc&) {
        return vr::set_error(VR_ERR_OOM, "vr_obj_parse: host allocation failed");
    } catch (const std::exception& e) {
        return vr::set_error(VR_ERR_INVALID, std::string("vr_obj_parse: ") + e.what());
    }
}

}  // extern "C"
