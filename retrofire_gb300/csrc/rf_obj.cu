// rf_obj.cu — Wavefront OBJ text to mesh arrays (host code), the ingestion
// path of include/rfgpu.h.  Restates retrofire's reader (geom/src/io.rs:
// do_parse_obj :145-230, Builder conversions :232-303, parse_face / indices
// :309-370): the same items, the same quad split, the same vertex
// de-duplication by (position, texcoord, normal) index triple in order of
// first use, the same errors (as status codes, where the reader panics too).
#include <locale.h>
#include <stdlib.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/rfgpu.h"

namespace {

constexpr uint64_t NONE = ~0ull;

struct Idx {
    uint64_t pos, uv, n;  // zero-based; NONE when absent
    bool operator<(const Idx &o) const { return std::tie(pos, uv, n) < std::tie(o.pos, o.uv, o.n); }
};

struct ObjErr {
    std::string msg;
};

bool is_ws(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\f' || c == '\r'; }

// split_ascii_whitespace of one line
std::vector<std::string> tokens_of(const char *b, const char *e) {
    std::vector<std::string> out;
    while (b < e) {
        while (b < e && is_ws(*b)) ++b;
        const char *s = b;
        while (b < e && !is_ws(*b)) ++b;
        if (b > s) out.emplace_back(s, b);
    }
    return out;
}

// The grammar of Rust's f32::from_str: Sign? ('inf' | 'infinity' | 'nan' |
// Number), the words in any case; Number = (Digit+ | Digit+ '.' Digit* |
// Digit* '.' Digit+) Exp?; Exp = ('e' | 'E') Sign? Digit+.  (No hexadecimal
// forms, no "nan(...)" payloads, no spaces.)
bool is_digit(char c) { return c >= '0' && c <= '9'; }
bool rust_f32_syntax(const std::string &t) {
    size_t i = 0;
    const size_t n = t.size();
    if (i < n && (t[i] == '+' || t[i] == '-')) ++i;
    std::string word;
    for (size_t k = i; k < n; ++k) word += (char)((t[k] >= 'A' && t[k] <= 'Z') ? t[k] - 'A' + 'a' : t[k]);
    if (word == "inf" || word == "infinity" || word == "nan") return true;
    size_t digits = 0;
    while (i < n && is_digit(t[i])) ++i, ++digits;
    if (i < n && t[i] == '.') {
        ++i;
        while (i < n && is_digit(t[i])) ++i, ++digits;
    }
    if (digits == 0) return false;
    if (i < n && (t[i] == 'e' || t[i] == 'E')) {
        ++i;
        if (i < n && (t[i] == '+' || t[i] == '-')) ++i;
        size_t ed = 0;
        while (i < n && is_digit(t[i])) ++i, ++ed;
        if (ed == 0) return false;
    }
    return i == n;
}

// The "C" locale, so that the decimal point is '.' whatever locale the
// calling process has set.
locale_t c_locale() {
    static const locale_t loc = newlocale(LC_NUMERIC_MASK, "C", (locale_t)0);
    return loc;
}

// f32 parsing as Rust's f32::from_str: its grammar, then the correctly
// rounded value (strtof; out of range gives +-inf or +-0 as Rust does).
float parse_f32(const std::string &t) {
    if (!rust_f32_syntax(t)) throw ObjErr{"invalid numeric value"};
    char *end = nullptr;
    const locale_t loc = c_locale();
    const float v = loc ? strtof_l(t.c_str(), &end, loc) : strtof(t.c_str(), &end);
    if (end != t.c_str() + t.size()) throw ObjErr{"invalid numeric value"};
    return v;
}

// usize parsing ("+" allowed, digits only), then OBJ's one-based index.
uint64_t parse_index(const std::string &t) {
    size_t i = 0;
    if (i < t.size() && t[i] == '+') ++i;
    if (i == t.size()) throw ObjErr{"invalid numeric value"};
    uint64_t v = 0;
    for (; i < t.size(); ++i) {
        if (t[i] < '0' || t[i] > '9') throw ObjErr{"invalid numeric value"};
        const uint64_t d = (uint64_t)(t[i] - '0');
        if (v > (~0ull - d) / 10) throw ObjErr{"invalid numeric value"};
        v = v * 10 + d;
    }
    if (v == 0) throw ObjErr{"index 0 is out of bounds (indices are one-based)"};
    return v - 1;
}

Idx parse_indices(const std::string &param) {
    // pos[/uv[/n]]; an empty uv field means none (`1//2`)
    std::vector<std::string> f;
    size_t s = 0;
    for (;;) {
        const size_t p = param.find('/', s);
        f.push_back(param.substr(s, p == std::string::npos ? std::string::npos : p - s));
        if (p == std::string::npos) break;
        s = p + 1;
    }
    Idx r{NONE, NONE, NONE};
    r.pos = parse_index(f[0]);
    if (f.size() > 1 && !f[1].empty()) r.uv = parse_index(f[1]);
    if (f.size() > 2) r.n = parse_index(f[2]);
    return r;
}

struct Obj {
    std::vector<float> coords, norms, texcs;  // 3, 3, 2 floats each
    std::vector<Idx> faces;                   // 3 per triangle
};

Obj parse(const char *text, size_t len) {
    Obj o;
    Idx mx{0, NONE, NONE};
    bool any_pos = false;
    const char *p = text, *end = text + len;
    while (p < end) {
        const char *nl = static_cast<const char *>(memchr(p, '\n', (size_t)(end - p)));
        const char *le = nl ? nl : end;
        const std::vector<std::string> t = tokens_of(p, le);
        p = nl ? nl + 1 : end;
        const std::string key = t.empty() ? std::string() : t[0];
        auto need = [&](size_t n) {
            if (t.size() < n + 1) throw ObjErr{"unexpected end of input"};
        };
        if (key.empty() || key[0] == '#' || key == "g" || key == "mtllib" || key == "usemtl" ||
            key == "s") {
            continue;
        } else if (key == "v") {
            need(3);
            for (int k = 1; k <= 3; ++k) o.coords.push_back(parse_f32(t[k]));
        } else if (key == "vt") {
            need(2);
            for (int k = 1; k <= 2; ++k) o.texcs.push_back(parse_f32(t[k]));
        } else if (key == "vn") {
            need(3);
            for (int k = 1; k <= 3; ++k) o.norms.push_back(parse_f32(t[k]));
        } else if (key == "f") {
            need(3);
            const size_t nidx = t.size() >= 5 ? 4 : 3;
            Idx is[4];
            for (size_t k = 0; k < nidx; ++k) is[k] = parse_indices(t[1 + k]);
            if (mx.n != NONE && is[0].n == NONE) throw ObjErr{"not all faces have normals"};
            if (mx.uv != NONE && is[0].uv == NONE) throw ObjErr{"not all faces have texcoords"};
            for (size_t k = 0; k < nidx; ++k) {
                mx.pos = std::max(mx.pos, is[k].pos);
                any_pos = true;
                if (is[k].uv != NONE) mx.uv = mx.uv == NONE ? is[k].uv : std::max(mx.uv, is[k].uv);
                if (is[k].n != NONE) mx.n = mx.n == NONE ? is[k].n : std::max(mx.n, is[k].n);
            }
            o.faces.insert(o.faces.end(), {is[0], is[1], is[2]});
            if (nidx == 4) o.faces.insert(o.faces.end(), {is[0], is[2], is[3]});
        } else {
            throw ObjErr{"unsupported item: " + key};
        }
    }
    const uint64_t ncoord = o.coords.size() / 3;
    if (any_pos && mx.pos >= ncoord) throw ObjErr{"vertex index out of bounds"};
    if (mx.uv != NONE && mx.uv >= o.texcs.size() / 2) throw ObjErr{"texcoord index out of bounds"};
    if (mx.n != NONE && mx.n >= o.norms.size() / 3) throw ObjErr{"normal index out of bounds"};
    return o;
}

// Builder<A> from the parsed items: nattr 0 (positions), 3 (normals),
// 2 (texcoords) or 5 (normal, then texcoord).
void build(const Obj &o, int32_t attrs, std::vector<float> &verts, std::vector<uint32_t> &idx,
           uint32_t &nattr) {
    const bool want_n = attrs == RF_OBJ_NORMAL || attrs == RF_OBJ_NORMAL_TEXCOORD;
    const bool want_uv = attrs == RF_OBJ_TEXCOORD || attrs == RF_OBJ_NORMAL_TEXCOORD;
    if (want_n && o.norms.empty()) throw ObjErr{"missing vertex attribute: normal"};
    if (want_uv && o.texcs.empty()) throw ObjErr{"missing vertex attribute: texcoord"};
    nattr = (want_n ? 3u : 0u) + (want_uv ? 2u : 0u);
    std::map<Idx, uint32_t> seen;
    idx.reserve(o.faces.size());
    for (size_t f = 0; f < o.faces.size(); f += 3) {
        for (size_t k = 0; k < 3; ++k) {
            const Idx &v = o.faces[f + k];
            if ((want_n && v.n == NONE) || (want_uv && v.uv == NONE))
                throw ObjErr{"missing vertex attribute"};
        }
        for (size_t k = 0; k < 3; ++k) {
            const Idx &v = o.faces[f + k];
            auto it = seen.find(v);
            if (it == seen.end()) {
                if (seen.size() >= 0xFFFFFFF0u) throw ObjErr{"too many vertices"};
                const uint32_t id = (uint32_t)seen.size();
                it = seen.emplace(v, id).first;
                verts.insert(verts.end(), &o.coords[3 * v.pos], &o.coords[3 * v.pos] + 3);
                if (want_n) verts.insert(verts.end(), &o.norms[3 * v.n], &o.norms[3 * v.n] + 3);
                if (want_uv) verts.insert(verts.end(), &o.texcs[2 * v.uv], &o.texcs[2 * v.uv] + 2);
            }
            idx.push_back(it->second);
        }
    }
}

void set_err(char *err, size_t err_len, const std::string &m) {
    if (err && err_len) snprintf(err, err_len, "%s", m.c_str());
}

}  // namespace

extern "C" {

rf_status rf_obj_parse(const char *text, size_t len, int32_t attrs, float **verts, uint32_t *nverts,
                       uint32_t *nattr, uint32_t **idx, uint32_t *ntri, char *err, size_t err_len) {
    if ((!text && len) || !verts || !nverts || !nattr || !idx || !ntri) return RF_ERR_BAD_ARG;
    if (attrs < RF_OBJ_POSITION || attrs > RF_OBJ_NORMAL_TEXCOORD) return RF_ERR_BAD_ARG;
    *verts = nullptr;
    *idx = nullptr;
    *nverts = *nattr = *ntri = 0;
    set_err(err, err_len, "");
    try {
        const Obj o = parse(text, len);
        std::vector<float> v;
        std::vector<uint32_t> ix;
        uint32_t na = 0;
        build(o, attrs, v, ix, na);
        const size_t stride = 3 + na;
        float *vo = static_cast<float *>(malloc(v.size() * sizeof(float) + 4));
        uint32_t *io = static_cast<uint32_t *>(malloc(ix.size() * sizeof(uint32_t) + 4));
        if (!vo || !io) {
            free(vo);
            free(io);
            return RF_ERR_OOM;
        }
        if (!v.empty()) memcpy(vo, v.data(), v.size() * sizeof(float));
        if (!ix.empty()) memcpy(io, ix.data(), ix.size() * sizeof(uint32_t));
        *verts = vo;
        *idx = io;
        *nverts = (uint32_t)(v.size() / stride);
        *nattr = na;
        *ntri = (uint32_t)(ix.size() / 3);
        return RF_OK;
    } catch (const ObjErr &e) {
        set_err(err, err_len, e.msg);
        return RF_ERR_BAD_ARG;
    } catch (const std::bad_alloc &) {
        return RF_ERR_OOM;
    }
}

void rf_obj_free(void *p) { free(p); }

rf_status rf_mesh_load_obj(rf_ctx *ctx, const char *text, size_t len, int32_t attrs, rf_mesh *out) {
    if (!ctx || !out) return RF_ERR_BAD_ARG;
    float *v = nullptr;
    uint32_t *ix = nullptr, nv = 0, na = 0, nt = 0;
    rf_status st = rf_obj_parse(text, len, attrs, &v, &nv, &na, &ix, &nt, nullptr, 0);
    if (st) return st;
    st = rf_mesh_upload(ctx, v, nv, 3, na, ix, nt, out);
    free(v);
    free(ix);
    return st;
}

}  // extern "C"
