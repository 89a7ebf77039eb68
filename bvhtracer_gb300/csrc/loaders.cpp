// Mesh decoders feeding the upload: the reference's `.tri` loader (BT/tri_loader/src/lexer.rs,
// loader.rs; TriMeshDecoder, BT/src/mesh/decoders.rs:108-133) and a Wavefront `.obj` reader with
// the conversions of ObjMeshDecoder (decoders.rs:157-215).
//
// `.tri`: tokens are separated by ' ', '\t' and '\\'; '\n' and '\r' are tokens of their own; '#'
// at the start of a token skips to the end of the line.  The file is a sequence of triangles of
// nine floats, with any number of "\n" tokens between triangles (not inside one).  A token that is
// not a float (a '\r' included) is ExpectedFloat, input that ends inside a triangle EndOfFile;
// line numbers count "\n" tokens from 1, as the reference's loader does.  Floats follow Rust's
// f32 grammar (optional sign, digits with an optional point and exponent, or inf / infinity /
// nan in any case) and are correctly rounded.  Per triangle the decoder stores the face normal
// normalize(normalize(v2 - v0) x normalize(v1 - v0)) at all three corners, and zero texture
// coordinates.
//
// `.obj`: the first object only (an "o" after faces or after another "o" ends it); "v" (f64,
// then cast to f32, as the reference casts the parser's f64 values), "vt", "vn", and "f" with
// v, v/t, v//n or v/t/n
// corners (1-based, negative = relative to the end), polygons split into a fan (v0, vi, vi+1).
// Missing texture coordinates and normals are zero, as in ObjMeshDecoder.
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "internal.hpp"

namespace bvhgpu {

int decode_tri(const char* text, size_t len, std::vector<float>& tris, std::vector<float>& normals,
               std::string& err);
int decode_obj(const char* text, size_t len, std::vector<float>& tris, std::vector<float>& normals,
               std::vector<float>& uvs, std::string& err);

namespace {

inline bool tri_ws(char c) { return c == ' ' || c == '\\' || c == '\t'; }
inline bool tri_nl(char c) { return c == '\n' || c == '\r'; }

struct TriLexer {  // BT/tri_loader/src/lexer.rs
    const char* s;
    size_t n, pos = 0;
    bool next(const char** tok, size_t* len) {
        while (pos < n && tri_ws(s[pos])) ++pos;
        if (pos < n && s[pos] == '#')
            while (pos < n && !tri_nl(s[pos])) ++pos;
        const size_t start = pos;
        if (pos >= n) return false;
        if (tri_nl(s[pos])) {
            ++pos;
        } else {
            while (pos < n && !tri_ws(s[pos]) && !tri_nl(s[pos])) ++pos;
            if (pos == start) return false;
        }
        *tok = s + start;
        *len = pos - start;
        return true;
    }
};

bool ieq(const char* a, size_t n, const char* lit) {
    if (std::strlen(lit) != n) return false;
    for (size_t i = 0; i < n; ++i)
        if (std::tolower((unsigned char)a[i]) != lit[i]) return false;
    return true;
}

// Rust's float grammar (str::parse::<f32> / ::<f64>); the value itself by strtod / strtof, which
// round correctly.
bool rust_float_syntax(const char* t, size_t n) {
    size_t i = 0;
    if (i < n && (t[i] == '+' || t[i] == '-')) ++i;
    if (ieq(t + i, n - i, "inf") || ieq(t + i, n - i, "infinity") || ieq(t + i, n - i, "nan")) return true;
    size_t digits = 0;
    while (i < n && std::isdigit((unsigned char)t[i])) ++i, ++digits;
    if (i < n && t[i] == '.') {
        ++i;
        while (i < n && std::isdigit((unsigned char)t[i])) ++i, ++digits;
    }
    if (digits == 0) return false;
    if (i < n && (t[i] == 'e' || t[i] == 'E')) {
        ++i;
        if (i < n && (t[i] == '+' || t[i] == '-')) ++i;
        size_t ed = 0;
        while (i < n && std::isdigit((unsigned char)t[i])) ++i, ++ed;
        if (ed == 0) return false;
    }
    return i == n;
}

bool parse_f32(const char* t, size_t n, float* out) {
    if (!rust_float_syntax(t, n)) return false;
    std::string tok(t, n);
    errno = 0;
    *out = std::strtof(tok.c_str(), nullptr);
    return true;
}
bool parse_f64(const char* t, size_t n, double* out) {
    if (!rust_float_syntax(t, n)) return false;
    std::string tok(t, n);
    *out = std::strtod(tok.c_str(), nullptr);
    return true;
}

// cglinalg's normalize: each component divided by the magnitude sqrt((x*x + y*y) + z*z).
void normalize3(const float* v, float* out) {
    const float m = std::sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
    out[0] = v[0] / m;
    out[1] = v[1] / m;
    out[2] = v[2] / m;
}

}  // namespace

int decode_tri(const char* text, size_t len, std::vector<float>& tris, std::vector<float>& normals,
               std::string& err) {
    TriLexer lx{text, len};
    size_t line = 1;
    const char* peek_tok = nullptr;
    size_t peek_len = 0;
    bool have_peek = false, peek_ok = false;
    auto peek = [&](const char** t, size_t* l) {
        if (!have_peek) {
            peek_ok = lx.next(&peek_tok, &peek_len);
            have_peek = true;
        }
        *t = peek_tok;
        *l = peek_len;
        return peek_ok;
    };
    auto next = [&](const char** t, size_t* l) {
        bool ok = peek(t, l);
        have_peek = false;
        if (ok && *l == 1 && (*t)[0] == '\n') ++line;
        return ok;
    };
    for (;;) {
        const char* t;
        size_t l;
        if (!peek(&t, &l)) break;
        if (l == 1 && t[0] == '\n') {
            next(&t, &l);
            continue;
        }
        float v[9];
        for (int k = 0; k < 9; ++k) {
            if (!next(&t, &l)) {
                err = "line " + std::to_string(line) + ": EndOfFile: the input ends inside a triangle";
                return BVHGPU_ERR_INVALID_ARG;
            }
            if (!parse_f32(t, l, &v[k])) {
                err = "line " + std::to_string(line) + ": ExpectedFloat: `" + std::string(t, l) + "`";
                return BVHGPU_ERR_INVALID_ARG;
            }
        }
        tris.insert(tris.end(), v, v + 9);
        // TriMeshDecoder::read_mesh (decoders.rs:120-129): the same face normal at every corner
        float a[3] = {v[6] - v[0], v[7] - v[1], v[8] - v[2]}, b[3] = {v[3] - v[0], v[4] - v[1], v[5] - v[2]};
        float an[3], bn[3], c[3], nn[3];
        normalize3(a, an);
        normalize3(b, bn);
        c[0] = an[1] * bn[2] - an[2] * bn[1];
        c[1] = an[2] * bn[0] - an[0] * bn[2];
        c[2] = an[0] * bn[1] - an[1] * bn[0];
        normalize3(c, nn);
        for (int k = 0; k < 3; ++k) normals.insert(normals.end(), nn, nn + 3);
    }
    return BVHGPU_OK;
}

int decode_obj(const char* text, size_t len, std::vector<float>& tris, std::vector<float>& normals,
               std::vector<float>& uvs, std::string& err) {
    std::vector<float> v, vt, vn;
    int objects = 0;
    size_t line_no = 0, pos = 0;
    while (pos < len) {
        size_t end = pos;
        while (end < len && text[end] != '\n') ++end;
        std::string line(text + pos, end - pos);
        pos = end + 1;
        ++line_no;
        const size_t hash = line.find('#');
        if (hash != std::string::npos) line.resize(hash);
        std::vector<std::string> tok;
        size_t i = 0;
        while (i < line.size()) {
            while (i < line.size() && std::isspace((unsigned char)line[i])) ++i;
            size_t j = i;
            while (j < line.size() && !std::isspace((unsigned char)line[j])) ++j;
            if (j > i) tok.emplace_back(line.substr(i, j - i));
            i = j;
        }
        if (tok.empty()) continue;
        auto fail = [&](const std::string& what) {
            err = "line " + std::to_string(line_no) + ": " + what;
            return BVHGPU_ERR_INVALID_ARG;
        };
        const std::string& kw = tok[0];
        if (kw == "o") {
            // the reference decodes objects[0] only: a second "o", or one after faces, ends it
            if (objects++ > 0 || !tris.empty()) break;
        } else if (kw == "v" || kw == "vn" || kw == "vt") {
            const size_t need = kw == "vt" ? 1 : 3;
            if (tok.size() < need + 1) return fail("too few coordinates");
            std::vector<float>& dst = kw == "v" ? v : (kw == "vn" ? vn : vt);
            const size_t keep = kw == "vt" ? 2 : 3;
            for (size_t k = 0; k < keep; ++k) {
                double d = 0.0;
                if (k + 1 < tok.size() && !parse_f64(tok[k + 1].data(), tok[k + 1].size(), &d))
                    return fail("expected a number, got `" + tok[k + 1] + "`");
                dst.push_back((float)d);  // `vp.x as f32`
            }
        } else if (kw == "f") {
            if (tok.size() < 4) return fail("a face needs three corners");
            struct Corner {
                long v, t, n;
            };
            std::vector<Corner> cs;
            for (size_t k = 1; k < tok.size(); ++k) {
                Corner c{0, 0, 0};
                long* dst[3] = {&c.v, &c.t, &c.n};
                const long counts[3] = {(long)(v.size() / 3), (long)(vt.size() / 2), (long)(vn.size() / 3)};
                size_t f = 0, a = 0;
                const std::string& s = tok[k];
                while (f < 3 && a <= s.size()) {
                    size_t b = s.find('/', a);
                    if (b == std::string::npos) b = s.size();
                    if (b > a) {
                        char* endp = nullptr;
                        const std::string num = s.substr(a, b - a);
                        long idx = std::strtol(num.c_str(), &endp, 10);
                        if (*endp != '\0' || idx == 0) return fail("bad face index `" + s + "`");
                        if (idx < 0) idx = counts[f] + idx + 1;  // relative to the end
                        if (idx < 1 || idx > counts[f]) return fail("face index out of range `" + s + "`");
                        *dst[f] = idx;
                    } else if (f == 0) {
                        return fail("a face corner needs a vertex index");
                    }
                    ++f;
                    a = b + 1;
                }
                cs.push_back(c);
            }
            for (size_t k = 1; k + 1 < cs.size(); ++k) {
                const Corner tri[3] = {cs[0], cs[k], cs[k + 1]};
                for (const Corner& c : tri) {
                    for (int q = 0; q < 3; ++q) tris.push_back(v[3 * (c.v - 1) + q]);
                    for (int q = 0; q < 3; ++q) normals.push_back(c.n ? vn[3 * (c.n - 1) + q] : 0.0f);
                    for (int q = 0; q < 2; ++q) uvs.push_back(c.t ? vt[2 * (c.t - 1) + q] : 0.0f);
                }
            }
        }
    }
    return BVHGPU_OK;
}

}  // namespace bvhgpu

// ---- C ABI -------------------------------------------------------------------------------------

namespace {

int decode_any(const char* text, size_t len, int format, bvhgpu_triangle* tris, float* normals, float* uvs,
               uint32_t cap, uint32_t* ntris, char* err, size_t errlen) {
    if ((!text && len) || !ntris) return BVHGPU_ERR_INVALID_ARG;
    std::vector<float> t, nrm, uv;
    std::string msg;
    int rc;
    if (format == BVHGPU_MESH_TRI) {
        rc = bvhgpu::decode_tri(text, len, t, nrm, msg);
        uv.assign(t.size() / 9 * 6, 0.0f);  // TextureCoordinates::default()
    } else if (format == BVHGPU_MESH_OBJ) {
        rc = bvhgpu::decode_obj(text, len, t, nrm, uv, msg);
    } else {
        msg = "unknown mesh format";
        rc = BVHGPU_ERR_INVALID_ARG;
    }
    if (err && errlen) std::snprintf(err, errlen, "%s", msg.c_str());
    if (rc) return rc;
    const size_t n = t.size() / 9;
    if (n > 0xFFFFFFFFull) return BVHGPU_ERR_TOO_LARGE;
    *ntris = (uint32_t)n;
    const size_t m = std::min<size_t>(n, cap);
    if (tris) std::memcpy(tris, t.data(), 36 * m);
    if (normals) std::memcpy(normals, nrm.data(), 36 * m);
    if (uvs) std::memcpy(uvs, uv.data(), 24 * m);
    return BVHGPU_OK;
}

}  // namespace

extern "C" {

int bvhgpu_mesh_decode(const char* text, size_t len, int format, bvhgpu_triangle* tris, float* normals, float* uvs,
                       uint32_t cap, uint32_t* ntris, char* err, size_t errlen) {
    return decode_any(text, len, format, tris, normals, uvs, cap, ntris, err, errlen);
}

int bvhgpu_mesh_decode_file(const char* path, int format, bvhgpu_triangle* tris, float* normals, float* uvs,
                            uint32_t cap, uint32_t* ntris, char* err, size_t errlen) {
    if (!path) return BVHGPU_ERR_INVALID_ARG;
    std::FILE* f = std::fopen(path, "rb");
    if (!f) {
        if (err && errlen) std::snprintf(err, errlen, "cannot open %s", path);
        return BVHGPU_ERR_INVALID_ARG;
    }
    std::string data;
    char buf[1 << 16];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) data.append(buf, got);
    std::fclose(f);
    return decode_any(data.data(), data.size(), format, tris, normals, uvs, cap, ntris, err, errlen);
}

}  // extern "C"
