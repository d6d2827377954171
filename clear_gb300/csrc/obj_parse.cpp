// Wavefront .obj / .mtl parsing for the model loader (host code).
//
// Reads what OBJ::load and OBJ::loadMtl read (ModelLoader.cpp:76-362) with
// the same line rules, so that a file gives the same vertices, faces, groups
// and materials as in the reference:
//   * a line is split at '\n' only; leading bytes from the set the reference
//     strips are removed -- the UTF-8 ideographic space (E3 80 80), ' ', the
//     UTF-8 yen sign (C2 A5) and the letter 't' -- and nothing else, so a
//     tab-indented statement is ignored;
//   * statements are recognised by their first byte(s) with the C library's
//     scanf conversions (strtof for %f, strtoul for %u, a run of non-space
//     bytes for %s): `o`, `g`, `s off` / `s N`, `v ` / `vt` / `vn` (vt stores
//     1 - v), `f`, `mtllib`, `usemtl`; in .mtl files `newmtl`, `K? r g b` (a
//     statement with fewer than three numbers sets zeros), `Ni`, `map_Kd`,
//     `map_Ks`, `map_Ka`, and `map_bump`, which sets the Kd map;
//   * consecutive `f` lines form a group that takes the current `g` name,
//     smoothing value and `usemtl` name; the group's first line fixes its face
//     format, v/t/n or v//n; only the first three corners of a face are read;
//   * only the first file named by an `mtllib` line is read, relative to the
//     .obj's directory; texture maps are relative to the .mtl's directory; an
//     .mtl that cannot be opened adds no materials.
// Where the reference's behaviour is undefined, this parser defines it:
// statements before the first `o` belong to an implicit object (the
// reference dereferences a null object), groups whose first face is v/t or v
// only are read in those formats, a face line that does not match its
// group's format or that names an index outside the file's vertex, uv or
// normal lists of the whole file is skipped and counted (indices are checked
// after the whole file is read: like the reference, a face may name a vertex
// defined later), missing vertex components read as 0, negative indices count
// back from the end of the list read so far as the OBJ format defines, and
// .mtl statements before the first `newmtl` are ignored.
#include <cctype>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include "clear_cuda.h"

int clr_set_error(int code, const char* fmt, ...);

struct clr_obj_model {
    std::vector<float> positions, uvs, normals;
    std::vector<uint32_t> faces;  // 9 per face: p0 p1 p2, uv0 uv1 uv2, n0 n1 n2
    std::vector<clr_obj_group> groups;
    std::vector<clr_obj_material> materials;
    std::string strings;  // NUL-terminated names; offset 0 is the empty string
    uint32_t skipped = 0;
};

namespace {

constexpr uint32_t kNone = 0xFFFFFFFFu;

uint32_t intern(clr_obj_model* m, const std::string& s) {
    if (s.empty()) return 0;
    const uint32_t at = (uint32_t)m->strings.size();
    m->strings.append(s);
    m->strings.push_back('\0');
    return at;
}

// The reference erases leading bytes found in its separator literal.
bool strip_byte(unsigned char c) {
    return c == 0xE3 || c == 0x80 || c == ' ' || c == 0xC2 || c == 0xA5 || c == 't';
}

// A cursor with the scanf-family conversions the statements use.
struct Cursor {
    const char* p;

    bool lit(const char* s) {
        const size_t n = strlen(s);
        if (strncmp(p, s, n) != 0) return false;
        p += n;
        return true;
    }
    bool lit(char c) {
        if (*p != c) return false;
        ++p;
        return true;
    }
    void space() {
        while (*p && isspace((unsigned char)*p)) ++p;
    }
    bool f32(float* v) {
        space();
        char* e;
        const float x = strtof(p, &e);
        if (e == p) return false;
        *v = x;
        p = e;
        return true;
    }
    // %u, kept signed so that a negative (relative) index can be recognised
    bool index(long long* v) {
        space();
        char* e;
        const long long x = strtoll(p, &e, 10);
        if (e == p) return false;
        *v = x;
        p = e;
        return true;
    }
    bool word(std::string* s) {
        space();
        const char* b = p;
        while (*p && !isspace((unsigned char)*p)) ++p;
        if (p == b) return false;
        s->assign(b, p);
        return true;
    }
};

bool read_lines(const char* path, std::vector<std::string>* lines) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::string line;
    while (std::getline(f, line)) {
        size_t k = 0;
        while (k < line.size() && strip_byte((unsigned char)line[k])) ++k;
        lines->push_back(line.substr(k));
    }
    return true;
}

std::string directory_of(const std::string& path) {
    const size_t k = path.find_last_of('/');
    return k == std::string::npos ? std::string() : path.substr(0, k + 1);
}

void parse_mtl(const std::string& path, clr_obj_model* m) {
    std::vector<std::string> lines;
    if (!read_lines(path.c_str(), &lines)) return;
    const std::string dir = directory_of(path);
    clr_obj_material* cur = nullptr;
    for (const std::string& line : lines) {
        Cursor c{line.c_str()};
        switch (line.empty() ? '\0' : line[0]) {
            case 'K': {
                if (line.size() < 2 || !cur) break;
                const char which = line[1];
                float v[3];
                Cursor k{line.c_str() + 2};
                if (!(k.f32(&v[0]) && k.f32(&v[1]) && k.f32(&v[2]))) v[0] = v[1] = v[2] = 0.0f;
                float* dst = which == 'd' ? cur->Kd : which == 's' ? cur->Ks : which == 'a' ? cur->Ka : nullptr;
                if (dst) memcpy(dst, v, sizeof(v));
                break;
            }
            case 'N': {
                float v;
                if (cur && c.lit("Ni") && c.f32(&v)) cur->Ni = v;
                break;
            }
            case 'm': {
                if (!cur) break;
                std::string name;
                static const char* const keys[4] = {"map_Kd", "map_Ks", "map_Ka", "map_bump"};
                for (int i = 0; i < 4; ++i) {
                    Cursor k{line.c_str()};
                    if (k.lit(keys[i]) && k.word(&name)) {
                        const uint32_t s = intern(m, dir + name);
                        if (i == 1) cur->map_Ks = s;
                        else if (i == 2) cur->map_Ka = s;
                        else cur->map_Kd = s;  // map_bump sets the Kd map too
                        break;
                    }
                }
                break;
            }
            case 'n': {
                std::string name;
                if (!(c.lit("newmtl") && c.word(&name))) break;
                clr_obj_material mat{};
                mat.Ns = 100.0f;
                mat.Ni = 1.0f;
                mat.name = intern(m, name);
                m->materials.push_back(mat);
                cur = &m->materials.back();
                break;
            }
            default:
                break;
        }
    }
}

enum Format : uint32_t { kVTN = CLR_OBJ_VTN, kVN = CLR_OBJ_VN, kVT = CLR_OBJ_VT, kV = CLR_OBJ_V };

// One face line in `fmt`: three corners of p[/t[/n]] (0-based, resolved).
bool parse_face(const char* line, Format fmt, long long out[9]) {
    Cursor c{line};
    if (!c.lit('f')) return false;
    for (int k = 0; k < 3; ++k) {
        long long p, t = 0, n = 0;
        if (!c.index(&p)) return false;
        switch (fmt) {
            case kVTN:
                if (!(c.lit('/') && c.index(&t) && c.lit('/') && c.index(&n))) return false;
                break;
            case kVN:
                if (!(c.lit('/') && c.lit('/') && c.index(&n))) return false;
                break;
            case kVT:
                if (!(c.lit('/') && c.index(&t))) return false;
                break;
            case kV:
                if (*c.p == '/') return false;
                break;
        }
        out[k] = p;
        out[3 + k] = t;
        out[6 + k] = n;
    }
    return true;
}

// 1-based OBJ index -> 0-based; a negative index counts back from `so_far`,
// the length of the list when the face is read.  kNone when it cannot be an
// index (the range check against the whole file's lists comes afterwards).
uint32_t resolve(long long i, size_t so_far) {
    const long long z = i < 0 ? (long long)so_far + i : i - 1;
    return (z >= 0 && z < (long long)kNone) ? (uint32_t)z : kNone;
}

// Drops the faces whose indices fall outside the file's lists.
void check_ranges(clr_obj_model* m) {
    const uint32_t np = (uint32_t)(m->positions.size() / 3), nt = (uint32_t)(m->uvs.size() / 2),
                   nn = (uint32_t)(m->normals.size() / 3);
    size_t out = 0;
    for (clr_obj_group& g : m->groups) {
        const bool has_t = g.format == CLR_OBJ_VTN || g.format == CLR_OBJ_VT;
        const bool has_n = g.format == CLR_OBJ_VTN || g.format == CLR_OBJ_VN;
        const uint32_t first = (uint32_t)(out / 9);
        uint32_t kept = 0;
        for (uint32_t f = g.first_face; f < g.first_face + g.num_faces; ++f) {
            const uint32_t* src = m->faces.data() + 9ull * f;
            bool ok = true;
            for (int k = 0; k < 3; ++k)
                ok = ok && src[k] < np && (!has_t || src[3 + k] < nt) && (!has_n || src[6 + k] < nn);
            if (!ok) {
                ++m->skipped;
                continue;
            }
            memmove(m->faces.data() + out, src, 9 * sizeof(uint32_t));
            out += 9;
            ++kept;
        }
        g.first_face = first;
        g.num_faces = kept;
    }
    m->faces.resize(out);
}

int parse_obj(const char* path, clr_obj_model* m) {
    std::vector<std::string> lines;
    if (!read_lines(path, &lines)) return clr_set_error(CLR_EINVAL, "clr_obj_parse: cannot open %s", path);
    const std::string dir = directory_of(path);
    m->strings.push_back('\0');
    std::string group_name, mat_name;
    uint32_t smooth = 0;
    bool in_faces = false;
    Format fmt = kVTN;
    bool fmt_ok = false;
    for (const std::string& line : lines) {
        const char c0 = line.empty() ? '\0' : line[0];
        if (in_faces && c0 != 'f') in_faces = false;
        Cursor c{line.c_str()};
        std::string w;
        switch (c0) {
            case 'g':
                if (c.lit('g') && c.word(&w)) group_name = w;
                break;
            case 's':
                if (line.compare(0, 5, "s off") == 0) {
                    smooth = 0;
                } else {
                    long long v;
                    if (c.lit('s') && c.index(&v)) smooth = (uint32_t)v;
                }
                break;
            case 'v': {
                const char c1 = line.size() > 1 ? line[1] : '\0';
                float v[3] = {0.0f, 0.0f, 0.0f};
                if (c1 == ' ') {
                    c.p += 1;
                    c.f32(&v[0]) && c.f32(&v[1]) && c.f32(&v[2]);
                    m->positions.insert(m->positions.end(), v, v + 3);
                } else if (c1 == 't') {
                    c.p += 2;
                    c.f32(&v[0]) && c.f32(&v[1]);
                    m->uvs.push_back(v[0]);
                    m->uvs.push_back(1.0f - v[1]);
                } else if (c1 == 'n') {
                    c.p += 2;
                    c.f32(&v[0]) && c.f32(&v[1]) && c.f32(&v[2]);
                    m->normals.insert(m->normals.end(), v, v + 3);
                }
                break;
            }
            case 'f': {
                long long idx[9];
                if (!in_faces) {
                    in_faces = true;
                    clr_obj_group g{};
                    g.first_face = (uint32_t)(m->faces.size() / 9);
                    g.smooth = smooth;
                    g.name = intern(m, group_name);
                    g.material = intern(m, mat_name);
                    fmt_ok = true;
                    if (parse_face(line.c_str(), kVTN, idx)) fmt = kVTN;
                    else if (parse_face(line.c_str(), kVN, idx)) fmt = kVN;
                    else if (parse_face(line.c_str(), kVT, idx)) fmt = kVT;
                    else if (parse_face(line.c_str(), kV, idx)) fmt = kV;
                    else fmt_ok = false;
                    g.format = fmt_ok ? (uint32_t)fmt : (uint32_t)CLR_OBJ_NONE;
                    m->groups.push_back(g);
                }
                if (!fmt_ok || !parse_face(line.c_str(), fmt, idx)) {
                    ++m->skipped;
                    break;
                }
                uint32_t f[9];
                for (int k = 0; k < 3; ++k) {
                    f[k] = resolve(idx[k], m->positions.size() / 3);
                    f[3 + k] = (fmt == kVTN || fmt == kVT) ? resolve(idx[3 + k], m->uvs.size() / 2) : kNone;
                    f[6 + k] = (fmt == kVTN || fmt == kVN) ? resolve(idx[6 + k], m->normals.size() / 3) : kNone;
                }
                m->faces.insert(m->faces.end(), f, f + 9);
                ++m->groups.back().num_faces;
                break;
            }
            case 'm':
                if (line.compare(0, 6, "mtllib") == 0 && c.lit("mtllib") && c.word(&w)) parse_mtl(dir + w, m);
                break;
            case 'u':
                if (line.compare(0, 6, "usemtl") == 0 && c.lit("usemtl") && c.word(&w)) mat_name = w;
                break;
            default:  // `o` starts a new object, which changes nothing in the flattened lists
                break;
        }
    }
    check_ranges(m);
    return CLR_OK;
}

}  // namespace

extern "C" int clr_obj_parse(const char* path, clr_obj_model** model) {
    if (!path || !model) return clr_set_error(CLR_EINVAL, "clr_obj_parse: NULL argument");
    *model = nullptr;
    std::unique_ptr<clr_obj_model> m(new (std::nothrow) clr_obj_model());
    if (!m) return clr_set_error(CLR_ENOMEM, "clr_obj_parse: out of host memory");
    try {
        const int rc = parse_obj(path, m.get());
        if (rc != CLR_OK) return rc;
    } catch (const std::bad_alloc&) {
        return clr_set_error(CLR_ENOMEM, "clr_obj_parse: out of host memory reading %s", path);
    }
    *model = m.release();
    return CLR_OK;
}

extern "C" int clr_obj_counts_of(const clr_obj_model* m, clr_obj_counts* counts) {
    if (!m || !counts) return clr_set_error(CLR_EINVAL, "clr_obj_counts_of: NULL argument");
    counts->num_positions = (uint32_t)(m->positions.size() / 3);
    counts->num_uvs = (uint32_t)(m->uvs.size() / 2);
    counts->num_normals = (uint32_t)(m->normals.size() / 3);
    counts->num_faces = (uint32_t)(m->faces.size() / 9);
    counts->num_groups = (uint32_t)m->groups.size();
    counts->num_materials = (uint32_t)m->materials.size();
    counts->num_skipped = m->skipped;
    counts->string_bytes = (uint32_t)m->strings.size();
    return CLR_OK;
}

extern "C" int clr_obj_data(const clr_obj_model* m, const float** positions, const float** uvs, const float** normals,
                            const uint32_t** faces, const clr_obj_group** groups,
                            const clr_obj_material** materials, const char** strings) {
    if (!m) return clr_set_error(CLR_EINVAL, "clr_obj_data: NULL model");
    if (positions) *positions = m->positions.data();
    if (uvs) *uvs = m->uvs.data();
    if (normals) *normals = m->normals.data();
    if (faces) *faces = m->faces.data();
    if (groups) *groups = m->groups.data();
    if (materials) *materials = m->materials.data();
    if (strings) *strings = m->strings.data();
    return CLR_OK;
}

extern "C" void clr_obj_free(clr_obj_model* m) { delete m; }
