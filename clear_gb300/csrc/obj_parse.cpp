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
#include <algorithm>
#include <cctype>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <new>
#include <string>
#include <thread>
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

// f(lo, hi) over [0, n) in contiguous ranges on the host's threads, at
// least min_per_thread items each.
template <typename F>
void parallel_ranges(size_t n, F f, size_t min_per_thread = 4096) {
    size_t threads = std::max<size_t>(1, std::thread::hardware_concurrency());
    threads = std::min(threads, std::max<size_t>(1, n / min_per_thread));
    if (threads <= 1) {
        f(size_t(0), n);
        return;
    }
    std::vector<std::thread> pool;
    pool.reserve(threads);
    for (size_t t = 0; t < threads; ++t) pool.emplace_back(f, n * t / threads, n * (t + 1) / threads);
    for (std::thread& th : pool) th.join();
}

// A whole file read in one piece, its lines NUL-terminated in place: each
// '\n' becomes a NUL and each line starts after the bytes the reference
// strips.
struct FileLines {
    std::unique_ptr<char[]> data;
    size_t size = 0;
    std::vector<size_t> starts;
};

bool read_buffer(const char* path, FileLines* fl) {
    std::FILE* f = std::fopen(path, "rb");
    if (!f) return false;
    const long end = std::fseek(f, 0, SEEK_END) == 0 ? std::ftell(f) : -1L;
    if (end < 0 || std::fseek(f, 0, SEEK_SET) != 0) {  // not a regular file
        std::fclose(f);
        return false;
    }
    size_t n = (size_t)end;
    fl->data.reset(new char[n + 1]);
    n = std::fread(fl->data.get(), 1, n, f);
    std::fclose(f);
    char* b = fl->data.get();
    b[n] = '\0';
    fl->size = n;
    // newline positions, found in parallel byte ranges and joined in order
    const size_t chunks = std::max<size_t>(1, std::min<size_t>(64, n >> 20));  // at least 1 MB each
    std::vector<std::vector<size_t>> nl(chunks);
    parallel_ranges(
        chunks,
        [&](size_t lo, size_t hi) {
            for (size_t c = lo; c < hi; ++c) {
                const char* p = b + n * c / chunks;
                const char* const e = b + n * (c + 1) / chunks;
                while ((p = static_cast<const char*>(memchr(p, '\n', (size_t)(e - p)))) != nullptr)
                    nl[c].push_back((size_t)(p++ - b));
            }
        },
        1);
    size_t lines = 0;
    for (const auto& v : nl) lines += v.size();
    std::vector<size_t> ends;
    ends.reserve(lines + 1);
    for (const auto& v : nl) ends.insert(ends.end(), v.begin(), v.end());
    if (ends.empty() ? n > 0 : ends.back() + 1 < n) ends.push_back(n);  // a last line without '\n'
    fl->starts.resize(ends.size());
    parallel_ranges(ends.size(), [&](size_t lo, size_t hi) {
        for (size_t i = lo; i < hi; ++i) {
            const size_t e = ends[i];
            size_t k = i == 0 ? 0 : ends[i - 1] + 1;
            b[e] = '\0';
            while (k < e && strip_byte((unsigned char)b[k])) ++k;
            fl->starts[i] = k;
        }
    });
    return true;
}

// A face line found by the statement pass: where it is, its group's format
// and the lengths of the three lists when it was read (for negative indices).
struct FaceLine {
    size_t at;
    uint32_t fmt, np, nt, nn;
};

// Two passes.  The statement pass walks the lines in order with the
// reference's state (groups, smoothing, materials, face-run boundaries, each
// group's face format) and only notes where each vertex, uv, normal and face
// line is; the number pass then converts those lines in parallel into their
// slots.  A face that does not parse in its group's format is stored with
// no valid index, so the range check drops and counts it as the reference's
// loop would.
int parse_obj(const char* path, clr_obj_model* m) {
    FileLines file;
    if (!read_buffer(path, &file)) return clr_set_error(CLR_EINVAL, "clr_obj_parse: cannot open %s", path);
    const std::vector<size_t>& starts = file.starts;
    const char* b = file.data.get();
    const std::string dir = directory_of(path);
    m->strings.push_back('\0');
    std::string group_name, mat_name;
    uint32_t smooth = 0;
    bool in_faces = false;
    Format fmt = kVTN;
    bool fmt_ok = false;
    std::vector<size_t> vlines, tlines, nlines;
    std::vector<FaceLine> flines;
    for (const size_t at : starts) {
        const char* line = b + at;
        const char c0 = line[0];
        if (in_faces && c0 != 'f') in_faces = false;
        Cursor c{line};
        std::string w;
        switch (c0) {
            case 'g':
                if (c.lit('g') && c.word(&w)) group_name = w;
                break;
            case 's':
                if (strncmp(line, "s off", 5) == 0) {
                    smooth = 0;
                } else {
                    long long v;
                    if (c.lit('s') && c.index(&v)) smooth = (uint32_t)v;
                }
                break;
            case 'v':
                if (line[1] == ' ') vlines.push_back(at);
                else if (line[1] == 't') tlines.push_back(at);
                else if (line[1] == 'n') nlines.push_back(at);
                break;
            case 'f': {
                if (!in_faces) {
                    in_faces = true;
                    clr_obj_group g{};
                    g.first_face = (uint32_t)flines.size();
                    g.smooth = smooth;
                    g.name = intern(m, group_name);
                    g.material = intern(m, mat_name);
                    long long idx[9];
                    fmt_ok = true;
                    if (parse_face(line, kVTN, idx)) fmt = kVTN;
                    else if (parse_face(line, kVN, idx)) fmt = kVN;
                    else if (parse_face(line, kVT, idx)) fmt = kVT;
                    else if (parse_face(line, kV, idx)) fmt = kV;
                    else fmt_ok = false;
                    g.format = fmt_ok ? (uint32_t)fmt : (uint32_t)CLR_OBJ_NONE;
                    m->groups.push_back(g);
                }
                if (!fmt_ok) {
                    ++m->skipped;
                    break;
                }
                flines.push_back(FaceLine{at, (uint32_t)fmt, (uint32_t)vlines.size(), (uint32_t)tlines.size(),
                                          (uint32_t)nlines.size()});
                ++m->groups.back().num_faces;
                break;
            }
            case 'm':
                if (strncmp(line, "mtllib", 6) == 0 && c.lit("mtllib") && c.word(&w)) parse_mtl(dir + w, m);
                break;
            case 'u':
                if (strncmp(line, "usemtl", 6) == 0 && c.lit("usemtl") && c.word(&w)) mat_name = w;
                break;
            default:  // `o` starts a new object, which changes nothing in the flattened lists
                break;
        }
    }
    m->positions.resize(3 * vlines.size());
    m->uvs.resize(2 * tlines.size());
    m->normals.resize(3 * nlines.size());
    m->faces.resize(9 * flines.size());
    parallel_ranges(vlines.size(), [&](size_t lo, size_t hi) {
        for (size_t i = lo; i < hi; ++i) {
            Cursor c{b + vlines[i] + 1};
            float v[3] = {0.0f, 0.0f, 0.0f};
            c.f32(&v[0]) && c.f32(&v[1]) && c.f32(&v[2]);
            memcpy(&m->positions[3 * i], v, sizeof(v));
        }
    });
    parallel_ranges(tlines.size(), [&](size_t lo, size_t hi) {
        for (size_t i = lo; i < hi; ++i) {
            Cursor c{b + tlines[i] + 2};
            float v[2] = {0.0f, 0.0f};
            c.f32(&v[0]) && c.f32(&v[1]);
            m->uvs[2 * i] = v[0];
            m->uvs[2 * i + 1] = 1.0f - v[1];
        }
    });
    parallel_ranges(nlines.size(), [&](size_t lo, size_t hi) {
        for (size_t i = lo; i < hi; ++i) {
            Cursor c{b + nlines[i] + 2};
            float v[3] = {0.0f, 0.0f, 0.0f};
            c.f32(&v[0]) && c.f32(&v[1]) && c.f32(&v[2]);
            memcpy(&m->normals[3 * i], v, sizeof(v));
        }
    });
    parallel_ranges(flines.size(), [&](size_t lo, size_t hi) {
        for (size_t i = lo; i < hi; ++i) {
            const FaceLine& fl = flines[i];
            const Format ff = (Format)fl.fmt;
            uint32_t* f = &m->faces[9 * i];
            long long idx[9];
            if (!parse_face(b + fl.at, ff, idx)) {
                for (int k = 0; k < 9; ++k) f[k] = kNone;
                continue;
            }
            for (int k = 0; k < 3; ++k) {
                f[k] = resolve(idx[k], fl.np);
                f[3 + k] = (ff == kVTN || ff == kVT) ? resolve(idx[3 + k], fl.nt) : kNone;
                f[6 + k] = (ff == kVTN || ff == kVN) ? resolve(idx[6 + k], fl.nn) : kNone;
            }
        }
    });
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
