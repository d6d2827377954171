/*
 * C entry points around the reference's own scene encoders
 * (OpenCL_PathTracer/CreateFunctions.cpp, the inline parts of Scene.h) and
 * its .obj loader (OpenCL_PathTracer/ModelLoader.cpp), compiled in place from
 * the reference checkout with the stand-in headers in oracle/ref_stubs.
 *
 * TEST INFRASTRUCTURE ONLY: it pins the Python scene encoders
 * (clear_gb300/scene.py), the .obj loader (clear_gb300/model_loader.py) and
 * the BMP writer (clear_gb300/postprocess.py, against BMPExporter.cpp) byte
 * for byte against the reference, and generates the golden fixtures
 * under tests/golden.  Built only where the reference sources are present
 * (oracle/build_oracle.py), into oracle/_ref/.
 *
 * Driven by a small command script, one command per line, each naming one
 * MaterialCreator / Scene / loadModel call with its arguments (floats in any
 * strtof form, "-" for a null name or an absent override); push / pop /
 * translate / scale / rotate act on the scene's local-to-world stack
 * (`*=` of LinearAlgebra.cpp's matrices).
 *
 * loadImage (ImageLoader.h) is replaced: the reference decodes PNG with
 * libpng and EXR with OpenEXR, neither of which is part of this build.  The
 * stand-in decodes the uncompressed formats the loader tests use into the
 * same texel layouts the reference's decoders produce
 * (ImageLoader.cpp:23-49, 144-205): binary PGM -> Gray8, 1 byte per texel;
 * binary PPM -> RGB8x3 stored as 4 bytes per texel with 0xFF filler (the
 * reference's png_set_filler); PAM RGB_ALPHA -> RGBA8x4; .npy float16
 * (h, w, 4) -> RGBA16Fx4, 8 bytes per texel; rows top to bottom.
 */
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "BMPExporter.h"
#include "CreateFunctions.hpp"
#include "ImageLoader.h"
#include "LinearAlgebra.h"
#include "ModelLoader.hpp"

namespace {

bool read_file(const char* path, std::string* out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    *out = ss.str();
    return true;
}

// netpbm header tokens: whitespace-separated, '#' comments to end of line
bool pnm_token(const std::string& s, size_t* pos, std::string* tok) {
    while (*pos < s.size()) {
        if (s[*pos] == '#') {
            while (*pos < s.size() && s[*pos] != '\n') ++*pos;
        } else if (isspace((unsigned char)s[*pos])) {
            ++*pos;
        } else {
            break;
        }
    }
    const size_t b = *pos;
    while (*pos < s.size() && !isspace((unsigned char)s[*pos]) && s[*pos] != '#') ++*pos;
    *tok = s.substr(b, *pos - b);
    return !tok->empty();
}

bool load_pnm(const std::string& s, std::vector<uint8_t>* storage, uint32_t* w, uint32_t* h,
              ColorChannel::Value* color) {
    size_t pos = 2;
    std::string t;
    uint32_t channels = 0, maxval = 0;
    if (s.compare(0, 2, "P5") == 0 || s.compare(0, 2, "P6") == 0) {
        channels = s[1] == '5' ? 1 : 3;
        if (!pnm_token(s, &pos, &t)) return false;
        *w = (uint32_t)strtoul(t.c_str(), nullptr, 10);
        if (!pnm_token(s, &pos, &t)) return false;
        *h = (uint32_t)strtoul(t.c_str(), nullptr, 10);
        if (!pnm_token(s, &pos, &t)) return false;
        maxval = (uint32_t)strtoul(t.c_str(), nullptr, 10);
        ++pos;  // the single whitespace byte before the raster
    } else if (s.compare(0, 2, "P7") == 0) {
        std::string tupltype;
        while (pnm_token(s, &pos, &t) && t != "ENDHDR") {
            std::string v;
            if (!pnm_token(s, &pos, &v)) return false;
            if (t == "WIDTH") *w = (uint32_t)strtoul(v.c_str(), nullptr, 10);
            else if (t == "HEIGHT") *h = (uint32_t)strtoul(v.c_str(), nullptr, 10);
            else if (t == "DEPTH") channels = (uint32_t)strtoul(v.c_str(), nullptr, 10);
            else if (t == "MAXVAL") maxval = (uint32_t)strtoul(v.c_str(), nullptr, 10);
            else if (t == "TUPLTYPE") tupltype = v;
        }
        ++pos;
    } else {
        return false;
    }
    if (maxval != 255 || (channels != 1 && channels != 3 && channels != 4)) return false;
    const size_t n = (size_t)*w * *h;
    if (s.size() < pos + n * channels) return false;
    const uint8_t* src = (const uint8_t*)s.data() + pos;
    const uint32_t stride = channels == 1 ? 1 : 4;
    const size_t at = storage->size();
    storage->resize(at + n * stride);
    uint8_t* dst = storage->data() + at;
    for (size_t i = 0; i < n; ++i)
        for (uint32_t c = 0; c < stride; ++c) dst[i * stride + c] = c < channels ? src[i * channels + c] : 0xFF;
    *color = channels == 1 ? ColorChannel::Gray8 : channels == 3 ? ColorChannel::RGB8x3 : ColorChannel::RGBA8x4;
    return true;
}

bool load_npy_half4(const std::string& s, std::vector<uint8_t>* storage, uint32_t* w, uint32_t* h,
                    ColorChannel::Value* color) {
    if (s.size() < 10 || s.compare(0, 6, "\x93NUMPY") != 0) return false;
    const uint8_t major = (uint8_t)s[6];
    size_t hlen, hoff;
    if (major == 1) {
        hlen = (uint8_t)s[8] | ((size_t)(uint8_t)s[9] << 8);
        hoff = 10;
    } else {
        hlen = (uint8_t)s[8] | ((size_t)(uint8_t)s[9] << 8) | ((size_t)(uint8_t)s[10] << 16) |
               ((size_t)(uint8_t)s[11] << 24);
        hoff = 12;
    }
    const std::string head = s.substr(hoff, hlen);
    if (head.find("'<f2'") == std::string::npos || head.find("'fortran_order': False") == std::string::npos)
        return false;
    const size_t sp = head.find("'shape': (");
    if (sp == std::string::npos) return false;
    unsigned long dh = 0, dw = 0, dc = 0;
    if (sscanf(head.c_str() + sp, "'shape': (%lu, %lu, %lu)", &dh, &dw, &dc) != 3 || dc != 4) return false;
    *w = (uint32_t)dw;
    *h = (uint32_t)dh;
    const size_t bytes = dh * dw * 4 * 2;
    if (s.size() < hoff + hlen + bytes) return false;
    storage->insert(storage->end(), s.begin() + hoff + hlen, s.begin() + hoff + hlen + bytes);
    *color = ColorChannel::RGBA16Fx4;
    return true;
}

std::vector<std::string> split(const std::string& line) {
    std::vector<std::string> out;
    std::istringstream ss(line);
    std::string t;
    while (ss >> t) out.push_back(t);
    return out;
}

float F(const std::string& s) { return strtof(s.c_str(), nullptr); }
const char* N(const std::string& s) { return s == "-" ? nullptr : s.c_str(); }
uint64_t U64(const std::string& s) { return s == "-" ? UINT64_MAX : strtoull(s.c_str(), nullptr, 10); }

struct Harness {
    Scene scene;
};

// OBJ::objID of the next successful .obj load: process-wide, like the
// reference's own counter (ModelLoader.cpp:32)
int64_t g_loads = 0;

}  // namespace

bool loadImage(const char* fileName, std::vector<uint8_t>* storage, uint32_t* width, uint32_t* height,
               ColorChannel::Value* color, bool /*gammaCorrection*/) {
    std::string s;
    if (!read_file(fileName, &s)) return false;
    if (s.size() >= 2 && s[0] == 'P') return load_pnm(s, storage, width, height, color);
    return load_npy_half4(s, storage, width, height, color);
}

extern "C" {

void* ref_scene_new() { return new Harness(); }

void ref_scene_free(void* h) { delete static_cast<Harness*>(h); }

/* Runs the commands of `script`; returns the number executed, or -(line
 * number) at the first command it does not know (nothing after it runs). */
int ref_scene_exec(void* hp, const char* script) {
    Harness* H = static_cast<Harness*>(hp);
    Scene* sc = &H->scene;
    MaterialCreator& mc = MaterialCreator::sharedInstance();
    mc.setScene(sc);
    std::istringstream in(script);
    std::string line;
    int n = 0, lineno = 0;
    while (std::getline(in, line)) {
        ++lineno;
        const std::vector<std::string> a = split(line);
        if (a.empty()) continue;
        const std::string& c = a[0];
        const size_t k = a.size();
        if (c == "f3tex" && k == 5) mc.createFloat3ConstantTexture(a[1].c_str(), F(a[2]), F(a[3]), F(a[4]));
        else if (c == "ftex" && k == 3) mc.createFloatConstantTexture(a[1].c_str(), F(a[2]));
        else if (c == "imgtex" && k == 3) mc.createImageTexture(a[1].c_str(), a[2].c_str());
        else if (c == "nrmtex" && k == 3) mc.createNormalMapTexture(a[1].c_str(), a[2].c_str());
        else if (c == "checker3" && k == 8)
            mc.createFloat3CheckerBoardTexture(a[1].c_str(), F(a[2]), F(a[3]), F(a[4]), F(a[5]), F(a[6]), F(a[7]));
        else if (c == "checkerbump" && k == 4)
            mc.createFloat3CheckerBoardBumpTexture(a[1].c_str(), F(a[2]), a[3] != "0");
        else if (c == "checker1" && k == 4) mc.createFloatCheckerBoardTexture(a[1].c_str(), F(a[2]), F(a[3]));
        else if (c == "fresnel_noop" && k == 2) mc.createFresnelNoOp(a[1].c_str());
        else if (c == "fresnel_cond" && k == 8)
            mc.createFresnelConductor(a[1].c_str(), F(a[2]), F(a[3]), F(a[4]), F(a[5]), F(a[6]), F(a[7]));
        else if (c == "fresnel_diel" && k == 4) mc.createFresnelDielectric(a[1].c_str(), F(a[2]), F(a[3]));
        else if (c == "matte" && k == 5) mc.createMatteMaterial(a[1].c_str(), N(a[2]), a[3].c_str(), a[4].c_str());
        else if (c == "glass" && k == 7)
            mc.createGlassMaterial(a[1].c_str(), N(a[2]), a[3].c_str(), a[4].c_str(), F(a[5]), F(a[6]));
        else if (c == "metal" && k == 10)
            mc.createMetalMaterial(a[1].c_str(), N(a[2]), a[3].c_str(), F(a[4]), F(a[5]), F(a[6]), F(a[7]), F(a[8]),
                                   F(a[9]));
        else if (c == "newward" && k == 6)
            mc.createNewWardMaterial(a[1].c_str(), N(a[2]), a[3].c_str(), a[4].c_str(), a[5].c_str());
        else if (c == "ashikhmin" && k == 7)
            mc.createAshikhminMaterial(a[1].c_str(), N(a[2]), a[3].c_str(), a[4].c_str(), a[5].c_str(),
                                       a[6].c_str());
        else if (c == "diffuse_light" && k == 3) mc.createDiffuseLightProperty(a[1].c_str(), a[2].c_str());
        else if (c == "ibl_light" && k == 4) mc.createImageBasedEnvLightPropety(a[1].c_str(), a[2].c_str(), F(a[3]));
        else if (c == "cc2d" && k == 4)
            mc.createContinuousConsts2D_H_FromImageTexture(a[1].c_str(), a[2].c_str(), a[3] != "0");
        else if (c == "vertex" && k == 4) sc->addVertex(F(a[1]), F(a[2]), F(a[3]));
        else if (c == "normal" && k == 4) sc->addNormal(F(a[1]), F(a[2]), F(a[3]));
        else if (c == "uv" && k == 3) sc->addUV(F(a[1]), F(a[2]));
        else if (c == "light_dist" && k == 1) sc->calcLightPowerDistribution();
        else if (c == "push" && k == 1) sc->localToWorld.push();
        else if (c == "pop" && k == 1) sc->localToWorld.pop();
        else if (c == "translate" && k == 4) sc->localToWorld *= LinearAlgebra::TranslateMatrix(F(a[1]), F(a[2]), F(a[3]));
        else if (c == "scale" && k == 4) sc->localToWorld *= LinearAlgebra::ScaleMatrix(F(a[1]), F(a[2]), F(a[3]));
        else if (c == "rotate" && k == 5)
            sc->localToWorld *= LinearAlgebra::RotateMatrix(F(a[1]), F(a[2]), F(a[3]), F(a[4]));
        else if ((c == "obj" || c == "objn") && k == 4) {
            // obj: overrides as numbers; objn: as a material and a light
            // property name.  OBJ::load numbers the models it finishes
            // (ModelLoader.cpp:405, 489); loadModel reports nothing, so mirror
            // its two early exits.
            const std::string path = a[1];
            const size_t dot = path.find_first_of('.');
            std::ifstream probe(path);
            const bool loads = dot != std::string::npos && path.substr(dot + 1) == "obj" && probe.good();
            const uint64_t mat = c == "obj" ? U64(a[2]) : a[2] == "-" ? UINT64_MAX : sc->idxOfMat(a[2]);
            const uint64_t lit = c == "obj" ? U64(a[3]) : a[3] == "-" ? UINT64_MAX : sc->idxOfLight(a[3]);
            loadModel(path.c_str(), sc, mat, lit);
            if (loads) ++g_loads;
        } else {
            return -lineno;
        }
        ++n;
    }
    return n;
}

/* Blob `which`: 0 vertices, 1 normals, 2 tangents, 3 uvs, 4 faces,
 * 5 light infos, 6 materials, 7 textures, 8 other resources, 9 light powers.
 * Returns the byte count and sets *data (valid until the next exec). */
uint64_t ref_scene_blob(void* hp, int which, const void** data) {
    Scene* sc = &static_cast<Harness*>(hp)->scene;
    switch (which) {
        case 0: *data = sc->vertices.data(); return sc->vertices.size() * sizeof(cl_float3);
        case 1: *data = sc->normals.data(); return sc->normals.size() * sizeof(cl_float3);
        case 2: *data = sc->tangents.data(); return sc->tangents.size() * sizeof(cl_float3);
        case 3: *data = sc->uvs.data(); return sc->uvs.size() * sizeof(cl_float2);
        case 4: *data = sc->faces.data(); return sc->faces.size() * sizeof(Face);
        case 5: *data = sc->lightInfos.data(); return sc->lightInfos.size() * sizeof(LightInfo);
        case 6: *data = sc->materialsData.data(); return sc->materialsData.size();
        case 7: *data = sc->texturesData.data(); return sc->texturesData.size();
        case 8: *data = sc->otherResouces.data(); return sc->otherResouces.size();
        case 9: *data = sc->lightPowers.data(); return sc->lightPowers.size() * sizeof(float);
        default: *data = nullptr; return 0;
    }
}

/* Name map `which` (0 materials, 1 light properties, 2 textures, 3 other
 * resources, 4 texture files) as "name\toffset\n" lines in key order;
 * returns the bytes needed, writing at most cap. */
uint64_t ref_scene_names(void* hp, int which, char* buf, uint64_t cap) {
    Scene* sc = &static_cast<Harness*>(hp)->scene;
    const std::map<std::string, uint64_t>* m = which == 0   ? &sc->materialsRef
                                               : which == 1 ? &sc->lightPropsRef
                                               : which == 2 ? &sc->texturesRef
                                               : which == 3 ? &sc->othersRef
                                                            : &sc->texFilesDatabase;
    std::string out;
    for (const auto& kv : *m) out += kv.first + "\t" + std::to_string(kv.second) + "\n";
    if (buf && cap) memcpy(buf, out.data(), std::min<uint64_t>(cap, out.size()));
    return out.size();
}

/* saveBMP (BMPExporter.cpp) of `pixels`, the 3 * width + width % 4 byte
 * rows the tone-mapping kernel writes. */
void ref_save_bmp(const char* path, const void* pixels, uint32_t width, uint32_t height) {
    saveBMP(path, pixels, width, height);
}

/* The model number the next successful .obj load will use. */
int64_t ref_scene_next_model_id(void*) { return g_loads; }

}  // extern "C"
