// importer.cpp — scene files into a host scene (srt_import_scene).  Host code.
//
// .pbrt: the subset the reference's PBRTParser reads
//   (src/importer/pbrtparse.cu): before WorldBegin, Transform (world to
//   camera, turned into the camera frame as the reference does), Film
//   xresolution / yresolution, Camera fov, and Integrator / Sampler /
//   PixelFilter skipped; after it, Transform (replaces the current
//   transform), Material and MakeNamedMaterial of types diffuse,
//   coateddiffuse, conductor, dielectric, diffusetransmission (the
//   reference's parameter mapping, pbrtparse.cu:232-316), NamedMaterial,
//   Shape trianglemesh / plymesh, AreaLightSource diffuse "rgb L",
//   AttributeBegin / AttributeEnd (one shape per attribute block, its
//   emission written into the block's material, pbrtparse.cu:474-491),
//   MakeNamedMedium / MediumInterface skipped, Texture "name" "spectrum"
//   "imagemap" (the image flipped in y as load_texture does) with
//   "texture reflectance" naming a material's colour texture, and
//   trianglemesh "point2 uv" / "float3 tangent".
// .ply meshes: ascii or binary_little_endian; vertex x y z (float or double),
//   optional nx ny nz and u v, other vertex properties skipped; triangular
//   faces from a "vertex_indices" (or "vertex_index") list.
// .obj (with .mtl): what the reference reads through Assimp
//   (src/importer/assimp.cu:17-79, flags Triangulate | GenNormals): one
//   mesh per object / group and material, polygons split into triangle
//   fans, "vn" normals kept per corner (no normals: flat shading, which is
//   what the geometric normal gives), materials as ai_convert maps them —
//   Kd (or Ks when Kd is black) as base colour, Ke as emission (intensity
//   |Ke|), Ni as ior, Pr roughness, Pm metallic, Ps sheen, Pc clearcoat,
//   Pcr clearcoat roughness, aniso anisotropic, with ai_convert's defaults
//   for the rest; faces before any usemtl get a grey (0.6) default; "vt"
//   texture coordinates with v flipped (aiProcess_FlipUVs), map_Kd as the
//   colour texture and norm / map_Kn as the normal texture, loaded
//   unflipped next to the model (AssimpImporter::load_texture).
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "common.h"
#include "host_scene.h"

using namespace srt;

namespace {

std::string dir_of(const std::string& path)
{
    size_t s = path.find_last_of('/');
    return s == std::string::npos ? std::string() : path.substr(0, s + 1);
}

std::string ext_of(const std::string& path)
{
    size_t d = path.find_last_of('.');
    std::string e = d == std::string::npos ? std::string() : path.substr(d + 1);
    for (char& c : e) c = (char)std::tolower((unsigned char)c);
    return e;
}

srt_material disney_default()
{
    srt_material m{};
    m.bxdf.type = SRT_BXDF_DISNEY;
    m.bxdf.ior = 1.5f;
    m.bxdf.roughness = 0.5f;
    m.bxdf.specular = 0.5f;
    m.bxdf.clearcoatGloss = 0.001f;
    return m;
}

void set_emission(srt_material& m, float r, float g, float b)
{
    float in = std::sqrt(r * r + g * g + b * b);
    m.intensity = in;
    for (int k = 0; k < 3; ++k) m.emission_color[k] = in > 0.0f ? (k == 0 ? r : k == 1 ? g : b) / in : 0.0f;
}

// ---------------------------------------------------------------- OBJ --------
// Material of the OBJ reader the reference links (Assimp, ObjFileData.h):
// Kd 0.6 grey, Ks and Ke black, ior 1.0 unless the .mtl sets them; the
// physically based keys (Pr, Pm, Ps, Pc, Pcr) exist only when given, so
// ai_convert's own defaults stand for the others.
struct ObjMaterial {
    float kd[3] = {0.6f, 0.6f, 0.6f}, ks[3] = {0, 0, 0}, ke[3] = {0, 0, 0};
    float ni = 1.0f, pr = 0.5f, pm = 0.0f, ps = 0.0f, pc = 0.0f, pcr = 0.0f, aniso = 0.0f;
    std::string map_kd, norm;  // diffuse and normal textures (aiTextureType_DIFFUSE / _NORMALS)
};

// ai_convert(aiMaterial*), assimp.cu:17-79
srt_material obj_material(const ObjMaterial& o)
{
    srt_material m = disney_default();
    const bool kd_set = o.kd[0] * o.kd[0] + o.kd[1] * o.kd[1] + o.kd[2] * o.kd[2] > 0.0f;
    for (int k = 0; k < 3; ++k) m.base_color[k] = kd_set ? o.kd[k] : o.ks[k];
    set_emission(m, o.ke[0], o.ke[1], o.ke[2]);
    m.bxdf.ior = o.ni;
    m.bxdf.metallic = o.pm;
    m.bxdf.roughness = std::max(o.pr, 0.001f);
    m.bxdf.anisotropic = o.aniso;
    m.bxdf.sheen = o.ps;
    m.bxdf.clearcoat = o.pc;
    m.bxdf.clearcoatGloss = std::max(o.pcr, 0.001f);
    return m;
}

srt_status read_mtl(const std::string& path, std::map<std::string, ObjMaterial>& out)
{
    std::ifstream f(path);
    if (!f) return set_error(SRT_ERR_ARG, "cannot open material library " + path);
    std::string line, cur;
    while (std::getline(f, line)) {
        std::istringstream ls(line);
        std::string key;
        if (!(ls >> key) || key[0] == '#') continue;
        if (key == "newmtl") {
            ls >> cur;
            out[cur] = ObjMaterial();
            continue;
        }
        if (cur.empty()) continue;
        ObjMaterial& m = out[cur];
        auto rgb = [&](float* c) { ls >> c[0] >> c[1] >> c[2]; };
        if (key == "Kd") rgb(m.kd);
        else if (key == "Ks") rgb(m.ks);
        else if (key == "Ke") rgb(m.ke);
        else if (key == "Ni") ls >> m.ni;
        else if (key == "Pr") ls >> m.pr;
        else if (key == "Pm") ls >> m.pm;
        else if (key == "Ps") ls >> m.ps;
        else if (key == "Pc") ls >> m.pc;
        else if (key == "Pcr") ls >> m.pcr;
        else if (key == "aniso") ls >> m.aniso;
        else if (key == "map_Kd" || key == "norm" || key == "map_Kn") {
            // the file name is the last word (options such as -s u v come first)
            std::string w, last;
            while (ls >> w) last = w;
            std::replace(last.begin(), last.end(), '\\', '/');
            (key == "map_Kd" ? m.map_kd : m.norm) = last;
        }
    }
    return SRT_OK;
}

// Meshes as Assimp's OBJ reader makes them: every "o" / "g" statement starts
// an object, and a material change starts a new mesh once the current one
// has faces; the reference then gives each mesh its own copy of its material
// (AssimpImporter::load_meshes, assimp.cu:82-131).
srt_status import_obj(const std::string& path, srt_procedural& p)
{
    std::ifstream f(path);
    if (!f) return set_error(SRT_ERR_ARG, "cannot open " + path);
    std::vector<float> pos, nrm, uvs;
    std::map<std::string, ObjMaterial> lib;
    struct Build {
        HostMesh mesh;
        std::string material;
        std::map<std::array<int64_t, 3>, uint32_t> corner;  // (position, texcoord, normal) -> vertex
        bool any_normal = false, any_uv = false;
    };
    std::vector<Build> built;
    std::string material;
    bool fresh = true;  // the next face starts a new mesh
    std::string line;
    int lineno = 0;
    while (std::getline(f, line)) {
        ++lineno;
        std::istringstream ls(line);
        std::string key;
        if (!(ls >> key) || key[0] == '#') continue;
        if (key == "v") {
            float x = 0, y = 0, z = 0;
            ls >> x >> y >> z;
            pos.insert(pos.end(), {x, y, z});
        } else if (key == "vn") {
            float x = 0, y = 0, z = 0;
            ls >> x >> y >> z;
            nrm.insert(nrm.end(), {x, y, z});
        } else if (key == "vt") {
            float u = 0, v = 0;
            ls >> u >> v;
            uvs.insert(uvs.end(), {u, 1.0f - v});  // aiProcess_FlipUVs
        } else if (key == "o" || key == "g") {
            fresh = true;
        } else if (key == "usemtl") {
            std::string name;
            ls >> name;
            if (name != material) fresh = true;
            material = name;
        } else if (key == "mtllib") {
            std::string name;
            ls >> name;
            SRT_TRY(read_mtl(dir_of(path) + name, lib));
        } else if (key == "f") {
            std::vector<std::array<int64_t, 3>> corners;  // (position, texcoord or -1, normal or -1)
            std::string tok;
            const int64_t np = (int64_t)(pos.size() / 3), nn = (int64_t)(nrm.size() / 3), nt = (int64_t)(uvs.size() / 2);
            while (ls >> tok) {
                int64_t vi = 0, ti = 0, ni = 0;
                size_t s1 = tok.find('/');
                vi = std::strtoll(tok.substr(0, s1).c_str(), nullptr, 10);
                if (s1 != std::string::npos) {
                    size_t s2 = tok.find('/', s1 + 1);
                    const std::string t = tok.substr(s1 + 1, s2 == std::string::npos ? std::string::npos : s2 - s1 - 1);
                    if (!t.empty()) ti = std::strtoll(t.c_str(), nullptr, 10);
                    if (s2 != std::string::npos && s2 + 1 < tok.size())
                        ni = std::strtoll(tok.substr(s2 + 1).c_str(), nullptr, 10);
                }
                vi = vi < 0 ? np + vi : vi - 1;  // OBJ indices are 1-based; negative ones count back
                ti = ti == 0 ? -1 : (ti < 0 ? nt + ti : ti - 1);
                ni = ni == 0 ? -1 : (ni < 0 ? nn + ni : ni - 1);
                if (vi < 0 || vi >= np || ni >= nn || ni < -1 || ti >= nt || ti < -1)
                    return set_error(SRT_ERR_PARSE, path + ":" + std::to_string(lineno) + ": face index out of range");
                corners.push_back({vi, ti, ni});
            }
            if (corners.size() < 3) continue;
            if (fresh || built.empty()) {
                built.emplace_back();
                built.back().material = material;
                fresh = false;
            }
            Build& b = built.back();
            std::vector<uint32_t> id(corners.size());
            for (size_t c = 0; c < corners.size(); ++c) {
                const std::array<int64_t, 3>& k = corners[c];
                auto ct = b.corner.find(k);
                if (ct == b.corner.end()) {
                    const uint32_t v = (uint32_t)(b.mesh.v.size() / 3);
                    b.mesh.v.insert(b.mesh.v.end(), &pos[3 * k[0]], &pos[3 * k[0]] + 3);
                    if (k[2] >= 0) {
                        b.any_normal = true;
                        b.mesh.n.insert(b.mesh.n.end(), &nrm[3 * k[2]], &nrm[3 * k[2]] + 3);
                    } else {
                        b.mesh.n.insert(b.mesh.n.end(), {0.0f, 0.0f, 0.0f});
                    }
                    if (k[1] >= 0) {
                        b.any_uv = true;
                        b.mesh.tc.insert(b.mesh.tc.end(), &uvs[2 * k[1]], &uvs[2 * k[1]] + 2);
                    } else {
                        b.mesh.tc.insert(b.mesh.tc.end(), {0.0f, 0.0f});
                    }
                    ct = b.corner.emplace(k, v).first;
                }
                id[c] = ct->second;
            }
            // polygon as a fan around its first corner (the split Assimp's
            // Triangulate step makes of a convex quad)
            for (size_t c = 1; c + 1 < id.size(); ++c) b.mesh.idx.insert(b.mesh.idx.end(), {id[0], id[c], id[c + 1]});
        }
    }
    std::map<std::string, int> tex_index;  // texture file -> scene texture (load_texture, assimp.cu:170-190)
    auto texture = [&](const std::string& name, int& out) -> srt_status {
        out = -1;
        if (name.empty()) return SRT_OK;
        auto it = tex_index.find(name);
        if (it != tex_index.end()) {
            out = it->second;
            return SRT_OK;
        }
        HostTexture t;
        t.name = name;
        SRT_TRY(load_texture_image(dir_of(path) + name, false, t));
        p.textures.push_back(std::move(t));
        out = tex_index[name] = (int)p.textures.size() - 1;
        return SRT_OK;
    };
    for (Build& b : built) {
        if (!b.any_uv) b.mesh.tc.clear();
        if (!b.any_normal) {
            b.mesh.n.clear();
        } else {
            // corners without a file normal get their face's geometric normal
            for (size_t t = 0; t < b.mesh.idx.size(); t += 3) {
                const float* a = &b.mesh.v[3 * b.mesh.idx[t]];
                const float* c1 = &b.mesh.v[3 * b.mesh.idx[t + 1]];
                const float* c2 = &b.mesh.v[3 * b.mesh.idx[t + 2]];
                float e1[3], e2[3], g[3];
                for (int k = 0; k < 3; ++k) {
                    e1[k] = c1[k] - a[k];
                    e2[k] = c2[k] - a[k];
                }
                g[0] = e1[1] * e2[2] - e1[2] * e2[1];
                g[1] = e1[2] * e2[0] - e1[0] * e2[2];
                g[2] = e1[0] * e2[1] - e1[1] * e2[0];
                for (int j = 0; j < 3; ++j) {
                    float* nv = &b.mesh.n[3 * b.mesh.idx[t + j]];
                    if (nv[0] == 0.0f && nv[1] == 0.0f && nv[2] == 0.0f) std::memcpy(nv, g, sizeof(g));
                }
            }
        }
        // faces before any usemtl, or naming a material the library lacks,
        // get the reader's default material
        auto lt = lib.find(b.material);
        const ObjMaterial om = lt == lib.end() ? ObjMaterial() : lt->second;
        p.mats.push_back(obj_material(om));
        b.mesh.material = (int)p.mats.size() - 1;
        int ct = -1, nt = -1;
        SRT_TRY(texture(om.map_kd, ct));
        SRT_TRY(texture(om.norm, nt));
        if (ct >= 0 || nt >= 0 || !p.mat_tex.empty()) {
            p.mat_tex.resize(2 * p.mats.size(), -1);
            p.mat_tex[2 * b.mesh.material] = ct;
            p.mat_tex[2 * b.mesh.material + 1] = nt;
        }
        p.meshes.push_back(std::move(b.mesh));
    }
    return SRT_OK;
}

// ---------------------------------------------------------------- PLY --------
srt_status read_ply(const std::string& path, HostMesh& m)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) return set_error(SRT_ERR_ARG, "cannot open " + path);
    std::string line;
    std::getline(f, line);
    if (line.compare(0, 3, "ply") != 0) return set_error(SRT_ERR_PARSE, path + ": not a PLY file");
    bool binary = false;
    struct Prop {
        std::string name, type, count_type;
        bool list = false;
    };
    struct Elem {
        std::string name;
        int64_t count = 0;
        std::vector<Prop> props;
    };
    std::vector<Elem> elems;
    while (std::getline(f, line)) {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        std::istringstream ls(line);
        std::string k;
        ls >> k;
        if (k == "format") {
            std::string fmt;
            ls >> fmt;
            if (fmt == "binary_little_endian") binary = true;
            else if (fmt != "ascii") return set_error(SRT_ERR_UNSUPPORTED, path + ": PLY format " + fmt);
        } else if (k == "element") {
            Elem e;
            ls >> e.name >> e.count;
            elems.push_back(e);
        } else if (k == "property") {
            if (elems.empty()) return set_error(SRT_ERR_PARSE, path + ": property before element");
            Prop pr;
            ls >> pr.type;
            if (pr.type == "list") {
                pr.list = true;
                ls >> pr.count_type >> pr.type;
            }
            ls >> pr.name;
            elems.back().props.push_back(pr);
        } else if (k == "end_header") {
            break;
        }
    }
    auto size_of = [](const std::string& t) -> int {
        if (t == "char" || t == "uchar" || t == "int8" || t == "uint8") return 1;
        if (t == "short" || t == "ushort" || t == "int16" || t == "uint16") return 2;
        if (t == "int" || t == "uint" || t == "float" || t == "int32" || t == "uint32" || t == "float32") return 4;
        if (t == "double" || t == "float64") return 8;
        return 0;
    };
    auto read_bin = [&](const std::string& t, double& out) -> bool {
        unsigned char b[8];
        const int s = size_of(t);
        if (s == 0 || !f.read(reinterpret_cast<char*>(b), s)) return false;
        if (t == "float" || t == "float32") {
            float v;
            std::memcpy(&v, b, 4);
            out = v;
        } else if (t == "double" || t == "float64") {
            double v;
            std::memcpy(&v, b, 8);
            out = v;
        } else {
            uint64_t u = 0;
            for (int i = s - 1; i >= 0; --i) u = (u << 8) | b[i];
            const bool sign = t == "char" || t == "int8" || t == "short" || t == "int16" || t == "int" || t == "int32";
            if (sign && s < 8 && (u >> (8 * s - 1)) & 1u) u |= ~0ull << (8 * s);
            out = sign ? (double)(int64_t)u : (double)u;
        }
        return true;
    };
    auto read_val = [&](const std::string& t, double& out) -> bool {
        if (binary) return read_bin(t, out);
        return (bool)(f >> out);
    };
    for (const Elem& e : elems) {
        const bool is_v = e.name == "vertex", is_f = e.name == "face";
        int ix = -1, iy = -1, iz = -1, inx = -1, iny = -1, inz = -1, iu = -1, iv = -1;
        for (size_t i = 0; i < e.props.size(); ++i) {
            const std::string& n = e.props[i].name;
            if (n == "x") ix = (int)i;
            if (n == "y") iy = (int)i;
            if (n == "z") iz = (int)i;
            if (n == "nx") inx = (int)i;
            if (n == "ny") iny = (int)i;
            if (n == "nz") inz = (int)i;
            if (n == "u") iu = (int)i;
            if (n == "v") iv = (int)i;
        }
        const bool uvs = is_v && iu >= 0 && iv >= 0 && iu < 16 && iv < 16;
        const bool normals = is_v && inx >= 0 && iny >= 0 && inz >= 0;
        for (int64_t r = 0; r < e.count; ++r) {
            double vals[16] = {};
            for (size_t i = 0; i < e.props.size(); ++i) {
                const Prop& pr = e.props[i];
                if (pr.list) {
                    double cnt;
                    if (!read_val(pr.count_type, cnt)) return set_error(SRT_ERR_PARSE, path + ": truncated list");
                    const bool indices = is_f && (pr.name == "vertex_indices" || pr.name == "vertex_index");
                    if (indices && cnt != 3)
                        return set_error(SRT_ERR_UNSUPPORTED, path + ": only triangular PLY faces are read");
                    for (int64_t c = 0; c < (int64_t)cnt; ++c) {
                        double x;
                        if (!read_val(pr.type, x)) return set_error(SRT_ERR_PARSE, path + ": truncated list");
                        if (indices) m.idx.push_back((uint32_t)x);
                    }
                } else {
                    double x;
                    if (!read_val(pr.type, x)) return set_error(SRT_ERR_PARSE, path + ": truncated data");
                    if (i < 16) vals[i] = x;
                }
            }
            if (is_v) {
                if (ix < 0 || iy < 0 || iz < 0 || ix >= 16 || iy >= 16 || iz >= 16)
                    return set_error(SRT_ERR_PARSE, path + ": vertex without x y z");
                m.v.insert(m.v.end(), {(float)vals[ix], (float)vals[iy], (float)vals[iz]});
                if (normals && inx < 16 && iny < 16 && inz < 16)
                    m.n.insert(m.n.end(), {(float)vals[inx], (float)vals[iny], (float)vals[inz]});
                if (uvs) m.tc.insert(m.tc.end(), {(float)vals[iu], (float)vals[iv]});
            }
        }
    }
    const size_t nv = m.v.size() / 3;
    for (uint32_t i : m.idx)
        if (i >= nv) return set_error(SRT_ERR_PARSE, path + ": face index out of range");
    return SRT_OK;
}

// --------------------------------------------------------------- PBRT --------
// 4x4 matrices row-major; the reference builds SquareMatrix<4> from the 16
// numbers row by row and transposes (pbrt lists them column by column).
struct Mat4 {
    double m[4][4];
};

Mat4 from_pbrt(const std::vector<float>& v)
{
    Mat4 r{};
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) r.m[i][j] = v[4 * j + i];  // transpose of the row-by-row fill
    return r;
}

bool invert(const Mat4& a, Mat4& out)
{
    double m[4][8];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 8; ++j) m[i][j] = j < 4 ? a.m[i][j] : (j - 4 == i ? 1.0 : 0.0);
    for (int c = 0; c < 4; ++c) {
        int p = c;
        for (int r = c + 1; r < 4; ++r)
            if (std::fabs(m[r][c]) > std::fabs(m[p][c])) p = r;
        if (m[p][c] == 0.0) return false;
        for (int j = 0; j < 8; ++j) std::swap(m[c][j], m[p][j]);
        const double d = m[c][c];
        for (int j = 0; j < 8; ++j) m[c][j] /= d;
        for (int r = 0; r < 4; ++r)
            if (r != c) {
                const double k = m[r][c];
                for (int j = 0; j < 8; ++j) m[r][j] -= k * m[c][j];
            }
    }
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) out.m[i][j] = m[i][j + 4];
    return true;
}

struct PbrtReader {
    std::string text;
    size_t pos = 0;
    std::string file;

    void skip_space()
    {
        while (pos < text.size()) {
            if (text[pos] == '#') {
                while (pos < text.size() && text[pos] != '\n') ++pos;
            } else if (std::isspace((unsigned char)text[pos])) {
                ++pos;
            } else {
                break;
            }
        }
    }
    // a bare word (statement name), "" at the end
    std::string word()
    {
        skip_space();
        size_t b = pos;
        while (pos < text.size() && !std::isspace((unsigned char)text[pos]) && text[pos] != '"' && text[pos] != '[')
            ++pos;
        return text.substr(b, pos - b);
    }
    bool peek(char c)
    {
        skip_space();
        return pos < text.size() && text[pos] == c;
    }
    // "quoted" (false if the next token is not a string)
    bool quoted(std::string& out)
    {
        if (!peek('"')) return false;
        size_t e = text.find('"', pos + 1);
        if (e == std::string::npos) return false;
        out = text.substr(pos + 1, e - pos - 1);
        pos = e + 1;
        return true;
    }
    // [ values ] as text, or a single quoted value / bare number
    bool value(std::string& out)
    {
        skip_space();
        if (peek('[')) {
            size_t e = text.find(']', pos);
            if (e == std::string::npos) return false;
            out = text.substr(pos + 1, e - pos - 1);
            pos = e + 1;
            return true;
        }
        if (peek('"')) return quoted(out);
        out = word();
        return !out.empty();
    }
    // "type name" value pairs until the next statement
    bool params(std::map<std::string, std::string>& out)
    {
        std::string key;
        while (quoted(key)) {
            std::string v;
            if (!value(v)) return false;
            // "type  name" with any spacing -> "type name"
            std::istringstream ks(key);
            std::string t, n;
            ks >> t >> n;
            out[t + " " + n] = v;
        }
        return true;
    }
};

std::vector<float> floats(const std::string& s)
{
    std::vector<float> v;
    std::istringstream is(s);
    std::string tok;
    while (is >> tok) {
        if (!tok.empty() && tok.front() == '"') tok = tok.substr(1);
        if (!tok.empty() && tok.back() == '"') tok.pop_back();
        v.push_back(std::strtof(tok.c_str(), nullptr));
    }
    return v;
}

std::string unquote(std::string s)
{
    while (!s.empty() && (s.front() == '"' || std::isspace((unsigned char)s.front()))) s.erase(s.begin());
    while (!s.empty() && (s.back() == '"' || std::isspace((unsigned char)s.back()))) s.pop_back();
    return s;
}

float get_roughness(const std::map<std::string, std::string>& p, float def)
{
    auto it = p.find("float roughness");
    if (it != p.end()) return std::strtof(unquote(it->second).c_str(), nullptr);
    float u = 0.001f, v = 0.001f;
    if ((it = p.find("float uroughness")) != p.end()) u = std::strtof(unquote(it->second).c_str(), nullptr);
    if ((it = p.find("float vroughness")) != p.end()) v = std::strtof(unquote(it->second).c_str(), nullptr);
    (void)def;
    return (u + v) * 0.5f;
}

srt_status pbrt_material(const std::string& type, const std::map<std::string, std::string>& p, srt_material& m)
{
    m = disney_default();
    m.bxdf.roughness = 0.5f;
    m.base_color[0] = m.base_color[1] = m.base_color[2] = 0.0f;
    auto it = p.find("rgb reflectance");
    if (it != p.end()) {
        std::vector<float> c = floats(it->second);
        if (c.size() >= 3)
            for (int k = 0; k < 3; ++k) m.base_color[k] = c[k];
    }
    if (type == "diffuse") {
        m.bxdf.type = SRT_BXDF_DIFFUSE;
    } else if (type == "coateddiffuse") {
        m.bxdf.roughness = get_roughness(p, 0.001f);
        m.bxdf.clearcoat = 0.8f;
        m.bxdf.clearcoatGloss = 1.0f;
    } else if (type == "conductor") {
        m.bxdf.metallic = 1.0f;
        m.bxdf.roughness = get_roughness(p, 0.001f);
        m.base_color[0] = m.base_color[1] = m.base_color[2] = 1.0f;
    } else if (type == "dielectric") {
        m.bxdf.type = SRT_BXDF_DIELECTRIC;
        m.base_color[0] = m.base_color[1] = m.base_color[2] = 1.0f;
        if ((it = p.find("float eta")) != p.end()) m.bxdf.ior = std::strtof(unquote(it->second).c_str(), nullptr);
    } else if (type == "diffusetransmission") {
        m.bxdf.type = SRT_BXDF_DIFFUSE_TRANSMISSION;
        if (m.base_color[0] == 0.0f && m.base_color[1] == 0.0f && m.base_color[2] == 0.0f)
            m.base_color[0] = m.base_color[1] = m.base_color[2] = 1.0f;
    } else {
        return set_error(SRT_ERR_UNSUPPORTED, "Unsupported material type: " + type);
    }
    m.bxdf.roughness = std::max(m.bxdf.roughness, 0.001f);
    m.bxdf.clearcoatGloss = std::max(m.bxdf.clearcoatGloss, 0.001f);
    return SRT_OK;
}

srt_status pbrt_shape(const std::string& dir, const std::string& type, const std::map<std::string, std::string>& p,
                      HostMesh& m)
{
    if (type == "plymesh") {
        auto it = p.find("string filename");
        if (it == p.end()) return set_error(SRT_ERR_PARSE, "No filename specified for plymesh");
        return read_ply(dir + unquote(it->second), m);
    }
    if (type == "trianglemesh") {
        auto it = p.find("point3 P");
        if (it == p.end()) return set_error(SRT_ERR_PARSE, "No point3 P specified for trianglemesh");
        m.v = floats(it->second);
        if ((it = p.find("integer indices")) == p.end())
            return set_error(SRT_ERR_PARSE, "No integer indices specified for trianglemesh");
        for (float x : floats(it->second)) m.idx.push_back((uint32_t)x);
        if ((it = p.find("normal N")) != p.end()) m.n = floats(it->second);
        if ((it = p.find("point2 uv")) != p.end()) m.tc = floats(it->second);
        if ((it = p.find("float3 tangent")) != p.end()) m.tg = floats(it->second);
        const size_t nv = m.v.size() / 3;
        if (m.v.size() % 3 || m.idx.size() % 3 || (!m.n.empty() && m.n.size() != m.v.size()) ||
            (!m.tc.empty() && m.tc.size() != 2 * nv) || (!m.tg.empty() && m.tg.size() != m.v.size()))
            return set_error(SRT_ERR_PARSE, "trianglemesh arrays of the wrong size");
        for (uint32_t i : m.idx)
            if (i >= m.v.size() / 3) return set_error(SRT_ERR_PARSE, "trianglemesh index out of range");
        return SRT_OK;
    }
    return set_error(SRT_ERR_UNSUPPORTED, "Unsupported shape type: " + type);
}

srt_status import_pbrt(const std::string& path, srt_procedural& p, srt_camera_desc& cam)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) return set_error(SRT_ERR_ARG, "Failed to open file: " + path);
    PbrtReader R;
    std::ostringstream ss;
    ss << f.rdbuf();
    R.text = ss.str();
    const std::string dir = dir_of(path);
    auto bad = [&](const std::string& what) { return set_error(SRT_ERR_PARSE, path + ": " + what); };
    // ---- options (pbrtparse.cu parse_options) ----
    float fov = 60.0f;
    Mat4 c2w{};
    for (int i = 0; i < 4; ++i) c2w.m[i][i] = 1.0;
    for (;;) {
        std::string tok = R.word();
        if (tok.empty()) return bad("no WorldBegin");
        std::map<std::string, std::string> prm;
        std::string s;
        if (tok == "Integrator" || tok == "Sampler" || tok == "PixelFilter") {
            R.quoted(s);
            if (!R.params(prm)) return bad("malformed parameters");
        } else if (tok == "Transform") {
            std::string v;
            if (!R.value(v)) return bad("Transform without values");
            std::vector<float> a = floats(v);
            if (a.size() != 16) return bad("Transform needs 16 values");
            Mat4 w2c = from_pbrt(a), inv;
            if (!invert(w2c, inv)) return bad("singular camera transform");
            // left-handed camera: negate the first column (pbrtparse.cu, parse_options)
            for (int i = 0; i < 4; ++i) inv.m[i][0] = -inv.m[i][0];
            c2w = inv;
        } else if (tok == "Film") {
            R.quoted(s);
            if (!R.params(prm)) return bad("malformed Film parameters");
            p.width = (int)std::strtol(unquote(prm["integer xresolution"]).c_str(), nullptr, 10);
            p.height = (int)std::strtol(unquote(prm["integer yresolution"]).c_str(), nullptr, 10);
        } else if (tok == "Camera") {
            R.quoted(s);
            if (!R.params(prm)) return bad("malformed Camera parameters");
            if (prm.count("float fov")) fov = std::strtof(unquote(prm["float fov"]).c_str(), nullptr);
        } else if (tok == "WorldBegin") {
            break;
        } else {
            return set_error(SRT_ERR_UNSUPPORTED, path + ": Unsupported token: " + tok);
        }
    }
    // camera frame from the camera-to-world transform, radius 1
    // (CameraController(Transform, r), camera.h:41-53): its columns are the
    // axes x, y, z.  As LookAt(pos, pos + z, up = y) the x axis comes out
    // as cross(y, z); the file's x is that or its mirror (det < 0 frames,
    // which the negated column makes of an ordinary pbrt camera).
    cam = srt_camera_desc{};
    {
        const double x[3] = {c2w.m[0][0], c2w.m[1][0], c2w.m[2][0]};
        const double y[3] = {c2w.m[0][1], c2w.m[1][1], c2w.m[2][1]};
        const double z[3] = {c2w.m[0][2], c2w.m[1][2], c2w.m[2][2]};
        const double yz[3] = {y[1] * z[2] - y[2] * z[1], y[2] * z[0] - y[0] * z[2], y[0] * z[1] - y[1] * z[0]};
        const bool mirrored = x[0] * yz[0] + x[1] * yz[1] + x[2] * yz[2] < 0.0;
        cam.type = SRT_CAMERA_PERSPECTIVE | (mirrored ? SRT_CAMERA_MIRROR_X : 0);
    }
    cam.fov = fov;
    cam.aspect = (p.width > 0 && p.height > 0) ? (float)p.width / (float)p.height : 1.0f;
    cam.focal = 1.0f;
    double zx = c2w.m[0][2], zy = c2w.m[1][2], zz = c2w.m[2][2];
    const double zl = std::sqrt(zx * zx + zy * zy + zz * zz);
    for (int k = 0; k < 3; ++k) {
        cam.position[k] = (float)c2w.m[k][3];
        cam.target[k] = (float)(c2w.m[k][3] + c2w.m[k][2] / zl);
        cam.up[k] = (float)c2w.m[k][1];
    }
    // ---- world (pbrtparse.cu parse_world) ----
    struct State {
        int material = -1;
        float emission[3] = {0, 0, 0};
        float xf[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
        int mesh = -1;
    };
    State global, attr;
    bool in_attr = false;
    std::map<std::string, int> named;
    // "texture reflectance": the colour texture of the material just made
    // (Scene::find_texture; an unknown name leaves it untextured)
    auto reflectance_texture = [&](const std::map<std::string, std::string>& prm) {
        auto it = prm.find("texture reflectance");
        if (it == prm.end()) return;
        const std::string tn = unquote(it->second);
        for (size_t k = 0; k < p.textures.size(); ++k)
            if (p.textures[k].name == tn) {
                p.mat_tex.resize(2 * p.mats.size(), -1);
                p.mat_tex[2 * (p.mats.size() - 1)] = (int32_t)k;
                return;
            }
    };
    for (;;) {
        std::string tok = R.word();
        if (tok.empty() || tok == "WorldEnd") break;
        State& st = in_attr ? attr : global;
        std::map<std::string, std::string> prm;
        std::string s;
        if (tok == "Transform") {
            std::string v;
            if (!R.value(v)) return bad("Transform without values");
            std::vector<float> a = floats(v);
            if (a.size() != 16) return bad("Transform needs 16 values");
            Mat4 t = from_pbrt(a);
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 4; ++j) st.xf[4 * i + j] = (float)t.m[i][j];
        } else if (tok == "MakeNamedMedium") {
            R.quoted(s);
            if (!R.params(prm)) return bad("malformed medium");
        } else if (tok == "MediumInterface") {
            R.quoted(s);
            R.quoted(s);
        } else if (tok == "MakeNamedMaterial") {
            std::string name;
            if (!R.quoted(name) || !R.params(prm)) return bad("malformed MakeNamedMaterial");
            auto it = prm.find("string type");
            if (it == prm.end()) return bad("No type specified for material");
            srt_material m;
            SRT_TRY(pbrt_material(unquote(it->second), prm, m));
            p.mats.push_back(m);
            named[name] = (int)p.mats.size() - 1;
            reflectance_texture(prm);
        } else if (tok == "NamedMaterial") {
            std::string name;
            if (!R.quoted(name)) return bad("NamedMaterial without a name");
            auto it = named.find(name);
            if (it == named.end()) return bad("unknown material " + name);
            st.material = it->second;
        } else if (tok == "Material") {
            std::string type;
            if (!R.quoted(type) || !R.params(prm)) return bad("malformed Material");
            srt_material m;
            SRT_TRY(pbrt_material(type, prm, m));
            p.mats.push_back(m);
            st.material = (int)p.mats.size() - 1;
            reflectance_texture(prm);
        } else if (tok == "Texture") {
            // Texture "name" "spectrum" "imagemap" "string filename" ... (pbrtparse.cu:412-419, 319-331):
            // the image loaded with load_from_file(path, false, true)
            std::string name, a, b2;
            if (!R.quoted(name) || !R.quoted(a) || !R.quoted(b2) || !R.params(prm)) return bad("malformed Texture");
            if (b2 != "imagemap") return set_error(SRT_ERR_UNSUPPORTED, path + ": texture class " + b2 + " (imagemap is read)");
            auto it = prm.find("string filename");
            if (it == prm.end()) return bad("No filename specified for texture");
            HostTexture t;
            t.name = name;
            SRT_TRY(load_texture_image(dir + unquote(it->second), true, t));
            p.textures.push_back(std::move(t));
        } else if (tok == "Shape") {
            std::string type;
            if (!R.quoted(type) || !R.params(prm)) return bad("malformed Shape");
            HostMesh m;
            SRT_TRY(pbrt_shape(dir, type, prm, m));
            p.meshes.push_back(std::move(m));
            const int id = (int)p.meshes.size() - 1;
            if (in_attr) {
                attr.mesh = id;
            } else {
                if (global.material < 0) return bad("shape without a material");
                p.meshes[id].material = global.material;
                HostInstance in{id, {}};
                std::memcpy(in.xf, global.xf, sizeof(in.xf));
                p.instances.push_back(in);
            }
        } else if (tok == "AreaLightSource") {
            R.quoted(s);
            if (!R.params(prm)) return bad("malformed AreaLightSource");
            if (!in_attr) return bad("AreaLightSource outside AttributeBegin / AttributeEnd");
            std::vector<float> L = floats(prm["rgb L"]);
            if (L.size() < 3) return bad("AreaLightSource needs rgb L");
            for (int k = 0; k < 3; ++k) attr.emission[k] = L[k];
        } else if (tok == "AttributeBegin") {
            in_attr = true;
            attr = global;
        } else if (tok == "AttributeEnd") {
            if (attr.material >= 0 && attr.mesh >= 0) {
                srt_material& m = p.mats[attr.material];
                const float e2 = attr.emission[0] * attr.emission[0] + attr.emission[1] * attr.emission[1] +
                                 attr.emission[2] * attr.emission[2];
                if (e2 > 0.0f) set_emission(m, attr.emission[0], attr.emission[1], attr.emission[2]);
                p.meshes[attr.mesh].material = attr.material;
                HostInstance in{attr.mesh, {}};
                std::memcpy(in.xf, attr.xf, sizeof(in.xf));
                p.instances.push_back(in);
            }
            in_attr = false;
        } else {
            return set_error(SRT_ERR_UNSUPPORTED, path + ": Unsupported token: " + tok);
        }
    }
    // shapes never instanced (a block without a material) carry no geometry
    return SRT_OK;
}

}  // namespace

extern "C" srt_status srt_import_scene(const char* path, srt_procedural** out)
{
    clear_error();
    if (!path || !out) return set_error(SRT_ERR_ARG, "NULL argument");
    *out = nullptr;
    srt_procedural* p = new (std::nothrow) srt_procedural();
    if (!p) return set_error(SRT_ERR_OOM, "host allocation failed");
    const std::string file(path), ext = ext_of(file);
    srt_camera_desc cam{};
    cam.type = SRT_CAMERA_PERSPECTIVE;
    cam.position[2] = 1.0f;
    cam.up[1] = 1.0f;
    cam.fov = 60.0f;
    cam.aspect = 1.0f;
    cam.focal = 1.0f;
    srt_status st;
    if (ext == "pbrt") {
        st = import_pbrt(file, *p, cam);
        p->has_camera = true;
    }
    else if (ext == "obj")
        st = import_obj(file, *p);
    else if (ext == "ply") {
        HostMesh m;
        st = read_ply(file, m);
        if (st == SRT_OK) {
            srt_material d = disney_default();
            d.base_color[0] = d.base_color[1] = d.base_color[2] = 0.6f;
            p->mats.push_back(d);
            p->meshes.push_back(std::move(m));
        }
    } else
        st = set_error(SRT_ERR_UNSUPPORTED, "unsupported scene file: " + file + " (pbrt, obj, ply)");
    if (st != SRT_OK) {
        delete p;
        return st;
    }
    const float env[3] = {0.0f, 0.0f, 0.0f};
    p->finish(cam, env);
    *out = p;
    return SRT_OK;
}

extern "C" srt_status srt_procedural_resolution(const srt_procedural* p, int32_t* width, int32_t* height)
{
    clear_error();
    if (!p || !width || !height) return set_error(SRT_ERR_ARG, "NULL argument");
    *width = p->width;
    *height = p->height;
    return SRT_OK;
}
