// procedural.cpp — seeded synthetic scenes for the Cornell-box and the
// 5.2M-triangle workloads (the reference's own scenes are not available;
// emission follows the reference's convention intensity = |Le|,
// emission_color = Le / |Le|, src/importer/pbrtparse.cu:474-491).
#include <cmath>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "common.h"
#include "host_scene.h"

namespace {

// PCG32 (O'Neill, pcg-random.org minimal C generator)
struct Pcg32 {
    uint64_t state = 0, inc = 1;
    uint32_t next()
    {
        uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return (xs >> rot) | (xs << ((32u - rot) & 31u));
    }
    void seed(uint64_t initstate, uint64_t initseq)
    {
        state = 0u;
        inc = (initseq << 1u) | 1u;
        next();
        state += initstate;
        next();
    }
    float uniform() { return (float)(next() >> 8) * (1.0f / 16777216.0f); }
};

uint32_t hash32(uint32_t v)
{
    uint32_t s = v * 747796405u + 2891336453u;
    uint32_t w = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
    return (w >> 22u) ^ w;
}

// 3-D value noise in [0, 1): hashed lattice values, smoothstep-weighted
// trilinear interpolation.
float value_noise(float x, float y, float z, uint32_t seed)
{
    float fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
    int ix = (int)fx, iy = (int)fy, iz = (int)fz;
    float tx = x - fx, ty = y - fy, tz = z - fz;
    tx = tx * tx * (3.0f - 2.0f * tx);
    ty = ty * ty * (3.0f - 2.0f * ty);
    tz = tz * tz * (3.0f - 2.0f * tz);
    auto lat = [&](int a, int b, int c) {
        uint32_t h = hash32(seed ^ hash32((uint32_t)a ^ hash32((uint32_t)b ^ hash32((uint32_t)c))));
        return (float)(h >> 8) * (1.0f / 16777216.0f);
    };
    float v[2][2][2];
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int c = 0; c < 2; ++c) v[a][b][c] = lat(ix + a, iy + b, iz + c);
    auto L = [](float p, float q, float t) { return p + (q - p) * t; };
    float x00 = L(v[0][0][0], v[1][0][0], tx), x10 = L(v[0][1][0], v[1][1][0], tx);
    float x01 = L(v[0][0][1], v[1][0][1], tx), x11 = L(v[0][1][1], v[1][1][1], tx);
    return L(L(x00, x10, ty), L(x01, x11, ty), tz);
}

using Mesh = srt::HostMesh;

srt_material lambert(float r, float g, float b)
{
    srt_material m{};
    m.bxdf = srt_bxdf{SRT_BXDF_DIFFUSE, 1.5f, 0.0f, 0.0f, 0.5f, 0.5f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.001f, 0.0f};
    m.base_color[0] = r;
    m.base_color[1] = g;
    m.base_color[2] = b;
    return m;
}

srt_material emitter(float r, float g, float b)
{
    srt_material m = lambert(0.0f, 0.0f, 0.0f);
    float in = std::sqrt(r * r + g * g + b * b);
    m.emission_color[0] = r / in;
    m.emission_color[1] = g / in;
    m.emission_color[2] = b / in;
    m.intensity = in;
    return m;
}

// axis-aligned box of size (sx, sy, sz) standing on y = y0, rotated by
// `deg` about +y (Transform::RotateY, transform.h:301-310), centred (cx, cz)
void add_box(Mesh& m, float cx, float cz, float y0, float sx, float sy, float sz, float deg)
{
    float th = deg * (float)M_PI / 180.0f;
    float c = std::cos(th), s = std::sin(th);
    float P[8][3];
    for (int k = 0; k < 8; ++k) {
        float x = (k & 1 ? 0.5f : -0.5f) * sx, y = (k & 2 ? sy : 0.0f), z = (k & 4 ? 0.5f : -0.5f) * sz;
        P[k][0] = c * x + s * z + cx;
        P[k][1] = y + y0;
        P[k][2] = -s * x + c * z + cz;
    }
    // faces with outward winding
    m.quad(P[0], P[1], P[3], P[2]);  // z-
    m.quad(P[4], P[6], P[7], P[5]);  // z+
    m.quad(P[0], P[4], P[5], P[1]);  // y-
    m.quad(P[2], P[3], P[7], P[6]);  // y+
    m.quad(P[0], P[2], P[6], P[4]);  // x-
    m.quad(P[1], P[5], P[7], P[3]);  // x+
}

void icosphere(int subdiv, std::vector<float>& v, std::vector<uint32_t>& f)
{
    const float t = (1.0f + std::sqrt(5.0f)) / 2.0f;
    float base[12][3] = {{-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
                         {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
    uint32_t faces[20][3] = {{0, 11, 5}, {0, 5, 1},  {0, 1, 7},   {0, 7, 10}, {0, 10, 11}, {1, 5, 9}, {5, 11, 4},
                             {11, 10, 2}, {10, 7, 6}, {7, 1, 8},  {3, 9, 4},  {3, 4, 2},   {3, 2, 6}, {3, 6, 8},
                             {3, 8, 9},  {4, 9, 5},  {2, 4, 11},  {6, 2, 10}, {8, 6, 7},   {9, 8, 1}};
    v.clear();
    f.clear();
    for (auto& p : base) {
        float l = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
        v.push_back(p[0] / l);
        v.push_back(p[1] / l);
        v.push_back(p[2] / l);
    }
    for (auto& q : faces) f.insert(f.end(), q, q + 3);
    for (int s = 0; s < subdiv; ++s) {
        std::unordered_map<uint64_t, uint32_t> mid;
        mid.reserve(f.size());
        auto midpoint = [&](uint32_t a, uint32_t b) {
            uint64_t key = a < b ? ((uint64_t)a << 32 | b) : ((uint64_t)b << 32 | a);
            auto it = mid.find(key);
            if (it != mid.end()) return it->second;
            float p[3];
            for (int k = 0; k < 3; ++k) p[k] = 0.5f * (v[3 * a + k] + v[3 * b + k]);
            float l = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
            uint32_t id = (uint32_t)(v.size() / 3);
            for (int k = 0; k < 3; ++k) v.push_back(p[k] / l);
            mid.emplace(key, id);
            return id;
        };
        std::vector<uint32_t> nf;
        nf.reserve(f.size() * 4);
        for (size_t i = 0; i < f.size(); i += 3) {
            uint32_t a = f[i], b = f[i + 1], c = f[i + 2];
            uint32_t ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
            uint32_t add[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
            nf.insert(nf.end(), add, add + 12);
        }
        f.swap(nf);
    }
}

}  // namespace

namespace {

// Cornell box: [-1,1]^3 open at +z; tall box 0.6x1.2x0.6 rotated +15 deg,
// short box 0.6^3 rotated -18 deg (Disney, roughness 0.5); 0.5x0.5 light
// at y = 0.99 facing -y with Le = (17, 12, 4); pinhole at (0, 0, 3.5)
// looking at the origin, 40 deg vertical fov.
void make_cornell(srt_procedural& p)
{
    p.mats.push_back(lambert(0.725f, 0.725f, 0.725f));  // 0 white
    p.mats.push_back(lambert(0.63f, 0.065f, 0.05f));    // 1 red
    p.mats.push_back(lambert(0.14f, 0.45f, 0.09f));     // 2 green
    srt_material box = lambert(0.725f, 0.725f, 0.725f);
    box.bxdf.type = SRT_BXDF_DISNEY;
    box.bxdf.roughness = 0.5f;
    p.mats.push_back(box);                              // 3 boxes
    p.mats.push_back(emitter(17.0f, 12.0f, 4.0f));      // 4 light

    const float A[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, -1, 1}, {-1, -1, 1},
                           {-1, 1, -1},  {1, 1, -1},  {1, 1, 1},  {-1, 1, 1}};
    Mesh white, red, green, tall, shrt, light;
    white.material = 0;
    red.material = 1;
    green.material = 2;
    tall.material = 3;
    shrt.material = 3;
    light.material = 4;
    white.quad(A[0], A[1], A[2], A[3]);  // floor
    white.quad(A[4], A[7], A[6], A[5]);  // ceiling
    white.quad(A[0], A[4], A[5], A[1]);  // back
    red.quad(A[0], A[3], A[7], A[4]);    // left  x = -1
    green.quad(A[1], A[5], A[6], A[2]);  // right x = +1
    add_box(tall, -0.35f, -0.30f, -1.0f, 0.6f, 1.2f, 0.6f, 15.0f);
    add_box(shrt, 0.35f, 0.35f, -1.0f, 0.6f, 0.6f, 0.6f, -18.0f);
    const float L[4][3] = {{-0.25f, 0.99f, -0.25f}, {0.25f, 0.99f, -0.25f}, {0.25f, 0.99f, 0.25f}, {-0.25f, 0.99f, 0.25f}};
    light.quad(L[0], L[1], L[2], L[3]);  // normal -y
    p.meshes = {white, red, green, tall, shrt, light};
    srt_camera_desc cam{};
    cam.type = SRT_CAMERA_PERSPECTIVE;
    cam.position[2] = 3.5f;
    cam.up[1] = 1.0f;
    cam.fov = 40.0f;
    cam.aspect = 1.0f;
    cam.focal = 1.0f;
    const float env[3] = {0.0f, 0.0f, 0.0f};
    p.has_camera = true;
    p.finish(cam, env);
}

// n_spheres icospheres (subdiv levels), centres U[-10,10]^3, scale U[0.3,2],
// radius 1 + 0.1 * (2 * value_noise - 1); per-sphere Disney parameters drawn
// like the Disney batch points; ground quad at y = -10; four 1x1 lights at
// y = 14 facing down with Le ~ U[5,20]^3; environment 0.05.
void make_spheres(srt_procedural& p, uint64_t seed, int n_spheres, int subdiv)
{
    std::vector<float> uv;
    std::vector<uint32_t> uf;
    icosphere(subdiv, uv, uf);
    p.mats.push_back(lambert(0.5f, 0.5f, 0.5f));  // 0 ground
    for (int k = 0; k < n_spheres; ++k) {
        Pcg32 g;
        g.seed(seed * 1000003ull + (uint64_t)k, 1u);
        float c[3], o[3];
        for (int j = 0; j < 3; ++j) c[j] = -10.0f + 20.0f * g.uniform();
        float sc = 0.3f + 1.7f * g.uniform();
        for (int j = 0; j < 3; ++j) o[j] = 100.0f * g.uniform();
        srt_material m = lambert(g.uniform(), g.uniform(), g.uniform());
        m.bxdf.type = SRT_BXDF_DISNEY;
        m.bxdf.ior = 1.5f;
        m.bxdf.metallic = g.uniform();
        m.bxdf.subsurface = g.uniform();
        m.bxdf.specular = g.uniform();
        m.bxdf.specularTint = g.uniform();
        m.bxdf.anisotropic = g.uniform();
        m.bxdf.sheen = g.uniform();
        m.bxdf.sheenTint = g.uniform();
        m.bxdf.clearcoat = g.uniform();
        m.bxdf.clearcoatGloss = g.uniform();
        m.bxdf.roughness = 0.05f + 0.95f * g.uniform();
        m.bxdf.specTrans = 0.0f;
        p.mats.push_back(m);
        Mesh s;
        s.material = (int)p.mats.size() - 1;
        s.idx = uf;
        s.v.resize(uv.size());
        uint32_t nseed = hash32((uint32_t)seed ^ hash32((uint32_t)k));
        for (size_t i = 0; i < uv.size(); i += 3) {
            float x = uv[i], y = uv[i + 1], z = uv[i + 2];
            float r = 1.0f + 0.1f * (2.0f * value_noise(3.0f * x + o[0], 3.0f * y + o[1], 3.0f * z + o[2], nseed) - 1.0f);
            s.v[i] = c[0] + sc * r * x;
            s.v[i + 1] = c[1] + sc * r * y;
            s.v[i + 2] = c[2] + sc * r * z;
        }
        p.meshes.push_back(std::move(s));
    }
    Mesh ground;
    ground.material = 0;
    const float G[4][3] = {{-40, -10, -40}, {-40, -10, 40}, {40, -10, 40}, {40, -10, -40}};
    ground.quad(G[0], G[1], G[2], G[3]);  // normal +y
    p.meshes.push_back(ground);
    Pcg32 g;
    g.seed(seed * 1000003ull + 999999ull, 2u);
    for (int l = 0; l < 4; ++l) {
        float x = -8.0f + 16.0f * g.uniform(), z = -8.0f + 16.0f * g.uniform();
        float le[3];
        for (int j = 0; j < 3; ++j) le[j] = 5.0f + 15.0f * g.uniform();
        p.mats.push_back(emitter(le[0], le[1], le[2]));
        Mesh m;
        m.material = (int)p.mats.size() - 1;
        const float Q[4][3] = {{x - 0.5f, 14.0f, z - 0.5f}, {x + 0.5f, 14.0f, z - 0.5f},
                               {x + 0.5f, 14.0f, z + 0.5f}, {x - 0.5f, 14.0f, z + 0.5f}};
        m.quad(Q[0], Q[1], Q[2], Q[3]);  // normal -y
        p.meshes.push_back(m);
    }
    srt_camera_desc cam{};
    cam.type = SRT_CAMERA_PERSPECTIVE;
    cam.position[0] = 0.0f;
    cam.position[1] = 6.0f;
    cam.position[2] = 38.0f;
    cam.target[1] = -1.0f;
    cam.up[1] = 1.0f;
    cam.fov = 40.0f;
    cam.aspect = 16.0f / 9.0f;
    cam.focal = 1.0f;
    const float env[3] = {0.05f, 0.05f, 0.05f};
    p.has_camera = true;
    p.finish(cam, env);
}

}  // namespace

extern "C" srt_status srt_procedural_create(const char* name, uint64_t seed, int32_t n_spheres, int32_t subdiv,
                                            srt_procedural** out)
{
    srt::clear_error();
    if (!name || !out) return srt::set_error(SRT_ERR_ARG, "NULL argument");
    *out = nullptr;
    std::string n(name);
    srt_procedural* p = new (std::nothrow) srt_procedural();
    if (!p) return srt::set_error(SRT_ERR_OOM, "host allocation failed");
    if (n == "cornell") {
        make_cornell(*p);
    } else if (n == "spheres") {
        if (n_spheres < 0 || n_spheres > 4096 || subdiv < 0 || subdiv > 8) {
            delete p;
            return srt::set_error(SRT_ERR_ARG, "spheres: n_spheres in [0, 4096], subdiv in [0, 8]");
        }
        make_spheres(*p, seed, n_spheres, subdiv);
    } else {
        delete p;
        return srt::set_error(SRT_ERR_NOT_FOUND, "unknown procedural scene: " + n);
    }
    *out = p;
    return SRT_OK;
}

extern "C" srt_status srt_procedural_desc(const srt_procedural* p, srt_scene_desc* desc)
{
    srt::clear_error();
    if (!p || !desc) return srt::set_error(SRT_ERR_ARG, "NULL argument");
    *desc = p->desc;
    return SRT_OK;
}

extern "C" void srt_procedural_destroy(srt_procedural* p) { delete p; }
