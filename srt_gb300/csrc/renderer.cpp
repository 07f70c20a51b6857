// renderer.cpp — PathTracer / Wavefront / Accumulate / ToneMapping / Measure
// passes, the renderer that loads a JSON config, and their C ABI.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <random>
#include <sstream>
#include <vector>

#include "common.h"
#include "host_scene.h"
#include "renderpass.h"

namespace srt {

// ---- Film / Scene ----------------------------------------------------------

Film::~Film()
{
    if (pixels_) cudaFree(pixels_);
}

srt_status Film::allocate()
{
    size_t bytes = (size_t)width_ * height_ * 16;
    SRT_CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&pixels_), bytes));
    SRT_CUDA_TRY(cudaMemset(pixels_, 0, bytes));
    return SRT_OK;
}

Scene::~Scene()
{
    if (handle) srt_scene_destroy(handle);
    if (proc) srt_procedural_destroy(proc);
}

// ---- factory ----------------------------------------------------------------

std::unordered_map<std::string, RenderPassFactory::Creator>& RenderPassFactory::get_map()
{
    static std::unordered_map<std::string, Creator> map;
    return map;
}

srt_status RenderPassFactory::create_pass(const std::string& name, const Json& params,
                                          std::shared_ptr<RenderPass>& out)
{
    auto& map = get_map();
    auto it = map.find(name);
    if (it == map.end()) return set_error(SRT_ERR_NOT_FOUND, "Render pass " + name + " not found!");
    out = it->second(params);
    return SRT_OK;
}

std::string RenderPassFactory::registered_passes()
{
    std::vector<std::string> names;
    for (auto& kv : get_map()) names.push_back(kv.first);
    std::sort(names.begin(), names.end());
    std::string s;
    for (auto& n : names) s += (s.empty() ? "" : ";") + n;
    return s;
}

// host frame seed: random_int(0, INT32_MAX) from a static
// std::default_random_engine(0) (src/device_include/math/random.h:49-63)
static int host_random_int(int lo, int hi)
{
    static std::default_random_engine g(0);
    static std::uniform_real_distribution<float> d(0, 1);
    return lo + d(g) * (hi - lo);
}

// ---- PathTracer (src/passes/integrator/path_tracer.{h,cu}) -------------------

class PathTracer : public RenderPass {
public:
    explicit PathTracer(const Json& j)
    {
        if (j.is_null()) return;
        samples_per_pixel = (int)j.number("samples_per_pixel", 1);
        max_depth = (int)j.number("max_depth", 16);
        rr_depth = (int)j.number("rr_depth", 4);
        use_nee = j.boolean("use_nee", true);
        use_mis = j.boolean("use_mis", true);
    }
    ~PathTracer() override
    {
        if (pt) srt_pt_destroy(pt);
    }
    srt_status init() override { return srt_pt_create(scene->handle, width, height, &pt); }
    srt_status render(std::shared_ptr<Film> film) override
    {
        if (!enable) return SRT_OK;
        srt_pt_params p{};
        p.samples_per_pixel = samples_per_pixel;
        p.max_depth = max_depth;
        p.rr_depth = rr_depth;
        p.use_nee = use_nee;
        p.use_mis = use_mis;
        p.seed = host_random_int(0, INT32_MAX);
        p.rng_mode = SRT_RNG_CURAND;
        p.flags = 0;
        return srt_pt_render(pt, film->get_pixels(), &p, nullptr);
    }

protected:
    srt_pt* pt = nullptr;
    int samples_per_pixel = 1, max_depth = 16, rr_depth = 4;
    bool use_nee = true, use_mis = true;
    static RenderPassFactory::Register<PathTracer> reg;
};
RenderPassFactory::Register<PathTracer> PathTracer::reg("PathTracer");

// The reference's queue-based pass (src/passes/wavefront/wavefront.cu) is
// served by the same wavefront engine with the megakernel's semantics.
class Wavefront : public PathTracer {
public:
    explicit Wavefront(const Json& j) : PathTracer(j) {}
    static RenderPassFactory::Register<Wavefront> reg;
};
RenderPassFactory::Register<Wavefront> Wavefront::reg("Wavefront");

// ---- LightTracer (src/passes/integrator/light_tracer.{h,cu}) -----------------

class LightTracer : public RenderPass {
public:
    explicit LightTracer(const Json& j)
    {
        if (j.is_null()) return;
        samples_per_pixel = (int)j.number("samples_per_pixel", 1);
        max_depth = (int)j.number("max_depth", 16);
        rr_depth = (int)j.number("rr_depth", 4);
    }
    srt_status render(std::shared_ptr<Film> film) override
    {
        if (!enable) return SRT_OK;
        srt_pt_params p{};
        p.samples_per_pixel = samples_per_pixel;
        p.max_depth = max_depth;
        p.rr_depth = rr_depth;
        p.seed = host_random_int(0, INT32_MAX);
        p.rng_mode = SRT_RNG_CURAND;
        return srt_lt_render(scene->handle, width, height, film->get_pixels(), &p, nullptr, nullptr);
    }

private:
    int samples_per_pixel = 1, max_depth = 16, rr_depth = 4;
    static RenderPassFactory::Register<LightTracer> reg;
};
RenderPassFactory::Register<LightTracer> LightTracer::reg("LightTracer");

// ---- NeuralRadiosity (src/passes/npr/neural_radiosity.{h,cu}) ----------------

class NeuralRadiosity : public RenderPass {
public:
    explicit NeuralRadiosity(const Json& j)
    {
        if (j.is_null()) return;
        type = j.string("type", "LHS") == "RHS" ? SRT_NR_RHS : SRT_NR_LHS;
        samples_per_pixel = (int)j.number("samples_per_pixel", 1);
        train_model = j.boolean("train_model", false);
        model_path = j.string("model_path", "");
    }
    ~NeuralRadiosity() override
    {
        if (nr) srt_nr_destroy(nr);
    }
    srt_status init() override
    {
        SRT_TRY(srt_nr_create(0, &nr));
        // load_model: a missing file leaves the initialised network (neural_radiosity.cu:60-70)
        if (!model_path.empty()) {
            std::ifstream probe(model_path, std::ios::binary);
            if (probe) SRT_TRY(srt_nr_load(nr, model_path.c_str()));
        }
        return SRT_OK;
    }
    srt_status render(std::shared_ptr<Film> film) override
    {
        if (!enable) return SRT_OK;
        if (train_model && !model_path.empty()) SRT_TRY(srt_nr_save(nr, model_path.c_str()));  // train() = save_model
        std::vector<int32_t> seeds((size_t)std::max(samples_per_pixel, 0));
        for (int32_t& s : seeds) s = host_random_int(0, INT32_MAX);
        return srt_nr_render(scene->handle, nr, width, height, type, samples_per_pixel, seeds.data(),
                             film->get_pixels(), nullptr);
    }

private:
    srt_nr* nr = nullptr;
    int type = SRT_NR_LHS, samples_per_pixel = 1;
    bool train_model = false;
    std::string model_path;
    static RenderPassFactory::Register<NeuralRadiosity> reg;
};
RenderPassFactory::Register<NeuralRadiosity> NeuralRadiosity::reg("NeuralRadiosity");

// ---- Accumulate (src/passes/postprocess/accumulate.{h,cu}) -----------------

class Accumulate : public RenderPass {
public:
    explicit Accumulate(const Json&) {}
    ~Accumulate() override
    {
        if (acc) cudaFree(acc);
    }
    srt_status init() override
    {
        size_t bytes = (size_t)width * height * 16;
        SRT_CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&acc), bytes));
        SRT_CUDA_TRY(cudaMemset(acc, 0, bytes));
        return SRT_OK;
    }
    srt_status render(std::shared_ptr<Film> film) override
    {
        if (!enable || !scene->is_static()) {
            frame_count = 0;
            return SRT_OK;
        }
        SRT_TRY(srt_film_accumulate(film->get_pixels(), acc, (int64_t)width * height, frame_count, nullptr));
        SRT_CUDA_TRY(cudaDeviceSynchronize());
        frame_count++;
        return SRT_OK;
    }

private:
    int frame_count = 0;
    float* acc = nullptr;
    static RenderPassFactory::Register<Accumulate> reg;
};
RenderPassFactory::Register<Accumulate> Accumulate::reg("Accumulate");

// ---- ToneMapping (src/passes/postprocess/tonemapping.{h,cu}) ---------------

class ToneMapping : public RenderPass {
public:
    explicit ToneMapping(const Json& j)
    {
        if (j.is_null()) return;
        std::string t = j.string("type", "None");
        type = t == "Clamp" ? SRT_TONE_CLAMP
             : t == "Reinhard" ? SRT_TONE_REINHARD
             : t == "Uncharted2" ? SRT_TONE_UNCHARTED2
             : t == "ACES" ? SRT_TONE_ACES
             : SRT_TONE_NONE;
        exposure = (float)j.number("exposure", 0.0);
        use_gamma = j.boolean("use_gamma", true);
    }
    srt_status render(std::shared_ptr<Film> film) override
    {
        if (!enable) return SRT_OK;
        SRT_TRY(srt_film_tonemap(film->get_pixels(), (int64_t)width * height, type, exposure, use_gamma, nullptr));
        SRT_CUDA_TRY(cudaDeviceSynchronize());
        return SRT_OK;
    }

private:
    int type = SRT_TONE_NONE;
    float exposure = 0.0f;
    bool use_gamma = true;
    static RenderPassFactory::Register<ToneMapping> reg;
};
RenderPassFactory::Register<ToneMapping> ToneMapping::reg("ToneMapping");

// ---- Measure (src/passes/postprocess/measure.{h,cu}); reference image: exr, hdr or pfm

class Measure : public RenderPass {
public:
    explicit Measure(const Json& j)
    {
        ref_path = j.string("ref_path", "");
        std::string t = j.string("type", "MSE");
        type = t == "MAPE" ? SRT_METRIC_MAPE : t == "SMAPE" ? SRT_METRIC_SMAPE : t == "RelMSE" ? SRT_METRIC_RELMSE
                                                                                                   : SRT_METRIC_MSE;
        discard = (float)j.number("discard", 0.1);
        const std::string o = j.string("option", "None");  // Measure::string_to_option
        option = o == "Reference" ? SRT_MEASURE_REFERENCE : o == "Error" ? SRT_MEASURE_ERROR : SRT_MEASURE_NONE;
    }
    ~Measure() override
    {
        if (ref) cudaFree(ref);
        if (scratch) cudaFree(scratch);
    }
    srt_status init() override
    {
        if (ref_path.empty()) return set_error(SRT_ERR_ARG, "Measure: no ref_path specified");
        // Image::load_from_file(ref_path, true, true) of a float image (measure.cu:5-16)
        int32_t w = 0, h = 0;
        srt_status st = srt_image_read(ref_path.c_str(), &w, &h, nullptr, 1);
        if (st != SRT_OK || w != width || h != height)
            return set_error(st == SRT_OK || st == SRT_ERR_UNSUPPORTED ? SRT_ERR_ARG : st,
                             "Measure: reference image size or format not match (" + ref_path + ")");
        std::vector<float> rgba((size_t)w * h * 4);
        SRT_TRY(srt_image_read(ref_path.c_str(), &w, &h, rgba.data(), 1));
        size_t n = (size_t)w * h;
        SRT_CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&ref), n * 16));
        SRT_CUDA_TRY(cudaMemcpy(ref, rgba.data(), n * 16, cudaMemcpyHostToDevice));
        SRT_CUDA_TRY(cudaMalloc(&scratch, srt_film_metric_scratch_bytes((int64_t)n)));
        return SRT_OK;
    }
    srt_status render(std::shared_ptr<Film> film) override
    {
        if (!enable) return SRT_OK;
        SRT_TRY(srt_film_metric(film->get_pixels(), ref, (int64_t)width * height, type, discard, scratch, &error,
                                nullptr));
        SRT_TRY(srt_film_measure_view(film->get_pixels(), ref, (int64_t)width * height, type, option, nullptr));
        if (!online) {
            std::printf("%s error: %g\n\n", type_name(), (double)error);
            std::fflush(stdout);  // the reference ends the line with endl
        }
        return SRT_OK;
    }
    const char* type_name() const
    {
        return type == SRT_METRIC_MAPE ? "MAPE" : type == SRT_METRIC_SMAPE ? "SMAPE" : type == SRT_METRIC_RELMSE ? "RelMSE" : "MSE";
    }

private:
    std::string ref_path;
    int type = SRT_METRIC_MSE;
    int option = SRT_MEASURE_NONE;
    float discard = 0.1f, error = 0.0f;
    float* ref = nullptr;
    void* scratch = nullptr;
    static RenderPassFactory::Register<Measure> reg;
};
RenderPassFactory::Register<Measure> Measure::reg("Measure");

// ---- Renderer -----------------------------------------------------------------

static bool vec3(const Json* j, float out[3])
{
    if (!j || !j->is_array() || j->arr.size() != 3) return false;
    for (int k = 0; k < 3; ++k) out[k] = (float)j->arr[k].num;
    return true;
}

srt_status Renderer::load_scene(const Json& config)
{
    std::string model = config.string("model", "");
    const std::string pre = "procedural:";
    scene = std::make_shared<Scene>();
    if (model.compare(0, pre.size(), pre) == 0) {
        std::vector<std::string> parts;
        std::stringstream ss(model.substr(pre.size()));
        std::string tok;
        while (std::getline(ss, tok, ':')) parts.push_back(tok);
        if (parts.empty()) return set_error(SRT_ERR_ARG, "empty procedural scene name");
        int n_spheres = parts.size() > 1 ? std::atoi(parts[1].c_str()) : 64;
        int subdiv = parts.size() > 2 ? std::atoi(parts[2].c_str()) : 6;
        uint64_t seed = parts.size() > 3 ? std::strtoull(parts[3].c_str(), nullptr, 10) : 1;
        SRT_TRY(srt_procedural_create(parts[0].c_str(), seed, n_spheres, subdiv, &scene->proc));
    } else {
        // a scene file beside the config (renderer.cu:44-63): the pbrt film
        // size stands in for an unset resolution
        if (model.empty()) return set_error(SRT_ERR_ARG, "scene.model is empty");
        const std::string path = model[0] == '/' ? model : base_dir + model;
        SRT_TRY(srt_import_scene(path.c_str(), &scene->proc));
        if ((width == 0 || height == 0) && scene->proc->width > 0 && scene->proc->height > 0) {
            width = scene->proc->width;
            height = scene->proc->height;
        }
    }
    if (width == 0 || height == 0) {
        width = 1920;
        height = 1080;
    }
    const Json* env = config.find("environment");
    if (env && env->string("type", "constant") == "uvmap") {
        // a "uvmap" environment image beside the config (renderer.cu:155-161), loaded unflipped
        const std::string rel = env->string("path", "");
        if (rel.empty()) return set_error(SRT_ERR_ARG, "environment uvmap needs a path");
        HostTexture t;
        t.name = "environment";
        SRT_TRY(load_texture_image(rel[0] == '/' ? rel : base_dir + rel, false, t));
        scene->proc->textures.push_back(std::move(t));
        scene->proc->env_map = (int32_t)scene->proc->textures.size();
        scene->proc->sync_textures();
    }
    srt_scene_desc desc;
    SRT_TRY(srt_procedural_desc(scene->proc, &desc));
    desc.camera.aspect = (float)width / (float)height;
    if (!scene->proc->has_camera && !config.find("camera")) return set_error(SRT_ERR_ARG, "No camera specified");
    if (const Json* cam = config.find("camera")) {
        float pos[3], tgt[3], up[3];
        if (!vec3(cam->find("position"), pos) || !vec3(cam->find("target"), tgt) || !vec3(cam->find("up"), up))
            return set_error(SRT_ERR_ARG, "camera needs position, target and up");
        std::string t = cam->string("type", "perspective");
        if (t == "perspective")
            desc.camera.type = SRT_CAMERA_PERSPECTIVE;
        else if (t == "orthographic")
            desc.camera.type = SRT_CAMERA_ORTHOGRAPHIC;
        else
            return set_error(SRT_ERR_UNSUPPORTED, "Unknown or unsupported camera type: " + t);
        std::memcpy(desc.camera.position, pos, 12);
        std::memcpy(desc.camera.target, tgt, 12);
        std::memcpy(desc.camera.up, up, 12);
        desc.camera.fov = (float)cam->number("fov", 60.0);
    }
    if (env) {
        std::string t = env->string("type", "constant");
        if (t == "constant") {
            if (!vec3(env->find("color"), desc.env_color)) return set_error(SRT_ERR_ARG, "environment needs color");
        } else if (t != "uvmap") {
            return set_error(SRT_ERR_ARG, "Unknown environment type: " + t);
        }
    }
    SRT_TRY(srt_scene_create(&desc, &scene->handle));
    film = std::make_shared<Film>(width, height);
    return film->allocate();
}

srt_status Renderer::load_passes(const Json& config)
{
    if (!config.is_array()) return set_error(SRT_ERR_PARSE, "passes must be an array");
    for (const Json& c : config.arr) {
        std::string name = c.string("name", "");
        const Json* params = c.find("params");
        static const Json null_json;
        std::shared_ptr<RenderPass> pass;
        SRT_TRY(RenderPassFactory::create_pass(name, params ? *params : null_json, pass));
        pass->set_enable(c.boolean("enable", true));
        pass->set_online(false);
        pass->resize(width, height);
        pass->set_scene(scene);
        SRT_TRY(pass->init());
        passes.push_back(pass);
    }
    return SRT_OK;
}

srt_status Renderer::load(const Json& config)
{
    const Json* render = config.find("render");
    if (render) {
        const Json* res = render->find("resolution");
        if (res && res->is_array() && res->arr.size() == 2) {
            width = (int)res->arr[0].num;
            height = (int)res->arr[1].num;
        }
        output = render->string("output", "");
        std::string type = render->string("type", "image");
        if (type != "image") return set_error(SRT_ERR_UNSUPPORTED, "only the image renderer is built (no GUI / video)");
    }
    if (width < 0 || height < 0) return set_error(SRT_ERR_ARG, "negative resolution");
    const Json* sc = config.find("scene");
    if (!sc) return set_error(SRT_ERR_ARG, "config has no scene");
    SRT_TRY(load_scene(*sc));
    const Json* ps = config.find("passes");
    if (!ps) return set_error(SRT_ERR_ARG, "config has no passes");
    return load_passes(*ps);
}

srt_status Renderer::run(int frames)
{
    for (int f = 0; f < frames; ++f)
        for (auto& p : passes) SRT_TRY(p->render(film));
    SRT_CUDA_TRY(cudaDeviceSynchronize());
    return SRT_OK;
}

}  // namespace srt

using namespace srt;

struct srt_renderer {
    Renderer r;
};

namespace {

srt_status create_renderer(const char* json_config, const std::string& base_dir, const char* render,
                           const char* passes, const char* scene, srt_renderer** out)
{
    if (!json_config || !out) return set_error(SRT_ERR_ARG, "NULL argument");
    *out = nullptr;
    Json cfg;
    std::string err;
    if (!Json::parse(json_config, cfg, err)) return set_error(SRT_ERR_PARSE, "config: " + err);
    if (!cfg.is_object()) return set_error(SRT_ERR_PARSE, "config: not a JSON object");
    // each given section replaces the config's (src/main/main.cu:57-62)
    const std::pair<const char*, const char*> over[3] = {{"render", render}, {"passes", passes}, {"scene", scene}};
    for (const auto& o : over) {
        if (!o.second) continue;
        Json sec;
        if (!Json::parse(o.second, sec, err)) return set_error(SRT_ERR_PARSE, std::string(o.first) + ": " + err);
        bool found = false;
        for (auto& kv : cfg.obj)
            if (kv.first == o.first) {
                kv.second = sec;
                found = true;
            }
        if (!found) cfg.obj.emplace_back(o.first, sec);
    }
    srt_renderer* r = new (std::nothrow) srt_renderer();
    if (!r) return set_error(SRT_ERR_OOM, "host allocation failed");
    r->r.base_dir = base_dir;
    srt_status st = r->r.load(cfg);
    if (st != SRT_OK) {
        delete r;
        return st;
    }
    *out = r;
    return SRT_OK;
}

}  // namespace

extern "C" srt_status srt_renderer_create(const char* json_config, srt_renderer** out)
{
    clear_error();
    return create_renderer(json_config, "", nullptr, nullptr, nullptr, out);
}

extern "C" srt_status srt_renderer_create_ex(const char* json_config, const char* render, const char* passes,
                                             const char* scene, srt_renderer** out)
{
    clear_error();
    return create_renderer(json_config, "", render, passes, scene, out);
}

extern "C" srt_status srt_renderer_create_file(const char* config_path, const char* render, const char* passes,
                                               const char* scene, srt_renderer** out)
{
    clear_error();
    if (!config_path || !out) return set_error(SRT_ERR_ARG, "NULL argument");
    std::ifstream f(config_path, std::ios::binary);
    if (!f) return set_error(SRT_ERR_ARG, std::string("Failed to open file: ") + config_path);
    std::ostringstream text;
    text << f.rdbuf();
    const std::string p(config_path);
    const size_t slash = p.find_last_of('/');
    return create_renderer(text.str().c_str(), slash == std::string::npos ? std::string() : p.substr(0, slash + 1),
                           render, passes, scene, out);
}

extern "C" srt_status srt_renderer_run(srt_renderer* r, int32_t frames)
{
    clear_error();
    if (!r || frames < 0) return set_error(SRT_ERR_ARG, "bad arguments");
    return r->r.run(frames);
}

extern "C" srt_status srt_renderer_size(const srt_renderer* r, int32_t* w, int32_t* h)
{
    clear_error();
    if (!r || !w || !h) return set_error(SRT_ERR_ARG, "NULL argument");
    *w = r->r.width;
    *h = r->r.height;
    return SRT_OK;
}

extern "C" srt_status srt_renderer_read_film(const srt_renderer* r, float* host_rgba)
{
    clear_error();
    if (!r || !host_rgba) return set_error(SRT_ERR_ARG, "NULL argument");
    size_t bytes = (size_t)r->r.width * r->r.height * 16;
    SRT_CUDA_TRY(cudaMemcpy(host_rgba, r->r.film->get_pixels(), bytes, cudaMemcpyDeviceToHost));
    return SRT_OK;
}

extern "C" srt_status srt_renderer_save_pfm(const srt_renderer* r, const char* path)
{
    clear_error();
    if (!r || !path) return set_error(SRT_ERR_ARG, "NULL argument");
    int w = r->r.width, h = r->r.height;
    std::vector<float> rgba((size_t)w * h * 4);
    SRT_TRY(srt_renderer_read_film(r, rgba.data()));
    std::ofstream f(path, std::ios::binary);
    if (!f) return set_error(SRT_ERR_ARG, std::string("cannot open ") + path);
    f << "PF\n" << w << " " << h << "\n-1.0\n";
    std::vector<float> rgb((size_t)w * h * 3);
    for (size_t i = 0; i < (size_t)w * h; ++i)
        for (int c = 0; c < 3; ++c) rgb[3 * i + c] = rgba[4 * i + c];
    f.write(reinterpret_cast<const char*>(rgb.data()), (std::streamsize)(rgb.size() * 4));
    return f ? SRT_OK : set_error(SRT_ERR_ARG, "write failed");
}

extern "C" const char* srt_renderer_output(const srt_renderer* r) { return r ? r->r.output.c_str() : ""; }

extern "C" srt_status srt_renderer_save(const srt_renderer* r, const char* path)
{
    clear_error();
    if (!r || !path) return set_error(SRT_ERR_ARG, "NULL argument");
    std::vector<float> rgba((size_t)r->r.width * r->r.height * 4);
    SRT_TRY(srt_renderer_read_film(r, rgba.data()));
    return srt_image_write(path, r->r.width, r->r.height, rgba.data(), 1);
}

extern "C" void srt_renderer_destroy(srt_renderer* r) { delete r; }

extern "C" const char* srt_registered_passes(void)
{
    static std::string s = RenderPassFactory::registered_passes();
    return s.c_str();
}
