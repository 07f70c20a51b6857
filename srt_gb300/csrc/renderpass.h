// renderpass.h — the render-pass plugin layer (src/passes/renderpass.h:10-80,
// src/passes/film.h:7-19, src/renderer/renderer.h:22-42) on top of the C ABI.
//
// Same names and JSON keys as the reference: passes are registered by name
// in a static factory and created from {"name": ..., "enable": ...,
// "params": {...}}; an unknown name is SRT_ERR_NOT_FOUND instead of exit(-1).
#pragma once

#include <functional>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/srt.h"
#include "json.h"

namespace srt {

// Film: device float4[w*h], row-major idx = iy*w + ix (film.h:7-19).
class Film {
public:
    Film(int w, int h) : width_(w), height_(h) {}
    ~Film();
    srt_status allocate();
    int get_width() const { return width_; }
    int get_height() const { return height_; }
    float* get_pixels() { return pixels_; }

private:
    int width_, height_;
    float* pixels_ = nullptr;
};

// Scene: host description (procedural generator) + resident device scene.
class Scene {
public:
    ~Scene();
    srt_procedural* proc = nullptr;
    srt_scene* handle = nullptr;
    bool moved = false;
    bool is_static() const { return !moved; }
};

class RenderPass {
public:
    virtual ~RenderPass() = default;
    void set_enable(bool e) { enable = e; }
    void set_online(bool o) { online = o; }
    void resize(int w, int h)
    {
        width = w;
        height = h;
    }
    void set_scene(std::shared_ptr<Scene> s) { scene = std::move(s); }

    virtual srt_status init() { return SRT_OK; }
    virtual srt_status render(std::shared_ptr<Film> film) = 0;
    virtual void update() {}
    virtual void render_ui() {}

protected:
    bool enable = true;
    bool online = false;
    int width = 0, height = 0;
    std::shared_ptr<Scene> scene;
};

class RenderPassFactory {
public:
    using Creator = std::function<std::shared_ptr<RenderPass>(const Json&)>;
    static std::unordered_map<std::string, Creator>& get_map();

    template <class T>
    struct Register {
        explicit Register(const std::string& name)
        {
            get_map().emplace(name, [](const Json& params) { return std::make_shared<T>(params); });
        }
    };

    static srt_status create_pass(const std::string& name, const Json& params, std::shared_ptr<RenderPass>& out);
    static std::string registered_passes();
};

// Renderer::load_scene / load_passes / ImageRenderer::run (renderer.cu:3-191).
class Renderer {
public:
    srt_status load(const Json& config);
    srt_status run(int frames);
    int width = 0, height = 0;
    std::string output;  // render.output: image file name, relative to the config file
    std::string base_dir;  // directory of the config file ("" or ending in '/'): scene files resolve against it
    std::shared_ptr<Scene> scene;
    std::shared_ptr<Film> film;
    std::vector<std::shared_ptr<RenderPass>> passes;

private:
    srt_status load_scene(const Json& config);
    srt_status load_passes(const Json& config);
};

}  // namespace srt
