// srt — command-line renderer (src/main/main.cu): reads a JSON config with
// "render", "passes" and "scene" sections, lets -r / -p / -s replace a
// section with the contents of another file, renders once with the image
// renderer and saves render.output next to the config file; a scene file
// named by scene.model is found next to the config file too.  Uses only the
// library's C ABI (include/srt.h).
//
//   srt -c config.json [-r render.json] [-p passes.json] [-s scene.json]
#include <chrono>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>

#include "srt.h"

static bool read_file(const std::string& path, std::string& out)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::ostringstream s;
    s << f.rdbuf();
    out = s.str();
    return true;
}

static int fail(const char* what)
{
    std::fprintf(stderr, "ERROR::%s: %s\n", what, srt_last_error());
    return 1;
}

int main(int argc, char* argv[])
{
    std::string paths[4];  // config, render, passes, scene
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        const int k = (a == "-c" || a == "--config")   ? 0
                      : (a == "-r" || a == "--render") ? 1
                      : (a == "-p" || a == "--passes") ? 2
                      : (a == "-s" || a == "--scene")  ? 3
                                                       : -1;
        if (a == "-h" || a == "--help" || k < 0 || i + 1 >= argc) {
            std::printf("usage: %s -c config.json [-r render.json] [-p passes.json] [-s scene.json]\n", argv[0]);
            return (a == "-h" || a == "--help") ? 0 : 1;
        }
        paths[k] = argv[++i];
    }
    if (paths[0].empty()) {
        std::fprintf(stderr, "ERROR::no config file (-c)\n");
        return 1;
    }
    std::string text[4];
    for (int k = 1; k < 4; ++k)
        if (!paths[k].empty() && !read_file(paths[k], text[k])) {
            std::fprintf(stderr, "ERROR::Failed to open file: %s\n", paths[k].c_str());
            return 1;
        }
    auto opt = [&](int k) { return paths[k].empty() ? nullptr : text[k].c_str(); };
    srt_renderer* r = nullptr;
    if (srt_renderer_create_file(paths[0].c_str(), opt(1), opt(2), opt(3), &r) != SRT_OK) return fail("config");
    const auto t0 = std::chrono::steady_clock::now();
    if (srt_renderer_run(r, 1) != SRT_OK) return fail("render");
    const auto t1 = std::chrono::steady_clock::now();
    std::printf("Render: %.3f ms\n", std::chrono::duration<double, std::milli>(t1 - t0).count());
    std::string out = srt_renderer_output(r);
    if (!out.empty()) {
        const size_t slash = paths[0].find_last_of('/');
        const std::string dir = slash == std::string::npos ? std::string() : paths[0].substr(0, slash + 1);
        if (out[0] != '/') out = dir + out;
        if (srt_renderer_save(r, out.c_str()) != SRT_OK) return fail("save");
        const auto t2 = std::chrono::steady_clock::now();
        std::printf("Save: %.3f ms -> %s\n", std::chrono::duration<double, std::milli>(t2 - t1).count(), out.c_str());
    }
    srt_renderer_destroy(r);
    return 0;
}
