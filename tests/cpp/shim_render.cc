// Renders through the C++ renderer layer the way a host application written
// against the reference's IRenderer / RendererFactory would:
//   shim_render <dataset_dir> <config.json> <out_prefix>
// writes <out_prefix>.offline.rgba and <out_prefix>.realtime.rgba (raw RGBA8,
// width x height from the config), then updates one parameter and renders
// <out_prefix>.updated.rgba.  Exit status 0 on success.
#include <cstdio>
#include <fstream>
#include <string>

#include "hydrant_gb300_renderer.hpp"

static bool dump(const hygb::Image &img, const std::string &path) {
    std::ofstream os(path, std::ios::binary);
    os.write(reinterpret_cast<const char *>(img.rgba.data()), std::streamsize(img.rgba.size()));
    return bool(os);
}

int main(int argc, char **argv) {
    if (argc != 4) {
        std::fprintf(stderr, "usage: %s <dataset_dir> <config.json> <out_prefix>\n", argv[0]);
        return 2;
    }
    try {
        const hygb::Config cfg = hygb::Config::from_file(argv[2]);
        hygb::RendererFactory factory(argv[1]);
        auto renderer = factory.create(cfg.render);
        const std::string out = argv[3];
        if (!dump(renderer->offline_render(cfg.camera), out + ".offline.rgba")) return 1;
        if (!dump(renderer->realtime_render(cfg.camera), out + ".realtime.rgba")) return 1;
        renderer->update(hygb::json::parse(R"({"clear_color": [0.25, 0.5, 1.0]})"));
        if (!dump(renderer->offline_render(cfg.camera), out + ".updated.rgba")) return 1;
    } catch (const std::exception &e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
