// Renders through the C++ renderer layer the way a host application written
// against the reference's IRenderer / RendererFactory would:
//   shim_render <dataset_dir> <config.json> <out_prefix>
// writes <out_prefix>.offline.rgba and <out_prefix>.realtime.rgba (raw RGBA8,
// width x height from the config), drives two three-frame realtime sessions
// through IRenderLoop (Dynamic and Lossless quality; the first two frames at a
// moved camera, the last at the configured one) and writes their last frames
// as <out_prefix>.loop_dynamic.rgba / .loop_lossless.rgba with the callback
// counts on stdout, then updates one parameter and renders
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

// A session in the shape of the reference's (slave.cc: Session : IRenderLoop):
// three frames, the camera moved by the loop between them.
struct SessionLoop : hygb::IRenderLoop {
    explicit SessionLoop(const hygb::CameraConfig &c) : IRenderLoop(c), base(c) {}
    void post_loop() override { ++post_loop_n; }
    bool should_stop() override { return frames >= 3; }
    void post_frame() override {
        ++post_frame_n;
        camera = base;
        if (frames < 2) camera.arm[0] += 10.f * float(frames + 1);
    }
    void on_frame(hygb::Image &frame) override {
        ++frames;
        last = frame;
    }
    void after_frame() override { ++after_frame_n; }
    void after_loop() override { ++after_loop_n; }

    hygb::CameraConfig base;
    hygb::Image last;
    int post_loop_n = 0, post_frame_n = 0, frames = 0, after_frame_n = 0, after_loop_n = 0;
};

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
        for (int lossless = 0; lossless < 2; ++lossless) {
            SessionLoop loop(cfg.camera);
            hygb::RealtimeRenderOptions opts;
            opts.quality = lossless ? hygb::RealtimeRenderQuality::Lossless
                                    : hygb::RealtimeRenderQuality::Dynamic;
            renderer->realtime_render(loop, opts);
            std::printf("loop %s post_loop=%d post_frame=%d frames=%d after_frame=%d after_loop=%d\n",
                        lossless ? "lossless" : "dynamic", loop.post_loop_n, loop.post_frame_n,
                        loop.frames, loop.after_frame_n, loop.after_loop_n);
            if (!dump(loop.last, out + (lossless ? ".loop_lossless.rgba" : ".loop_dynamic.rgba")))
                return 1;
        }
        renderer->update(hygb::json::parse(R"({"clear_color": [0.25, 0.5, 1.0]})"));
        if (!dump(renderer->offline_render(cfg.camera), out + ".updated.rgba")) return 1;
    } catch (const std::exception &e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
