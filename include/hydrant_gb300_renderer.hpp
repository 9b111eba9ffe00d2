// hydrant_gb300_renderer.hpp -- C++17 renderer layer over the C ABI.
//
// Mirrors the reference's renderer-level plugin interface so that a host
// application written against it switches by changing includes and names:
//   * IRenderer {init(dataset, RendererConfig), update(json params),
//     offline_render(Camera) -> image, realtime_render(IRenderLoop &,
//     RealtimeRenderOptions)} with IRenderLoop's callbacks
//     (include/hydrant/core/renderer.hpp:17-49, render_loop.hpp:12-34);
//   * RendererRegistry + HYGB_REGISTER_RENDERER(T, "name") and
//     RendererFactory(dataset_path).create(cfg) / list_candidates()
//     (renderer.hpp:51-89);
//   * the JSON configuration objects: Config {data_path, params {camera,
//     render}} (config.schema.hpp), CameraConfig {ptu | orbit, perspective}
//     (scene.schema.hpp), RendererConfig {resolution, renderer, params}
//     (renderer.schema.hpp), BasicRendererParams {device, comm_rank,
//     sample_rate, max_steps, clear_color} (basic_renderer.schema.hpp), and
//     the Volume / Blocks / Isosurface params (ui/*.schema.hpp).
// The built-in renderers "Volume", "Blocks", "Isosurface" and "Paging"
// follow volume.cc, blocks.cc, isosurface.cc and paging.cc: offline_render
// pages the dataset through the lossless pager (Blocks reads only the
// thumbnails: one emit pass; Paging returns an unrendered film, as there),
// realtime_render renders one frame through the realtime pager with the
// mem_limit_mb cache (and the dataset's coarse level as fallback).
//
// Differences from the reference, by design:
//   * images are RGBA8 (A = saturated opacity; RGB as the reference writes);
//   * "device": "Cpu" is rejected (the CPU path is the test oracle, not a
//     product path); "comm_rank" selects the CUDA device as in
//     basic_renderer.hpp:43-52;
//   * transfer_fn.values may be the flat float list of the schema or the
//     nested [[r,g,b,a], ...] form the reference's README shows;
//   * Volume takes "density" (opacity scale, 1 = the reference);
//   * errors are thrown as hygb::Error (the reference aborts in LOG(FATAL)).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <functional>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "hydrant_gb300.h"
#include "hydrant_gb300_json.hpp"

namespace hygb {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc, hy_ctx *ctx, const char *what) {
    if (rc == HY_OK) return;
    std::string msg = what;
    if (ctx) {
        const char *e = hy_last_error(ctx);
        if (e && *e) msg += std::string(": ") + e;
    }
    throw Error(rc, msg);
}

namespace detail {

inline void vec3(const json::Value &v, float out[3]) {
    if (v.is_null()) return;
    if (!v.is_array() || v.size() != 3) throw Error(HY_ERR_INVALID, "config: expected [x, y, z]");
    for (int i = 0; i < 3; ++i) out[i] = float(v[i].as_number());
}

inline std::string read_text(const std::string &path) {
    std::ifstream is(path);
    if (!is) throw Error(HY_ERR_INVALID, "cannot read " + path);
    std::stringstream ss;
    ss << is.rdbuf();
    return ss.str();
}

inline std::string join(const std::string &dir, const std::string &name) {
    if (dir.empty() || dir.back() == '/') return dir + name;
    return dir + "/" + name;
}

// VM_ENUM names -> index, as the reference's JSON binding spells them
inline int enum_index(const json::Value &v, std::initializer_list<const char *> names, int dflt,
                      const char *what) {
    if (v.is_null()) return dflt;
    if (v.is_number()) return int(v.as_int());
    int i = 0;
    for (const char *n : names) {
        if (v.as_string() == n) return i;
        ++i;
    }
    throw Error(HY_ERR_INVALID, std::string("config: unknown ") + what + " '" + v.as_string() + "'");
}

}  // namespace detail

// ---- configuration -----------------------------------------------------------

// CameraConfig (scene.schema.hpp): exactly one of ptu / orbit, fovy 60.
struct CameraConfig {
    bool ptu = false;
    float position[3] = {0, 0, 0}, target[3] = {0, 0, 0}, up[3] = {0, 1, 0};
    float center[3] = {0, 0, 0}, arm[3] = {0, 0, 0};
    float fovy = 60.f;

    static CameraConfig from_json(const json::Value &v) {
        CameraConfig c;
        if (v["ptu"].is_object()) {
            c.ptu = true;
            detail::vec3(v["ptu"]["position"], c.position);
            detail::vec3(v["ptu"]["target"], c.target);
            detail::vec3(v["ptu"]["up"], c.up);
        } else if (v["orbit"].is_object()) {
            detail::vec3(v["orbit"]["center"], c.center);
            detail::vec3(v["orbit"]["arm"], c.arm);
        } else {
            throw Error(HY_ERR_INVALID, "config: camera needs 'ptu' or 'orbit'");
        }
        if (v["perspective"].is_object()) c.fovy = float(v["perspective"].number_or("fovy", 60.0));
        return c;
    }

    hy_camera camera() const {
        hy_camera out{};
        const int rc = ptu ? hy_camera_ptu(position, target, up, fovy, &out)
                           : hy_camera_orbit(arm, center, fovy, &out);
        check(rc, nullptr, "camera");
        return out;
    }
};

// RendererConfig (renderer.schema.hpp)
struct RendererConfig {
    int resolution[2] = {512, 512};
    std::string renderer;
    json::Value params;

    static RendererConfig from_json(const json::Value &v) {
        RendererConfig r;
        if (!v["resolution"].is_null()) {
            r.resolution[0] = int(v["resolution"][0].as_int());
            r.resolution[1] = int(v["resolution"][1].as_int());
        }
        r.renderer = v.string_or("renderer", "");
        r.params = v["params"];
        return r;
    }
};

// Config (config.schema.hpp): {"data_path": ..., "params": {"camera", "render"}};
// the README's form without the wrapper is accepted too.
struct Config {
    std::string data_path;
    CameraConfig camera;
    RendererConfig render;

    static Config from_json(const json::Value &v) {
        const json::Value &p = v["params"].is_object() ? v["params"] : v;
        Config c;
        c.data_path = v.string_or("data_path", "");
        c.camera = CameraConfig::from_json(p["camera"]);
        c.render = RendererConfig::from_json(p["render"]);
        return c;
    }
    static Config from_file(const std::string &path) {
        return from_json(json::parse(detail::read_text(path)));
    }
};

// ---- dataset (renderer.hpp:17-21) ------------------------------------------------

// A dataset directory (package_meta.json + bricks, hy_store_save) opened
// into a pinned brick store on one device context.
struct Dataset {
    std::string root;
    json::Value meta;
    hy_ctx *ctx = nullptr;
    hy_store *store = nullptr;
    int device = 0;

    Dataset(const std::string &path, int dev = 0) : root(path), device(dev) {
        meta = json::parse(detail::read_text(detail::join(path, "package_meta.json")));
        check(hy_ctx_create(dev, &ctx), nullptr, "context");
        const int rc = hy_store_open(ctx, path.c_str(), &store);
        if (rc != HY_OK) {
            const std::string msg = hy_last_error(ctx);
            hy_ctx_destroy(ctx);
            ctx = nullptr;
            throw Error(rc, "dataset " + path + ": " + msg);
        }
    }
    ~Dataset() {
        if (store) hy_store_destroy(store);
        if (ctx) hy_ctx_destroy(ctx);
    }
    Dataset(const Dataset &) = delete;
    Dataset &operator=(const Dataset &) = delete;

    hy_volume_info info() const {
        hy_volume_info i{};
        check(hy_store_get_info(store, &i), ctx, "store info");
        return i;
    }
};

// RGBA8 image, rows top to bottom.
struct Image {
    int width = 0, height = 0;
    std::vector<uint8_t> rgba;

    // binary PPM (RGB), the reference's dump format family
    bool write_ppm(const std::string &path) const {
        FILE *f = std::fopen(path.c_str(), "wb");
        if (!f) return false;
        std::fprintf(f, "P6\n%d %d\n255\n", width, height);
        bool ok = true;
        for (size_t i = 0; i < size_t(width) * height && ok; ++i) ok = std::fwrite(&rgba[4 * i], 1, 3, f) == 3;
        return std::fclose(f) == 0 && ok;
    }
};

// ---- renderer interface ----------------------------------------------------------

// The realtime session's callbacks (include/hydrant/core/render_loop.hpp:12-34):
// realtime_render(loop, opts) calls post_loop once, then per frame post_frame,
// one frame at `camera` (which the loop may change between frames), on_frame
// and after_frame until should_stop, then after_loop.
struct IRenderLoop {
    explicit IRenderLoop(CameraConfig const &cam) : camera(cam) {}
    virtual ~IRenderLoop() = default;
    IRenderLoop(IRenderLoop const &) = delete;
    IRenderLoop &operator=(IRenderLoop const &) = delete;

    virtual void post_loop() {}
    virtual bool should_stop() = 0;
    virtual void post_frame() {}
    virtual void on_frame(Image &frame) = 0;
    virtual void after_frame() {}
    virtual void after_loop() {}

    CameraConfig camera;
};

// renderer.hpp:17-27: Lossless frames page every visible brick through the
// lossless pager (offline_render), Dynamic frames come from the realtime
// pager (realtime_render(camera)).  There is one rank, so no communicator.
enum class RealtimeRenderQuality { Lossless, Dynamic };
struct RealtimeRenderOptions {
    RealtimeRenderQuality quality = RealtimeRenderQuality::Dynamic;
};

class IRenderer {
public:
    virtual ~IRenderer() = default;

    virtual bool init(std::shared_ptr<Dataset> const &ds, RendererConfig const &cfg) {
        dataset = ds;
        resolution[0] = cfg.resolution[0];
        resolution[1] = cfg.resolution[1];
        return true;
    }
    virtual void update(json::Value const &params) { (void)params; }
    virtual Image offline_render(CameraConfig const &camera) = 0;
    // one frame of the realtime path
    virtual Image realtime_render(CameraConfig const &camera) = 0;

    // the realtime session (basic_renderer.hpp:106-133): frames until the
    // loop says stop
    void realtime_render(IRenderLoop &loop, RealtimeRenderOptions const &opts = {}) {
        loop.post_loop();
        while (!loop.should_stop()) {
            loop.post_frame();
            Image frame = opts.quality == RealtimeRenderQuality::Lossless
                              ? offline_render(loop.camera)
                              : realtime_render(loop.camera);
            loop.on_frame(frame);
            loop.after_frame();
        }
        loop.after_loop();
    }

protected:
    std::shared_ptr<Dataset> dataset;
    int resolution[2] = {512, 512};
};

struct RendererRegistry {
    static RendererRegistry &instance() {
        static RendererRegistry r;
        return r;
    }
    std::map<std::string, std::function<IRenderer *()>> types;
};

#define HYGB_REGISTER_RENDERER(T, name)                                              \
    inline const bool hygb_registered_##T = [] {                                      \
        ::hygb::RendererRegistry::instance().types[name] = [] { return new T(); };   \
        return true;                                                                  \
    }()

// BasicRenderer (basic_renderer.hpp:57-131): device, comm_rank, sample_rate,
// max_steps, clear_color; owns the pagers for the dataset.
class BasicRenderer : public IRenderer {
public:
    ~BasicRenderer() override { release(); }

    bool init(std::shared_ptr<Dataset> const &ds, RendererConfig const &cfg) override {
        IRenderer::init(ds, cfg);
        const json::Value &p = cfg.params;
        if (detail::enum_index(p["device"], {"Cpu", "Cuda"}, 1, "device") != 1)
            throw Error(HY_ERR_UNSUPPORTED, "device Cpu: the CUDA path is the only product path");
        if (int(p.number_or("comm_rank", 0)) != ds->device)
            throw Error(HY_ERR_INVALID, "comm_rank must name the dataset's device");
        update(p);
        return true;
    }

    void update(json::Value const &p) override {
        sample_rate = float(p.number_or("sample_rate", sample_rate));
        max_steps = int(p.number_or("max_steps", max_steps));
        detail::vec3(p["clear_color"], clear_color);
    }

protected:
    float sample_rate = 1.f;
    int max_steps = 4000000;
    float clear_color[3] = {0, 0, 0};
    hy_pager *offline_pager = nullptr, *realtime_pager = nullptr;
    size_t offline_mb = 0, realtime_mb = 0;
    int realtime_sampler = HY_PAGER_LOADS;

    void release() {
        if (offline_pager) hy_pager_destroy(offline_pager);
        if (realtime_pager) hy_pager_destroy(realtime_pager);
        offline_pager = realtime_pager = nullptr;
    }

    hy_shader_params base_params(int shader) const {
        hy_shader_params p{};
        p.shader = shader;
        p.sample_rate = sample_rate;
        p.max_steps = max_steps;
        p.density = 1.f;
        p.isovalue = 0.5f;
        for (int i = 0; i < 3; ++i) {
            p.surface_color[i] = 1.f;
            p.clear_color[i] = clear_color[i];
        }
        return p;
    }

    int slots_for(size_t mem_limit_mb, int cap) const {
        const hy_volume_info i = dataset->info();
        long long n = (long long)(mem_limit_mb * 1024 * 1024 / size_t(i.slot_bytes));
        if (cap > 0 && n > cap) n = cap;
        return int(n < 1 ? 1 : n);
    }

    // LosslessBlockPagingServer batches: min(mem_limit / brick, 4096)
    // (lossless_block_paging.cc:6, 25-27)
    hy_pager *offline(size_t mem_limit_mb) {
        if (!offline_pager || offline_mb != mem_limit_mb) {
            if (offline_pager) hy_pager_destroy(offline_pager);
            offline_pager = nullptr;
            hy_pager_desc d{slots_for(mem_limit_mb, 4096), HY_PAGER_LOSSLESS, 0, HY_EVICT_LRU, HY_PAGER_LOADS};
            check(hy_pager_create(dataset->ctx, dataset->store, &d, &offline_pager), dataset->ctx,
                  "offline pager");
            offline_mb = mem_limit_mb;
        }
        return offline_pager;
    }

    // RtBlockPagingServer cache: mem_limit / brick slots (rt_block_paging.cc:230-233).
    // `gathers`: the cache in gather textures (the Volume shader's Default
    // mode samples it by texture gathers), where the dataset allows it;
    // otherwise, and for every other use, a device pool read by loads.
    hy_pager *realtime(size_t mem_limit_mb, bool gathers = false) {
        const int sampler = gathers ? HY_PAGER_GATHERS : HY_PAGER_LOADS;
        if (!realtime_pager || realtime_mb != mem_limit_mb || realtime_sampler != sampler) {
            if (realtime_pager) hy_pager_destroy(realtime_pager);
            realtime_pager = nullptr;
            hy_pager_desc d{slots_for(mem_limit_mb, 0), HY_PAGER_REALTIME, 0, HY_EVICT_LRU, sampler};
            int rc = hy_pager_create(dataset->ctx, dataset->store, &d, &realtime_pager);
            if (rc == HY_ERR_UNSUPPORTED && sampler == HY_PAGER_GATHERS) {
                d.sampler = HY_PAGER_LOADS;  // e.g. an f32 dataset: the pool cache
                rc = hy_pager_create(dataset->ctx, dataset->store, &d, &realtime_pager);
            }
            check(rc, dataset->ctx, "realtime pager");
            realtime_mb = mem_limit_mb;
            realtime_sampler = sampler;
        }
        return realtime_pager;
    }

    Image frame(hy_pager *pg, hy_shader_params p, CameraConfig const &camera) {
        Image img;
        img.width = resolution[0];
        img.height = resolution[1];
        img.rgba.resize(size_t(img.width) * img.height * 4);
        const hy_camera cam = camera.camera();
        if (p.shader == HY_SHADER_ISOSURFACE) {
            hy_volume *v = nullptr;
            check(hy_pager_volume(pg, &v), dataset->ctx, "pager volume");
            check(hy_iso_lighting(v, &cam, &p), dataset->ctx, "isosurface lighting");
        }
        check(hy_pager_render_host(pg, &p, &cam, img.width, img.height, img.rgba.data()),
              dataset->ctx, "render");
        return img;
    }
};

// VolumeRenderer (volume.cc:58-70; ui/volume.schema.hpp)
class VolumeRenderer : public BasicRenderer {
public:
    void update(json::Value const &p) override {
        BasicRenderer::update(p);
        mode = detail::enum_index(p["mode"], {"Default", "Partition", "Paging"}, mode, "Volume mode");
        mem_limit_mb = size_t(p.number_or("mem_limit_mb", double(mem_limit_mb)));
        density = float(p.number_or("density", density));
        rank = float(p.number_or("rank", rank));
        const json::Value &tf = p["transfer_fn"];
        if (tf.is_object() && tf["values"].size()) {
            std::vector<float> flat;
            for (const json::Value &e : tf["values"].as_array()) {
                if (e.is_array())
                    for (const json::Value &x : e.as_array()) flat.push_back(float(x.as_number()));
                else
                    flat.push_back(float(e.as_number()));
            }
            if (flat.size() % 4 != 0) throw Error(HY_ERR_INVALID, "transfer_fn: values are RGBA quadruples");
            knots = flat;
        }
    }
    Image offline_render(CameraConfig const &camera) override {
        return frame(offline(mem_limit_mb), params(), camera);
    }
    using IRenderer::realtime_render;  // keep the loop overload visible
    Image realtime_render(CameraConfig const &camera) override {
        return frame(realtime(mem_limit_mb, mode == HY_VOLUME_DEFAULT), params(), camera);
    }

private:
    int mode = HY_VOLUME_DEFAULT;
    size_t mem_limit_mb = 2048;
    float density = 1.f;
    float rank = 0.f;
    std::vector<float> knots = {0, 0, 0, 0, 1, 1, 1, 1};  // TransferFnConfig default

    hy_shader_params params() {
        check(hy_tf_set(dataset->ctx, knots.data(), int32_t(knots.size() / 4)), dataset->ctx,
              "transfer function");
        hy_shader_params p = base_params(HY_SHADER_VOLUME);
        p.mode = mode;
        p.density = density;
        p.rank = rank;
        return p;
    }
};

// BlocksRenderer (blocks.cc:30-72; ui/blocks.schema.hpp): thumbnails only,
// one emit pass over the dataset's geometry.
class BlocksRenderer : public BasicRenderer {
public:
    void update(json::Value const &p) override {
        BasicRenderer::update(p);
        mode = detail::enum_index(p["mode"], {"Volume", "Solid"}, mode, "Blocks mode");
        density = float(p.number_or("density", density));
    }
    Image offline_render(CameraConfig const &camera) override { return render(camera); }
    using IRenderer::realtime_render;  // keep the loop overload visible
    Image realtime_render(CameraConfig const &camera) override { return render(camera); }

private:
    int mode = HY_BLOCKS_VOLUME;
    float density = 1e-2f;

    Image render(CameraConfig const &camera) {
        hy_shader_params p = base_params(HY_SHADER_BLOCKS);
        p.mode = mode;
        p.density = density;
        hy_pager *pg = offline(64);
        hy_volume *v = nullptr;
        check(hy_pager_volume(pg, &v), dataset->ctx, "pager volume");
        const hy_camera cam = camera.camera();
        hy_view view{};
        check(hy_camera_view(v, &cam, &view), dataset->ctx, "view");
        Image img;
        img.width = resolution[0];
        img.height = resolution[1];
        img.rgba.resize(size_t(img.width) * img.height * 4);
        check(hy_render(dataset->ctx, v, &p, &view, img.width, img.height, img.rgba.data(), nullptr,
                        nullptr),
              dataset->ctx, "render");
        return img;
    }
};

// IsosurfaceRenderer (isosurface.cc:56-70, 108-113; ui/isosurface.schema.hpp)
class IsosurfaceRenderer : public BasicRenderer {
public:
    void update(json::Value const &p) override {
        BasicRenderer::update(p);
        mode = detail::enum_index(p["mode"], {"Color", "Normal", "Position"}, mode, "Isosurface mode");
        detail::vec3(p["surface_color"], surface_color);
        isovalue = float(p.number_or("isovalue", isovalue));
        mem_limit_mb = size_t(p.number_or("mem_limit_mb", double(mem_limit_mb)));
    }
    Image offline_render(CameraConfig const &camera) override {
        return frame(offline(mem_limit_mb), params(), camera);
    }
    using IRenderer::realtime_render;  // keep the loop overload visible
    Image realtime_render(CameraConfig const &camera) override {
        return frame(realtime(mem_limit_mb), params(), camera);
    }

private:
    int mode = HY_ISO_COLOR;
    float surface_color[3] = {1, 1, 1};
    float isovalue = 0.5f;
    size_t mem_limit_mb = 2048;

    hy_shader_params params() const {
        hy_shader_params p = base_params(HY_SHADER_ISOSURFACE);
        p.mode = mode;
        p.isovalue = isovalue;
        for (int i = 0; i < 3; ++i) p.surface_color[i] = surface_color[i];
        return p;
    }
};

// PagingRenderer (src/slave/renderers/paging/paging.cc; paging.schema.hpp):
// the paging debug view.  Its offline render is an unrendered (clear) film,
// as in the reference (paging.cc:60-65); a realtime frame shows the realtime
// cache: green bricks resident, red ones drawn from the coarse level.
class PagingRenderer : public BasicRenderer {
public:
    void update(json::Value const &p) override {
        BasicRenderer::update(p);
        mem_limit_mb = size_t(p.number_or("mem_limit_mb", double(mem_limit_mb)));
    }
    Image offline_render(CameraConfig const &camera) override {
        (void)camera;
        Image img;
        img.width = resolution[0];
        img.height = resolution[1];
        img.rgba.assign(size_t(img.width) * img.height * 4, 0);
        return img;
    }
    using IRenderer::realtime_render;  // keep the loop overload visible
    Image realtime_render(CameraConfig const &camera) override {
        return frame(realtime(mem_limit_mb), base_params(HY_SHADER_PAGING), camera);
    }

private:
    size_t mem_limit_mb = 2048;
};

HYGB_REGISTER_RENDERER(VolumeRenderer, "Volume");
HYGB_REGISTER_RENDERER(PagingRenderer, "Paging");
HYGB_REGISTER_RENDERER(BlocksRenderer, "Blocks");
HYGB_REGISTER_RENDERER(IsosurfaceRenderer, "Isosurface");

// RendererFactory (renderer.hpp:51-67)
class RendererFactory {
public:
    explicit RendererFactory(const std::string &dataset_path, int device = 0)
        : dataset(std::make_shared<Dataset>(dataset_path, device)) {}

    std::unique_ptr<IRenderer> create(RendererConfig const &cfg) {
        auto &types = RendererRegistry::instance().types;
        auto it = types.find(cfg.renderer);
        if (it == types.end()) throw Error(HY_ERR_INVALID, "unknown renderer '" + cfg.renderer + "'");
        std::unique_ptr<IRenderer> r(it->second());
        r->init(dataset, cfg);
        return r;
    }

    static std::vector<std::string> list_candidates() {
        std::vector<std::string> names;
        for (auto &kv : RendererRegistry::instance().types) names.push_back(kv.first);
        return names;
    }

    std::shared_ptr<Dataset> const &get_dataset() const { return dataset; }

private:
    std::shared_ptr<Dataset> dataset;
};

}  // namespace hygb
