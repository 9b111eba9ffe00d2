// Checks of the JSON reader/writer (include/hydrant_gb300_json.hpp) and of
// the configuration parsing in include/hydrant_gb300_renderer.hpp that needs
// no device.  Prints "ok" and exits 0, or prints the failed check and exits 1.
#include <cstdio>
#include <string>

#include "hydrant_gb300_renderer.hpp"

using hygb::json::Value;

static int failures = 0;
#define CHECK(cond)                                                  \
    do {                                                             \
        if (!(cond)) {                                               \
            std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #cond); \
            ++failures;                                              \
        }                                                            \
    } while (0)

template <typename F>
static bool throws(F f) {
    try {
        f();
    } catch (const std::exception &) {
        return true;
    }
    return false;
}

int main() {
    // the reference README's configuration
    const char *readme = R"({
        "camera": { "orbit": { "arm": [ 25, 65, 2.2 ] } },
        "render": {
            "resolution": [ 512, 512 ],
            "renderer": "Volume",
            "params": {
                "mode": "Volume",
                "density": 1e-2,
                "transfer_fn": { "values": [ [ 0, 0, 0, 0 ], [ 1, 0, 0, 1 ], [ 1, 0.5, 0, 1 ] ] }
            }
        }
    })";
    Value v = hygb::json::parse(readme);
    CHECK(v["render"]["resolution"][1].as_int() == 512);
    CHECK(v["render"]["params"]["density"].as_number() == 1e-2);
    CHECK(v["render"]["params"]["transfer_fn"]["values"][2][1].as_number() == 0.5);
    CHECK(v["camera"]["orbit"]["arm"][2].as_number() == 2.2);
    CHECK(v["missing"].is_null() && v["render"]["missing"]["deeper"].is_null());

    hygb::Config c = hygb::Config::from_json(v);
    CHECK(!c.camera.ptu && c.camera.arm[0] == 25.f && c.camera.fovy == 60.f);
    CHECK(c.render.renderer == "Volume" && c.render.resolution[0] == 512);
    CHECK(c.render.params["mode"].as_string() == "Volume");

    // config.schema.hpp's wrapped form and a ptu camera
    Value w = hygb::json::parse(R"({"data_path": "/data/x", "params": {
        "camera": {"ptu": {"position": [0, 0, 3]}, "perspective": {"fovy": 45}},
        "render": {"renderer": "Isosurface"}}})");
    hygb::Config c2 = hygb::Config::from_json(w);
    CHECK(c2.data_path == "/data/x" && c2.camera.ptu && c2.camera.position[2] == 3.f);
    CHECK(c2.camera.up[1] == 1.f && c2.camera.fovy == 45.f);
    CHECK(c2.render.resolution[0] == 512 && c2.render.renderer == "Isosurface");

    // strings, escapes, numbers, round trip
    Value s = hygb::json::parse(R"(["a\"b\\c\/\n", "\u00e9\ud83d\ude00", -0.5e-3, 1E2, true, false, null, {}, []])");
    CHECK(s[0].as_string() == "a\"b\\c/\n");
    CHECK(s[1].as_string() == "\xc3\xa9\xf0\x9f\x98\x80");
    CHECK(s[2].as_number() == -0.5e-3 && s[3].as_number() == 100.0);
    CHECK(s[4].as_bool() && !s[5].as_bool() && s[6].is_null());
    CHECK(s[7].is_object() && s[7].size() == 0 && s[8].is_array() && s[8].size() == 0);
    Value back = hygb::json::parse(s.dump());
    CHECK(back.dump() == s.dump());
    CHECK(hygb::json::parse(s.dump(2)).dump() == s.dump());

    // malformed documents are rejected with an offset
    const char *bad[] = {"", "{", "[1,]", "{\"a\" 1}", "01", "1.", "\"\\x\"", "tru", "[1] 2",
                         "\"a\nb\"", "{\"a\":1,}", "\"\\ud800\""};
    for (const char *b : bad) CHECK(throws([&] { hygb::json::parse(b); }));
    try {
        hygb::json::parse("[1, 2, x]");
    } catch (const hygb::json::ParseError &e) {
        CHECK(e.offset == 7);
    }

    // type errors and bad configs throw
    CHECK(throws([&] { v["render"]["renderer"].as_number(); }));
    CHECK(throws([&] { hygb::Config::from_json(hygb::json::parse(R"({"camera": {}, "render": {}})")); }));
    CHECK(throws([&] { hygb::CameraConfig::from_json(hygb::json::parse(R"({"orbit": {"arm": [1, 2]}})")); }));

    // built-in renderers are registered
    auto names = hygb::RendererFactory::list_candidates();
    CHECK(names.size() == 4 && names[0] == "Blocks" && names[1] == "Isosurface" &&
          names[2] == "Paging" && names[3] == "Volume");

    if (failures) return 1;
    std::printf("ok\n");
    return 0;
}
