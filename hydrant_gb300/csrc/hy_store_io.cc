// hy_store_io.cc -- the on-disk brick store and raw-volume ingest.
//
// The reference reads a dataset directory through RendererFactory
// (include/hydrant/core/renderer.hpp:53-59: package_meta.json next to the
// archives) whose per-level archives and chebyshev thumbnails are written by
// build_dataset.sh:77-126 (varch's archiver, archive-thumbnailer,
// downsampler, meta-builder; H.264 brick streams).  Here a dataset directory
// holds uncompressed bricks instead:
//
//   package_meta.json   {"format": "hydrant-gb300-bricks", "version": 1,
//                        "dim": [x, y, z], "block_size": bs, "padding": p,
//                        "dtype": "u8" | "f32",
//                        "sample_levels": [
//                          {"level": 0, "grid": [gx, gy, gz], "nonempty": n,
//                           "bricks": "level0.bricks",
//                           "thumbnails": {"chebyshev": "level0.chebyshev.i32",
//                                          "mean": "level0.mean.f32"}},
//                          {"level": L, "grid": [...], "bricks": "levelL.bricks"}]}
//   level0.bricks       the padded bricks (P^3 voxels, x fastest) of every
//                       brick whose chebyshev value is 0, by brick index
//   level0.chebyshev.i32, level0.mean.f32   one value per brick
//   levelL.bricks       (optional) every brick of the coarse level
//
// All binary files are little-endian.  Ingest bricks a raw volume file on the
// host in slabs of block_size (+ apron) z-slices, in two passes (emptiness and
// thumbnails, then the bricks straight into the pinned store).

#include <sys/stat.h>

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "../../include/hydrant_gb300_json.hpp"
#include "hy_internal.h"

namespace {

using hygb::json::Value;

const char *kFormat = "hydrant-gb300-bricks";

template <typename F>
void parallel_for(int n, F fn) {
    const int nt = std::max(1, std::min<int>(n, int(std::thread::hardware_concurrency())));
    std::atomic<int> next{0};
    std::vector<std::thread> ts;
    for (int t = 0; t < nt; ++t)
        ts.emplace_back([&]() {
            for (int i = next++; i < n; i = next++) fn(i);
        });
    for (auto &t : ts) t.join();
}

std::string join(const std::string &dir, const std::string &name) {
    if (dir.empty() || dir.back() == '/') return dir + name;
    return dir + "/" + name;
}

bool write_file(const std::string &path, const void *data, size_t bytes) {
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    const bool ok = bytes == 0 || std::fwrite(data, 1, bytes, f) == bytes;
    return std::fclose(f) == 0 && ok;
}

bool read_file(const std::string &path, void *data, size_t bytes) {
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    const bool ok = bytes == 0 || std::fread(data, 1, bytes, f) == bytes;
    // the file must hold exactly `bytes`
    const bool at_end = std::fgetc(f) == EOF;
    std::fclose(f);
    return ok && at_end;
}

Value ivec3(const int v[3]) { return Value(Value::array_t{Value(v[0]), Value(v[1]), Value(v[2])}); }

size_t elem_bytes(int dtype) { return dtype == HY_DTYPE_U8 ? 1 : 4; }

size_t brick_bytes(const hy_store *s) {
    return size_t(s->P) * s->P * s->P * elem_bytes(s->desc.dtype);
}

// ---- ingest -----------------------------------------------------------------

// Reads raw z-slices [z0, z1) (x fastest) into buf.
bool read_slices(FILE *f, const hy_volume_desc &d, int z0, int z1, std::vector<unsigned char> &buf) {
    const size_t slice = size_t(d.dim[0]) * d.dim[1] * elem_bytes(d.dtype);
    buf.resize(slice * size_t(z1 - z0));
    if (fseeko(f, off_t(slice) * off_t(z0), SEEK_SET) != 0) return false;  // 64-bit offset
    return std::fread(buf.data(), 1, buf.size(), f) == buf.size();
}

// One padded brick of the slab starting at raw slice zs: apron clamped at
// the volume border.  Returns whether any voxel is non-zero; core_sum gets
// the sum of the core voxels (clamped ones included, as the device upload
// sums them).
template <typename T>
bool brick_from_slab(const hy_volume_desc &d, const std::vector<unsigned char> &slab, int zs,
                     int bx, int by, int bz, T *dst, double *core_sum) {
    const int bs = d.block_size, pad = d.padding, P = bs + 2 * pad;
    const T *raw = reinterpret_cast<const T *>(slab.data());
    bool any = false;
    double sum = 0.0;
    for (int k = 0; k < P; ++k) {
        const int Z = std::min(std::max(bz * bs + k - pad, 0), d.dim[2] - 1) - zs;
        for (int j = 0; j < P; ++j) {
            const int Y = std::min(std::max(by * bs + j - pad, 0), d.dim[1] - 1);
            const T *row = raw + (size_t(Z) * d.dim[1] + Y) * d.dim[0];
            const bool core_jk = k >= pad && k < pad + bs && j >= pad && j < pad + bs;
            for (int i = 0; i < P; ++i) {
                const int X = std::min(std::max(bx * bs + i - pad, 0), d.dim[0] - 1);
                const T v = row[X];
                if (dst) dst[(size_t(k) * P + j) * P + i] = v;
                any |= v != T(0);
                if (core_jk && i >= pad && i < pad + bs) sum += double(v);
            }
        }
    }
    if (core_sum) *core_sum = sum;
    return any;
}

template <typename T>
int ingest(hy_ctx *ctx, FILE *f, hy_store *s) {
    const hy_volume_desc &d = s->desc;
    const int bs = d.block_size, pad = d.padding;
    const int *g = s->grid;
    const int row_bricks = g[0] * g[1];
    std::vector<unsigned char> slab;
    std::vector<unsigned char> ne(s->nbricks, 0);
    std::vector<double> sums(s->nbricks, 0.0);
    auto slab_range = [&](int bz, int &z0, int &z1) {
        z0 = std::max(bz * bs - pad, 0);
        z1 = std::min(bz * bs + bs + pad, d.dim[2]);
    };
    // pass 1: emptiness and core sums
    for (int bz = 0; bz < g[2]; ++bz) {
        int z0, z1;
        slab_range(bz, z0, z1);
        if (!read_slices(f, d, z0, z1, slab)) return hy_fail(ctx, HY_ERR_INVALID, "ingest: read failed");
        parallel_for(row_bricks, [&](int r) {
            const int b = bz * row_bricks + r;
            ne[b] = brick_from_slab<T>(d, slab, z0, r % g[0], r / g[0], bz, nullptr, &sums[b]) ? 1 : 0;
        });
    }
    hy_chebyshev_transform(ne, s->grid, s->cheb);
    const double ncore = double(bs) * bs * bs;
    s->mean.resize(s->nbricks);
    s->offset.assign(s->nbricks, -1);
    int nonempty = 0;
    for (int b = 0; b < s->nbricks; ++b) {
        s->mean[b] = sizeof(T) == 1 ? float(sums[b] / 255.0 / ncore) : float(sums[b] / ncore);
        if (ne[b]) s->offset[b] = (long long)(nonempty++) * (long long)s->slot_stride;
    }
    int rc = hy_store_alloc(s, nonempty);
    if (rc) return rc;
    // pass 2: the non-empty bricks into the pinned store
    for (int bz = 0; bz < g[2]; ++bz) {
        bool any = false;
        for (int r = 0; r < row_bricks; ++r) any |= ne[bz * row_bricks + r] != 0;
        if (!any) continue;
        int z0, z1;
        slab_range(bz, z0, z1);
        if (!read_slices(f, d, z0, z1, slab)) return hy_fail(ctx, HY_ERR_INVALID, "ingest: read failed");
        parallel_for(row_bricks, [&](int r) {
            const int b = bz * row_bricks + r;
            if (!ne[b]) return;
            T *dst = reinterpret_cast<T *>(s->host + s->offset[b]);
            brick_from_slab<T>(d, slab, z0, r % g[0], r / g[0], bz, dst, nullptr);
        });
    }
    return HY_OK;
}

int parse_dtype(const std::string &name) {
    if (name == "u8") return HY_DTYPE_U8;
    if (name == "f32") return HY_DTYPE_F32;
    return -1;
}

}  // namespace

extern "C" int hy_store_ingest_raw(hy_ctx *ctx, const char *path, const hy_volume_desc *desc,
                                   hy_store **out) {
    if (!ctx || !path || !desc || !out) return HY_ERR_INVALID;
    *out = nullptr;
    hy_volume tmp;
    int rc = hy_volume_init(ctx, desc, &tmp);  // validates the descriptor
    if (rc) return rc;
    struct stat st;
    if (stat(path, &st) != 0) return hy_fail(ctx, HY_ERR_INVALID, std::string("ingest: cannot stat ") + path);
    const unsigned long long want = (unsigned long long)desc->dim[0] * desc->dim[1] * desc->dim[2] *
                                    elem_bytes(desc->dtype);
    if ((unsigned long long)st.st_size != want)
        return hy_fail(ctx, HY_ERR_INVALID,
                       "ingest: file size " + std::to_string((long long)st.st_size) +
                           " != dim product * element size " + std::to_string(want));
    FILE *f = std::fopen(path, "rb");
    if (!f) return hy_fail(ctx, HY_ERR_INVALID, std::string("ingest: cannot open ") + path);
    hy_store *s = new hy_store();
    s->ctx = ctx;
    hy_store_geometry(s, *desc);
    rc = desc->dtype == HY_DTYPE_U8 ? ingest<unsigned char>(ctx, f, s) : ingest<float>(ctx, f, s);
    std::fclose(f);
    if (rc) {
        hy_store_destroy(s);
        return rc;
    }
    *out = s;
    return HY_OK;
}

extern "C" int hy_store_save(const hy_store *s, const char *dir) {
    if (!s || !dir) return HY_ERR_INVALID;
    hy_ctx *ctx = s->ctx;
    const std::string root(dir);
    if (mkdir(dir, 0755) != 0 && errno != EEXIST)
        return hy_fail(ctx, HY_ERR_INVALID, "store save: cannot create " + root);
    const size_t bb = brick_bytes(s);
    // level 0: non-empty bricks by index, without the slot padding
    {
        const std::string path = join(root, "level0.bricks");
        FILE *f = std::fopen(path.c_str(), "wb");
        if (!f) return hy_fail(ctx, HY_ERR_INVALID, "store save: cannot write " + path);
        bool ok = true;
        for (int b = 0; b < s->nbricks && ok; ++b)
            if (s->offset[b] >= 0) ok = std::fwrite(s->host + s->offset[b], 1, bb, f) == bb;
        ok = (std::fclose(f) == 0) && ok;
        if (!ok) return hy_fail(ctx, HY_ERR_INVALID, "store save: short write " + path);
    }
    if (!write_file(join(root, "level0.chebyshev.i32"), s->cheb.data(), s->cheb.size() * 4) ||
        !write_file(join(root, "level0.mean.f32"), s->mean.data(), s->mean.size() * 4))
        return hy_fail(ctx, HY_ERR_INVALID, "store save: cannot write thumbnails");
    Value lvl0;
    lvl0.set("level", 0).set("grid", ivec3(s->grid)).set("nonempty", s->nonempty)
        .set("bricks", "level0.bricks");
    Value thumbs;
    thumbs.set("chebyshev", "level0.chebyshev.i32").set("mean", "level0.mean.f32");
    lvl0.set("thumbnails", thumbs);
    Value levels;
    levels.push(lvl0);
    if (s->coarse_level > 0) {
        const std::string name = "level" + std::to_string(s->coarse_level) + ".bricks";
        std::vector<unsigned char> packed(size_t(s->ncoarse) * bb);
        for (int c = 0; c < s->ncoarse; ++c)
            std::memcpy(packed.data() + size_t(c) * bb, s->coarse.data() + size_t(c) * s->slot_stride, bb);
        if (!write_file(join(root, name), packed.data(), packed.size()))
            return hy_fail(ctx, HY_ERR_INVALID, "store save: cannot write " + name);
        Value lc;
        lc.set("level", s->coarse_level).set("grid", ivec3(s->coarse_grid)).set("bricks", name);
        levels.push(lc);
    }
    Value meta;
    meta.set("format", kFormat).set("version", 1).set("dim", ivec3(s->desc.dim))
        .set("block_size", s->desc.block_size).set("padding", s->desc.padding)
        .set("dtype", s->desc.dtype == HY_DTYPE_U8 ? "u8" : "f32").set("sample_levels", levels);
    const std::string text = meta.dump(2) + "\n";
    if (!write_file(join(root, "package_meta.json"), text.data(), text.size()))
        return hy_fail(ctx, HY_ERR_INVALID, "store save: cannot write package_meta.json");
    return HY_OK;
}

extern "C" int hy_store_open(hy_ctx *ctx, const char *dir, hy_store **out) {
    if (!ctx || !dir || !out) return HY_ERR_INVALID;
    *out = nullptr;
    const std::string root(dir);
    Value meta;
    try {
        std::ifstream is(join(root, "package_meta.json"));
        if (!is) return hy_fail(ctx, HY_ERR_INVALID, "store open: no package_meta.json in " + root);
        std::stringstream ss;
        ss << is.rdbuf();
        meta = hygb::json::parse(ss.str());
        if (meta.string_or("format", "") != kFormat || meta["version"].as_int() != 1)
            return hy_fail(ctx, HY_ERR_INVALID, "store open: not a hydrant-gb300-bricks v1 dataset");
    } catch (const std::exception &e) {
        return hy_fail(ctx, HY_ERR_INVALID, std::string("store open: ") + e.what());
    }
    hy_store *s = new hy_store();
    s->ctx = ctx;
    auto fail = [&](const std::string &msg) {
        hy_store_destroy(s);
        return hy_fail(ctx, HY_ERR_INVALID, "store open: " + msg);
    };
    const Value *coarse = nullptr;
    try {
        hy_volume_desc d{};
        for (int i = 0; i < 3; ++i) d.dim[i] = int(meta["dim"][i].as_int());
        d.block_size = int(meta["block_size"].as_int());
        d.padding = int(meta["padding"].as_int());
        d.dtype = parse_dtype(meta["dtype"].as_string());
        if (d.dtype < 0) return fail("unknown dtype");
        hy_volume tmp;
        if (hy_volume_init(ctx, &d, &tmp)) return fail(hy_last_error(ctx));
        hy_store_geometry(s, d);
        const Value &levels = meta["sample_levels"];
        const Value *l0 = nullptr;
        for (size_t i = 0; i < levels.size(); ++i) {
            const long long lv = levels[i]["level"].as_int();
            if (lv == 0) l0 = &levels[i];
            else if (!coarse || lv > (*coarse)["level"].as_int()) coarse = &levels[i];
        }
        if (!l0) return fail("no level 0");
        for (int i = 0; i < 3; ++i)
            if ((*l0)["grid"][i].as_int() != s->grid[i]) return fail("level 0 grid does not match dim");
        s->cheb.resize(s->nbricks);
        s->mean.resize(s->nbricks);
        const Value &th = (*l0)["thumbnails"];
        if (!read_file(join(root, th["chebyshev"].as_string()), s->cheb.data(), s->cheb.size() * 4) ||
            !read_file(join(root, th["mean"].as_string()), s->mean.data(), s->mean.size() * 4))
            return fail("thumbnail files missing or of the wrong size");
        s->offset.assign(s->nbricks, -1);
        int nonempty = 0;
        for (int b = 0; b < s->nbricks; ++b)
            if (s->cheb[b] == 0) s->offset[b] = (long long)(nonempty++) * (long long)s->slot_stride;
        if ((*l0)["nonempty"].as_int() != nonempty) return fail("nonempty count does not match thumbnails");
        int rc = hy_store_alloc(s, nonempty);
        if (rc) {
            hy_store_destroy(s);
            return rc;
        }
        const size_t bb = brick_bytes(s);
        const std::string path = join(root, (*l0)["bricks"].as_string());
        FILE *f = std::fopen(path.c_str(), "rb");
        if (!f) return fail("cannot open " + path);
        bool ok = true;
        for (int b = 0; b < s->nbricks && ok; ++b)
            if (s->offset[b] >= 0) ok = std::fread(s->host + s->offset[b], 1, bb, f) == bb;
        ok = ok && std::fgetc(f) == EOF;
        std::fclose(f);
        if (!ok) return fail(path + " is not " + std::to_string(nonempty) + " bricks");
        if (coarse) {
            const int level = int((*coarse)["level"].as_int());
            if (level < 1 || level > 12 || d.block_size % (1 << level) != 0)
                return fail("bad coarse level");
            s->coarse_level = level;
            s->ncoarse = 1;
            for (int i = 0; i < 3; ++i) {
                const int cd = (d.dim[i] + (1 << level) - 1) >> level;
                s->coarse_grid[i] = (cd + d.block_size - 1) / d.block_size;
                if ((*coarse)["grid"][i].as_int() != s->coarse_grid[i]) return fail("coarse grid does not match dim");
                s->ncoarse *= s->coarse_grid[i];
            }
            std::vector<unsigned char> packed(size_t(s->ncoarse) * bb);
            if (!read_file(join(root, (*coarse)["bricks"].as_string()), packed.data(), packed.size()))
                return fail("coarse bricks missing or of the wrong size");
            s->coarse.assign(size_t(s->ncoarse) * s->slot_stride, 0);
            for (int c = 0; c < s->ncoarse; ++c)
                std::memcpy(s->coarse.data() + size_t(c) * s->slot_stride, packed.data() + size_t(c) * bb, bb);
        }
    } catch (const std::exception &e) {
        return fail(e.what());
    }
    *out = s;
    return HY_OK;
}
