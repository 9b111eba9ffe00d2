// hy_synth.cc -- seeded synthetic volumes (see include/hydrant_gb300_synth.h).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <thread>
#include <vector>

#include "../../include/hydrant_gb300_synth.h"

namespace {

uint64_t splitmix64(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
// uniform in [0, 1) with 53 random bits
double uniform(uint64_t &s) { return double(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }
double uniform(uint64_t &s, double lo, double hi) { return lo + (hi - lo) * uniform(s); }

// stateless hash of (seed, index) -> uniform [0,1)
double hash_uniform(uint64_t seed, uint64_t idx, uint64_t stream) {
    uint64_t s = seed ^ (idx * 0xD1B54A32D192ED03ull) ^ (stream * 0x8CB92BA72F3D8DD7ull);
    splitmix64(s);
    return uniform(s);
}

template <typename F>
void parallel_for(int n, int nthreads, F &&fn) {
    if (nthreads <= 0) nthreads = int(std::thread::hardware_concurrency());
    nthreads = std::max(1, std::min(nthreads, n));
    std::vector<std::thread> ts;
    for (int t = 0; t < nthreads; ++t)
        ts.emplace_back([&, t] {
            for (int i = t; i < n; i += nthreads) fn(i);
        });
    for (auto &t : ts) t.join();
}

struct Blob {
    double c[3], sigma, peak;
};

std::vector<Blob> draw_blobs(uint64_t seed, int n, double wlo, double whi) {
    uint64_t s = seed;
    std::vector<Blob> b(n);
    for (auto &x : b) {
        x.c[0] = uniform(s, 0.2, 0.8);
        x.c[1] = uniform(s, 0.2, 0.8);
        x.c[2] = uniform(s, 0.2, 0.8);
        x.sigma = uniform(s, 0.03, 0.12);
        x.peak = uniform(s, wlo, whi);
    }
    return b;
}

// Separable Gaussian: exp(-|x-c|^2/(2s^2)) = ex(i) * ey(j) * ez(k)
template <typename T, typename Q>
void blobs_impl(uint64_t seed, const int32_t dim[3], int nblobs, T *out, int nthreads, double wlo,
                double whi, Q &&quantise) {
    auto blobs = draw_blobs(seed, nblobs, wlo, whi);
    std::vector<std::vector<double>> e[3];
    for (int a = 0; a < 3; ++a) {
        e[a].resize(nblobs);
        for (int b = 0; b < nblobs; ++b) {
            e[a][b].resize(dim[a]);
            double inv = 1.0 / (2.0 * blobs[b].sigma * blobs[b].sigma);
            for (int i = 0; i < dim[a]; ++i) {
                double x = (i + 0.5) / dim[a] - blobs[b].c[a];
                e[a][b][i] = std::exp(-x * x * inv);
            }
        }
    }
    const size_t nx = dim[0], ny = dim[1];
    parallel_for(dim[2], nthreads, [&](int k) {
        std::vector<double> wz(nblobs), wyz(nblobs);
        for (int b = 0; b < nblobs; ++b) wz[b] = blobs[b].peak * e[2][b][k];
        for (size_t j = 0; j < ny; ++j) {
            for (int b = 0; b < nblobs; ++b) wyz[b] = wz[b] * e[1][b][j];
            T *row = out + (size_t(k) * ny + j) * nx;
            for (size_t i = 0; i < nx; ++i) {
                double v = 0.0;
                for (int b = 0; b < nblobs; ++b) v += wyz[b] * e[0][b][i];
                row[i] = quantise(v);
            }
        }
    });
}

}  // namespace

extern "C" int hy_synth_blobs_u8(uint64_t seed, const int32_t dim[3], int32_t nblobs,
                                 uint8_t *out, int32_t nthreads) {
    if (!dim || !out || nblobs < 0 || dim[0] <= 0 || dim[1] <= 0 || dim[2] <= 0) return -1;
    blobs_impl(seed, dim, nblobs, out, nthreads, 40.0, 255.0, [](double v) {
        double r = std::floor(v + 0.5);
        return uint8_t(std::min(255.0, std::max(0.0, r)));
    });
    return 0;
}

extern "C" int hy_synth_blobs_f32(uint64_t seed, const int32_t dim[3], int32_t nblobs, float *out,
                                  int32_t nthreads) {
    if (!dim || !out || nblobs < 0 || dim[0] <= 0 || dim[1] <= 0 || dim[2] <= 0) return -1;
    blobs_impl(seed, dim, nblobs, out, nthreads, 0.15, 0.6,
               [](double v) { return float(std::min(1.0, v)); });
    return 0;
}

extern "C" int hy_synth_tubes_u8(uint64_t seed, const int32_t dim[3], int32_t ntubes,
                                 uint8_t *out, int32_t nthreads) {
    if (!dim || !out || ntubes < 0 || dim[0] <= 0 || dim[1] <= 0 || dim[2] <= 0) return -1;
    const int nx = dim[0], ny = dim[1], nz = dim[2];
    // background ~ U{0..30}
    parallel_for(nz, nthreads, [&](int k) {
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                uint64_t idx = (uint64_t(k) * ny + j) * nx + i;
                out[idx] = uint8_t(std::min(30.0, std::floor(hash_uniform(seed, idx, 1) * 31.0)));
            }
    });
    struct Tube {
        double p[4][3];
        double r;
    };
    uint64_t s = seed ^ 0x5851F42D4C957F2Dull;
    std::vector<Tube> tubes(ntubes);
    for (auto &t : tubes) {
        for (int c = 0; c < 4; ++c)
            for (int a = 0; a < 3; ++a) t.p[c][a] = uniform(s, 0.05, 0.95) * dim[a];
        t.r = uniform(s, 2.0, 10.0);
    }
    // inside value: clamp(round(200 + 20 z)), z ~ N(0,1) by Box-Muller on the voxel hash
    auto inside = [&](uint64_t idx) {
        double u1 = hash_uniform(seed, idx, 2), u2 = hash_uniform(seed, idx, 3);
        double z = std::sqrt(-2.0 * std::log(1.0 - u1)) * std::cos(6.283185307179586 * u2);
        double v = std::floor(200.0 + 20.0 * z + 0.5);
        return uint8_t(std::min(255.0, std::max(0.0, v)));
    };
    // Stamp spheres of radius r along each curve at spacing <= r/2; each
    // thread owns a range of z-slices so no voxel is written twice at once.
    int nthr = nthreads > 0 ? nthreads : int(std::thread::hardware_concurrency());
    nthr = std::max(1, std::min(nthr, nz));
    parallel_for(nthr, nthr, [&](int t) {
        const int z0 = int((long long)nz * t / nthr), z1 = int((long long)nz * (t + 1) / nthr);
        for (const Tube &tb : tubes) {
            double len = 0.0;
            for (int c = 0; c < 3; ++c) {
                double d2 = 0.0;
                for (int a = 0; a < 3; ++a) d2 += (tb.p[c + 1][a] - tb.p[c][a]) * (tb.p[c + 1][a] - tb.p[c][a]);
                len += std::sqrt(d2);
            }
            const int n = std::max(2, int(std::ceil(len / (tb.r * 0.5))) + 1);
            const double r2 = tb.r * tb.r;
            for (int q = 0; q < n; ++q) {
                const double u = double(q) / (n - 1), w = 1.0 - u;
                const double b0 = w * w * w, b1 = 3 * w * w * u, b2 = 3 * w * u * u, b3 = u * u * u;
                double c[3];
                for (int a = 0; a < 3; ++a)
                    c[a] = b0 * tb.p[0][a] + b1 * tb.p[1][a] + b2 * tb.p[2][a] + b3 * tb.p[3][a];
                int lo[3], hi[3];
                for (int a = 0; a < 3; ++a) {
                    lo[a] = std::max(0, int(std::floor(c[a] - tb.r - 0.5)));
                    hi[a] = std::min(dim[a] - 1, int(std::ceil(c[a] + tb.r + 0.5)));
                }
                lo[2] = std::max(lo[2], z0);
                hi[2] = std::min(hi[2], z1 - 1);
                for (int k = lo[2]; k <= hi[2]; ++k)
                    for (int j = lo[1]; j <= hi[1]; ++j)
                        for (int i = lo[0]; i <= hi[0]; ++i) {
                            double dx = i + 0.5 - c[0], dy = j + 0.5 - c[1], dz = k + 0.5 - c[2];
                            if (dx * dx + dy * dy + dz * dz <= r2) {
                                uint64_t idx = (uint64_t(k) * ny + j) * nx + i;
                                out[idx] = inside(idx);
                            }
                        }
            }
        }
    });
    return 0;
}
