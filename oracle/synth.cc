// synth.cc -- TEST INFRASTRUCTURE ONLY.
//
// The seeded synthetic volumes of the benchmark workloads, generated on the
// host for the CPU side of the measurement (the reference arm and the CPU
// baseline), so that side loads nothing but the oracle.  Same definitions
// as the product's generators (include/hydrant_gb300_synth.h): splitmix64
// draws, double arithmetic in the same order, so the bytes are identical;
// tests/test_oracle_synth.py holds the two to that.
//
//  blobs: v = sum_b peak_b * g_b(z) * g_b(y) * g_b(x), g = exp(-d^2 / (2 s^2))
//         at voxel centres (i + 0.5) / n; u8 rounds half up and clamps to
//         [0, 255], f32 is min(1, v).
//  tubes: background U{0..30} and cubic Bezier tubes stamped as spheres,
//         inside value round(N(200, 20)) from per-voxel hashes.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <thread>
#include <vector>

namespace {

struct Rng {
    uint64_t s;
    uint64_t bits() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double unit() { return double(bits() >> 11) * (1.0 / 9007199254740992.0); }
    double range(double lo, double hi) { return lo + (hi - lo) * unit(); }
};

double voxel_hash(uint64_t seed, uint64_t idx, uint64_t stream) {
    Rng r{seed ^ (idx * 0xD1B54A32D192ED03ull) ^ (stream * 0x8CB92BA72F3D8DD7ull)};
    r.bits();
    return r.unit();
}

template <typename Fn>
void over_threads(int n, int nthreads, Fn fn) {
    if (nthreads <= 0) nthreads = int(std::thread::hardware_concurrency());
    nthreads = std::max(1, std::min(nthreads, n));
    std::vector<std::thread> pool;
    for (int t = 0; t < nthreads; ++t)
        pool.emplace_back([&, t] {
            for (int i = t; i < n; i += nthreads) fn(i);
        });
    for (auto &th : pool) th.join();
}

template <typename T, typename Q>
void blobs(uint64_t seed, const int32_t dim[3], int nb, T *out, int nthreads, double plo,
           double phi, Q quant) {
    Rng r{seed};
    std::vector<double> cen(3 * size_t(nb)), sig(nb), peak(nb);
    for (int b = 0; b < nb; ++b) {
        for (int a = 0; a < 3; ++a) cen[3 * b + a] = r.range(0.2, 0.8);
        sig[b] = r.range(0.03, 0.12);
        peak[b] = r.range(plo, phi);
    }
    // per axis and blob, the 1-D Gaussian factor at every voxel centre
    std::vector<double> g[3];
    for (int a = 0; a < 3; ++a) {
        g[a].resize(size_t(nb) * dim[a]);
        for (int b = 0; b < nb; ++b) {
            const double inv = 1.0 / (2.0 * sig[b] * sig[b]);
            for (int i = 0; i < dim[a]; ++i) {
                const double d = (i + 0.5) / dim[a] - cen[3 * b + a];
                g[a][size_t(b) * dim[a] + i] = std::exp(-d * d * inv);
            }
        }
    }
    const size_t nx = dim[0], ny = dim[1];
    over_threads(dim[2], nthreads, [&](int k) {
        std::vector<double> wz(nb), wyz(nb);
        for (int b = 0; b < nb; ++b) wz[b] = peak[b] * g[2][size_t(b) * dim[2] + k];
        for (size_t j = 0; j < ny; ++j) {
            for (int b = 0; b < nb; ++b) wyz[b] = wz[b] * g[1][size_t(b) * ny + j];
            T *row = out + (size_t(k) * ny + j) * nx;
            for (size_t i = 0; i < nx; ++i) {
                double v = 0.0;
                for (int b = 0; b < nb; ++b) v += wyz[b] * g[0][size_t(b) * nx + i];
                row[i] = quant(v);
            }
        }
    });
}

bool bad_dims(const int32_t dim[3]) { return !dim || dim[0] <= 0 || dim[1] <= 0 || dim[2] <= 0; }

}  // namespace

extern "C" int orc_synth_blobs_u8(uint64_t seed, const int32_t dim[3], int32_t nblobs,
                                  uint8_t *out, int32_t nthreads) {
    if (bad_dims(dim) || !out || nblobs < 0) return -1;
    blobs(seed, dim, nblobs, out, nthreads, 40.0, 255.0, [](double v) {
        const double q = std::floor(v + 0.5);
        return uint8_t(std::min(255.0, std::max(0.0, q)));
    });
    return 0;
}

extern "C" int orc_synth_blobs_f32(uint64_t seed, const int32_t dim[3], int32_t nblobs,
                                   float *out, int32_t nthreads) {
    if (bad_dims(dim) || !out || nblobs < 0) return -1;
    blobs(seed, dim, nblobs, out, nthreads, 0.15, 0.6,
          [](double v) { return float(v < 1.0 ? v : 1.0); });
    return 0;
}

extern "C" int orc_synth_tubes_u8(uint64_t seed, const int32_t dim[3], int32_t ntubes,
                                  uint8_t *out, int32_t nthreads) {
    if (bad_dims(dim) || !out || ntubes < 0) return -1;
    const int nx = dim[0], ny = dim[1], nz = dim[2];
    over_threads(nz, nthreads, [&](int k) {
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const uint64_t idx = (uint64_t(k) * ny + j) * nx + i;
                out[idx] = uint8_t(std::min(30.0, std::floor(voxel_hash(seed, idx, 1) * 31.0)));
            }
    });
    struct Curve {
        double p[4][3];
        double r;
    };
    Rng r{seed ^ 0x5851F42D4C957F2Dull};
    std::vector<Curve> curves(ntubes);
    for (auto &c : curves) {
        for (int q = 0; q < 4; ++q)
            for (int a = 0; a < 3; ++a) c.p[q][a] = r.range(0.05, 0.95) * dim[a];
        c.r = r.range(2.0, 10.0);
    }
    auto inside = [&](uint64_t idx) {
        const double u1 = voxel_hash(seed, idx, 2), u2 = voxel_hash(seed, idx, 3);
        const double z = std::sqrt(-2.0 * std::log(1.0 - u1)) * std::cos(6.283185307179586 * u2);
        const double v = std::floor(200.0 + 20.0 * z + 0.5);
        return uint8_t(std::min(255.0, std::max(0.0, v)));
    };
    // spheres of radius r every <= r/2 along each curve; thread t owns a
    // range of z-slices
    int nthr = nthreads > 0 ? nthreads : int(std::thread::hardware_concurrency());
    nthr = std::max(1, std::min(nthr, nz));
    over_threads(nthr, nthr, [&](int t) {
        const int z0 = int((long long)nz * t / nthr), z1 = int((long long)nz * (t + 1) / nthr);
        for (const Curve &c : curves) {
            double len = 0.0;
            for (int q = 0; q < 3; ++q) {
                double d2 = 0.0;
                for (int a = 0; a < 3; ++a)
                    d2 += (c.p[q + 1][a] - c.p[q][a]) * (c.p[q + 1][a] - c.p[q][a]);
                len += std::sqrt(d2);
            }
            const int n = std::max(2, int(std::ceil(len / (c.r * 0.5))) + 1);
            const double r2 = c.r * c.r;
            for (int q = 0; q < n; ++q) {
                const double u = double(q) / (n - 1), w = 1.0 - u;
                const double b0 = w * w * w, b1 = 3 * w * w * u, b2 = 3 * w * u * u, b3 = u * u * u;
                double ctr[3];
                int lo[3], hi[3];
                for (int a = 0; a < 3; ++a) {
                    ctr[a] = b0 * c.p[0][a] + b1 * c.p[1][a] + b2 * c.p[2][a] + b3 * c.p[3][a];
                    lo[a] = std::max(0, int(std::floor(ctr[a] - c.r - 0.5)));
                    hi[a] = std::min(dim[a] - 1, int(std::ceil(ctr[a] + c.r + 0.5)));
                }
                lo[2] = std::max(lo[2], z0);
                hi[2] = std::min(hi[2], z1 - 1);
                for (int k = lo[2]; k <= hi[2]; ++k)
                    for (int j = lo[1]; j <= hi[1]; ++j)
                        for (int i = lo[0]; i <= hi[0]; ++i) {
                            const double dx = i + 0.5 - ctr[0], dy = j + 0.5 - ctr[1],
                                         dz = k + 0.5 - ctr[2];
                            if (dx * dx + dy * dy + dz * dz <= r2) {
                                const uint64_t idx = (uint64_t(k) * ny + j) * nx + i;
                                out[idx] = inside(idx);
                            }
                        }
            }
        }
    });
    return 0;
}
