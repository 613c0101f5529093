// scene.cpp - procedural benchmark scenes (no reference counterpart: the reference's
// thesis scenes need .vox assets that are absent, so the benchmark configurations
// are generated). Deterministic across platforms: integer hashing plus IEEE double
// arithmetic (+, -, *, /, floor) only - no libm transcendental calls.
//
// Terrain: heightfield h(x,z) = s*(height_base + height_amp*fBm(x/s, z/s)), s = extent/256,
// fBm = normalised sum of value-noise octaves (smoothstep-interpolated lattice values,
// base frequency base_freq, frequency doubling, amplitude gain). Column voxels y < h are
// solid; optional caves remove voxels where 3D value noise exceeds cave_threshold.
// Visible voxels (solid with an empty 6-neighbour) get a random 4-bit albedo; voxels
// that no ray can reach (all 6 neighbours solid) get one interior colour, so that
// buried bricks collapse to solid cells. No ray ever hits an interior voxel first,
// so this choice does not change any rendered value.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <unordered_set>
#include <vector>

#include "world.hpp"

namespace vxr {

namespace {

inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline uint64_t hash4(uint64_t a, uint64_t b, uint64_t c, uint64_t d) {
    return mix64(a ^ mix64(b ^ mix64(c ^ mix64(d))));
}
inline double u01(uint64_t h) { return (double)(h >> 11) * (1.0 / 9007199254740992.0); }

struct Rng {  // counter-based stream
    uint64_t key, n = 0;
    explicit Rng(uint64_t k) : key(k) {}
    double next() { return u01(hash4(key, n++, 0x51ED, 7)); }
    uint32_t below(uint32_t m) { return (uint32_t)(next() * m) % m; }
    double normal() {  // Irwin-Hall(12) - 6: unit variance, no transcendental calls
        double s = 0;
        for (int i = 0; i < 12; i++) s += next();
        return s - 6.0;
    }
};

inline double smooth(double t) { return t * t * (3.0 - 2.0 * t); }

double value2(double x, double z, uint64_t key) {
    const double fx = std::floor(x), fz = std::floor(z);
    const int64_t ix = (int64_t)fx, iz = (int64_t)fz;
    const double tx = smooth(x - fx), tz = smooth(z - fz);
    const double v00 = u01(hash4(key, (uint64_t)ix, (uint64_t)iz, 11));
    const double v10 = u01(hash4(key, (uint64_t)(ix + 1), (uint64_t)iz, 11));
    const double v01 = u01(hash4(key, (uint64_t)ix, (uint64_t)(iz + 1), 11));
    const double v11 = u01(hash4(key, (uint64_t)(ix + 1), (uint64_t)(iz + 1), 11));
    const double a = v00 + (v10 - v00) * tx, b = v01 + (v11 - v01) * tx;
    return a + (b - a) * tz;
}

double value3(double x, double y, double z, uint64_t key) {
    const double fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
    const int64_t ix = (int64_t)fx, iy = (int64_t)fy, iz = (int64_t)fz;
    const double tx = smooth(x - fx), ty = smooth(y - fy), tz = smooth(z - fz);
    double c[2][2][2];
    for (int a = 0; a < 2; a++)
        for (int b = 0; b < 2; b++)
            for (int d = 0; d < 2; d++)
                c[a][b][d] = u01(hash4(key ^ 0xC0FFEEull, (uint64_t)(ix + a), (uint64_t)(iy + b), (uint64_t)(iz + d)));
    double e[2][2];
    for (int b = 0; b < 2; b++)
        for (int d = 0; d < 2; d++) e[b][d] = c[0][b][d] + (c[1][b][d] - c[0][b][d]) * tx;
    const double f0 = e[0][0] + (e[1][0] - e[0][0]) * ty, f1 = e[0][1] + (e[1][1] - e[0][1]) * ty;
    return f0 + (f1 - f0) * tz;
}

struct Terrain {
    vxr_scene_desc d;
    double s;
    uint32_t ext;
    std::vector<uint32_t> H;   // first empty y per column
    uint64_t key;

    explicit Terrain(const vxr_scene_desc& desc) : d(desc) {
        ext = std::min<uint32_t>(std::max<uint32_t>(desc.extent, 8), kMap);
        s = ext / 256.0;
        key = mix64(0xA11CE5ull + desc.seed);
        H.resize((size_t)ext * ext);
        for (uint32_t z = 0; z < ext; z++)
            for (uint32_t x = 0; x < ext; x++) H[(size_t)z * ext + x] = height_at(x, z);
    }
    uint32_t height_at(uint32_t x, uint32_t z) const {
        double sum = 0, norm = 0, amp = 1, f = d.base_freq;
        for (uint32_t o = 0; o < std::max<uint32_t>(d.octaves, 1); o++) {
            sum += amp * (2.0 * value2(x / s * f, z / s * f, key + 101 * o) - 1.0);
            norm += amp;
            amp *= d.gain;
            f *= 2.0;
        }
        const double h = s * (d.height_base + d.height_amp * (sum / norm));
        const double hc = std::min<double>(std::max<double>(std::floor(h), 1.0), (double)ext - 1.0);
        return (uint32_t)hc;
    }
    uint32_t height(uint32_t x, uint32_t z) const { return H[(size_t)z * ext + x]; }
    bool cave(uint32_t x, uint32_t y, uint32_t z) const {
        if (!(d.cave_threshold > 0) || y < 4) return false;
        const double f = 1.0 / (24.0 * s);
        return value3(x * f, y * f, z * f, key) > d.cave_threshold;
    }
    bool solid(int x, int y, int z) const {
        if (x < 0 || y < 0 || z < 0 || x >= (int)ext || z >= (int)ext) return false;
        if ((uint32_t)y >= height((uint32_t)x, (uint32_t)z)) return false;
        return !cave((uint32_t)x, (uint32_t)y, (uint32_t)z);
    }
    uint32_t albedo(uint32_t x, uint32_t y, uint32_t z) const {
        const double span = d.albedo_hi - d.albedo_lo;
        uint32_t q[3];
        for (int c = 0; c < 3; c++) {
            const double v = d.albedo_lo + span * u01(hash4(key + 7, x, y, ((uint64_t)z << 2) | (uint64_t)c));
            q[c] = (uint32_t)std::min(15.0, std::floor(15.0 * v + 0.5));
        }
        return VXR_VOXEL(q[0], q[1], q[2], 15, 0);
    }
    uint32_t air_top() const {
        const double top = std::ceil(s * (d.height_base + d.height_amp)) + 32.0 * s;
        return (uint32_t)std::min<double>(top, (double)ext);
    }
};

const uint32_t kInterior = VXR_VOXEL(8, 8, 8, 15, 0);

uint32_t encode_emitter(double r, double g, double b) {
    const double mx = std::max(r, std::max(g, b));
    uint32_t M = (uint32_t)std::min(255.0, std::max(1.0, std::ceil(mx)));
    uint32_t q[3];
    const double c[3] = {r, g, b};
    for (int i = 0; i < 3; i++) q[i] = (uint32_t)std::min(15.0, std::max(0.0, std::floor(15.0 * c[i] / M + 0.5)));
    return VXR_VOXEL(q[0], q[1], q[2], 15, M);
}

// Fill one 8^3 cell: returns true when uniform (value in *uniform), else writes 512 voxels.
bool build_cell(const Terrain& T, uint32_t bx, uint32_t by, uint32_t bz, uint32_t* out, uint32_t* uniform) {
    const uint32_t x0 = bx * 8, y0 = by * 8, z0 = bz * 8;
    // quick classification from the column heights of the cell and its 1-voxel ring
    uint32_t hmin = 0xFFFFFFFFu, hmax = 0;
    for (int dz = -1; dz <= 8; dz++)
        for (int dx = -1; dx <= 8; dx++) {
            const int x = (int)x0 + dx, z = (int)z0 + dz;
            uint32_t h = 0;
            if (x >= 0 && z >= 0 && x < (int)T.ext && z < (int)T.ext) h = T.height((uint32_t)x, (uint32_t)z);
            if (dx >= 0 && dx < 8 && dz >= 0 && dz < 8) hmax = std::max(hmax, h);
            hmin = std::min(hmin, h);
        }
    if (y0 >= hmax) { *uniform = 0; return true; }
    const bool caves = T.d.cave_threshold > 0;
    if (!caves && y0 + 9 <= hmin && y0 >= 1) { *uniform = kInterior; return true; }
    // general case: padded solidity block
    bool S[10][10][10];
    for (int dy = 0; dy < 10; dy++)
        for (int dz = 0; dz < 10; dz++)
            for (int dx = 0; dx < 10; dx++)
                S[dy][dz][dx] = T.solid((int)x0 + dx - 1, (int)y0 + dy - 1, (int)z0 + dz - 1);
    bool first = true, same = true;
    uint32_t v0 = 0;
    for (uint32_t lz = 0; lz < 8; lz++)
        for (uint32_t ly = 0; ly < 8; ly++)
            for (uint32_t lx = 0; lx < 8; lx++) {
                uint32_t v = 0;
                if (S[ly + 1][lz + 1][lx + 1]) {
                    const bool inner = S[ly][lz + 1][lx + 1] && S[ly + 2][lz + 1][lx + 1] && S[ly + 1][lz][lx + 1] &&
                                       S[ly + 1][lz + 2][lx + 1] && S[ly + 1][lz + 1][lx] && S[ly + 1][lz + 1][lx + 2];
                    v = inner ? kInterior : T.albedo(x0 + lx, y0 + ly, z0 + lz);
                }
                out[lx + ly * 8 + lz * 64] = v;
                if (first) { v0 = v; first = false; }
                else if (v != v0) same = false;
            }
    if (same) { *uniform = v0; return true; }
    return false;
}

}  // namespace

int scene_preset(int config, vxr_scene_desc* d) {
    std::memset(d, 0, sizeof(*d));
    d->extent = 256; d->seed = 1; d->octaves = 4; d->base_freq = 1.0f / 64.0f; d->gain = 0.5f;
    d->height_base = 64.0f; d->height_amp = 48.0f; d->albedo_lo = 0.2f; d->albedo_hi = 0.9f;
    d->cave_threshold = 0.0f; d->emitters = 64; d->emitter_mode = VXR_EMIT_ABOVE_SURFACE;
    d->radiance_lo = 1.0f; d->radiance_hi = 10.0f;
    d->blob_count = 32; d->blob_sigma = 24.0f; d->blob_fraction = 0.7f;
    d->layer_lo = 40; d->layer_hi = 44; d->scatter_fraction = 0.1f;
    switch (config) {
    case 0: break;
    case 1: d->extent = 1024; d->seed = 2; d->emitters = 4096; d->emitter_mode = VXR_EMIT_AIR; break;
    case 2: d->extent = 512; d->seed = 3; d->emitters = 1024; d->emitter_mode = VXR_EMIT_AIR; break;
    case 3: d->extent = 1024; d->seed = 4; d->emitters = 65536; d->emitter_mode = VXR_EMIT_BLOBS; break;
    case 4:
        d->extent = 1024; d->seed = 5; d->octaves = 6; d->cave_threshold = 0.6f; d->emitters = 1048576;
        d->emitter_mode = VXR_EMIT_LAYER; d->radiance_lo = 0.5f; d->radiance_hi = 20.0f;
        break;
    default: return VXR_E_INVALID;
    }
    return VXR_OK;
}

int scene_height(const vxr_scene_desc* d, uint32_t x, uint32_t z, uint32_t* h) {
    vxr_scene_desc dd = *d;
    Terrain T(dd);
    if (x >= T.ext || z >= T.ext) return VXR_E_INVALID;
    *h = T.height(x, z);
    return VXR_OK;
}

int scene_generate(World& w, const vxr_scene_desc& desc) {
    Terrain T(desc);
    w.clear();
    const uint32_t nc = (T.ext + 7) / 8;
    // pass 1 (parallel): classify every cell; pass 2 (serial): assign bricks in scan order
    const size_t ncell = (size_t)nc * nc * nc;
    std::vector<uint32_t> uniformVal(ncell, 0);
    std::vector<uint8_t> isUniform(ncell, 1);
    std::vector<std::vector<uint32_t>> tmp(ncell);
#pragma omp parallel for schedule(dynamic, 16)
    for (long long i = 0; i < (long long)ncell; i++) {
        const uint32_t bx = (uint32_t)(i % nc), bz = (uint32_t)((i / nc) % nc), by = (uint32_t)(i / ((size_t)nc * nc));
        uint32_t buf[512];
        uint32_t u = 0;
        if (build_cell(T, bx, by, bz, buf, &u)) {
            uniformVal[i] = u;
        } else {
            isUniform[i] = 0;
            tmp[i].assign(buf, buf + 512);
        }
    }
    for (size_t i = 0; i < ncell; i++) {
        const uint32_t bx = (uint32_t)(i % nc), bz = (uint32_t)((i / nc) % nc), by = (uint32_t)(i / ((size_t)nc * nc));
        const uint32_t ci = cell_index(bx, by, bz);
        if (isUniform[i]) {
            w.grid[ci] = uniformVal[i] << 1;
        } else {
            const uint32_t b = w.new_brick();
            std::copy(tmp[i].begin(), tmp[i].end(), w.bricks.begin() + (size_t)b * kBrick);
            uint32_t zc = 0;
            for (uint32_t v : tmp[i]) zc += (v == 0);
            w.zeroes[b] = zc;
            w.grid[ci] = (b << 1) | 1u;
            std::vector<uint32_t>().swap(tmp[i]);
        }
    }
    // emitters
    const bool track = w.trackLights;
    w.trackLights = false;
    Rng rng(mix64(0xE111ull + desc.seed));
    std::unordered_set<uint64_t> used;
    used.reserve(desc.emitters * 2 + 16);
    const uint32_t top = T.air_top();
    auto place = [&](uint32_t x, uint32_t y, uint32_t z) {
        const uint64_t key = (uint64_t)x | ((uint64_t)y << 20) | ((uint64_t)z << 40);
        if (!used.insert(key).second) return false;
        const double r = desc.radiance_lo + (desc.radiance_hi - desc.radiance_lo) * rng.next();
        const double g = desc.radiance_lo + (desc.radiance_hi - desc.radiance_lo) * rng.next();
        const double b = desc.radiance_lo + (desc.radiance_hi - desc.radiance_lo) * rng.next();
        w.set(x, y, z, encode_emitter(r, g, b));
        return true;
    };
    auto uniform_air = [&]() {
        for (int tries = 0; tries < 1000000; tries++) {
            const uint32_t x = rng.below(T.ext), z = rng.below(T.ext);
            const uint32_t y = rng.below(std::max<uint32_t>(top, 1));
            if (T.solid((int)x, (int)y, (int)z)) continue;
            if (place(x, y, z)) return;
        }
    };
    const uint32_t n = desc.emitters;
    if (desc.emitter_mode == VXR_EMIT_ABOVE_SURFACE) {
        for (uint32_t i = 0; i < n;) {
            const uint32_t x = rng.below(T.ext), z = rng.below(T.ext);
            const uint32_t y = T.height(x, z) + rng.below(8);   // 1..8 above the top solid voxel
            if (y < T.ext && !T.solid((int)x, (int)y, (int)z) && place(x, y, z)) i++;
        }
    } else if (desc.emitter_mode == VXR_EMIT_AIR) {
        for (uint32_t i = 0; i < n; i++) uniform_air();
    } else if (desc.emitter_mode == VXR_EMIT_BLOBS) {
        std::vector<double> c(3 * std::max<uint32_t>(desc.blob_count, 1));
        for (uint32_t k = 0; k < std::max<uint32_t>(desc.blob_count, 1); k++) {
            for (;;) {
                const uint32_t x = rng.below(T.ext), z = rng.below(T.ext), y = rng.below(std::max<uint32_t>(top, 1));
                if (!T.solid((int)x, (int)y, (int)z)) { c[3 * k] = x; c[3 * k + 1] = y; c[3 * k + 2] = z; break; }
            }
        }
        const uint32_t nb = (uint32_t)std::floor(n * (double)desc.blob_fraction + 0.5);
        for (uint32_t i = 0; i < nb;) {
            const uint32_t k = i % std::max<uint32_t>(desc.blob_count, 1);
            const double x = std::floor(c[3 * k] + desc.blob_sigma * rng.normal());
            const double y = std::floor(c[3 * k + 1] + desc.blob_sigma * rng.normal());
            const double z = std::floor(c[3 * k + 2] + desc.blob_sigma * rng.normal());
            if (x < 0 || y < 0 || z < 0 || x >= T.ext || y >= T.ext || z >= T.ext) continue;
            if (T.solid((int)x, (int)y, (int)z)) continue;
            if (place((uint32_t)x, (uint32_t)y, (uint32_t)z)) i++;
        }
        for (uint32_t i = nb; i < n; i++) uniform_air();
    } else if (desc.emitter_mode == VXR_EMIT_LAYER) {
        const uint32_t ns = (uint32_t)std::floor(n * (double)desc.scatter_fraction + 0.5);
        const uint32_t nl = n - ns;
        const uint32_t lo = desc.layer_lo, hi = std::max(desc.layer_hi, desc.layer_lo);
        for (uint32_t i = 0; i < nl;) {
            const uint32_t x = rng.below(T.ext), z = rng.below(T.ext), y = lo + rng.below(hi - lo + 1);
            if (place(x, y, z)) i++;
        }
        for (uint32_t i = 0; i < ns; i++) uniform_air();
    }
    w.trackLights = track;
    w.optimize();
    w.scan_lights();
    return VXR_OK;
}

// Catmull-Rom (uniform) through 8 seeded control points on a jittered ring above the
// terrain; the camera looks at the world centre at the base terrain height.
int camera_path(const vxr_scene_desc* d, uint32_t seed, uint32_t f, uint32_t n, float pos[3], float target[3]) {
    static const double dirs[8][2] = {{1, 0}, {0.70710678118654752, 0.70710678118654752}, {0, 1},
                                      {-0.70710678118654752, 0.70710678118654752}, {-1, 0},
                                      {-0.70710678118654752, -0.70710678118654752}, {0, -1},
                                      {0.70710678118654752, -0.70710678118654752}};
    const double ext = std::min<uint32_t>(std::max<uint32_t>(d->extent, 8), kMap);
    const double s = ext / 256.0;
    Rng rng(mix64(0xCA11ull + seed));
    double P[8][3];
    for (int i = 0; i < 8; i++) {
        const double r = ext * (0.22 + 0.12 * rng.next());
        P[i][0] = ext * 0.5 + r * dirs[i][0];
        P[i][2] = ext * 0.5 + r * dirs[i][1];
        P[i][1] = s * (d->height_base + d->height_amp) + s * (8.0 + 24.0 * rng.next());
    }
    const double t = (n > 0 ? (double)(f % n) / n : 0.0) * 8.0;
    const int seg = (int)std::floor(t);
    const double u = t - seg;
    const double* p0 = P[(seg + 7) % 8];
    const double* p1 = P[seg % 8];
    const double* p2 = P[(seg + 1) % 8];
    const double* p3 = P[(seg + 2) % 8];
    const double u2 = u * u, u3 = u2 * u;
    for (int k = 0; k < 3; k++) {
        const double v = 0.5 * ((2 * p1[k]) + (-p0[k] + p2[k]) * u + (2 * p0[k] - 5 * p1[k] + 4 * p2[k] - p3[k]) * u2 +
                                (-p0[k] + 3 * p1[k] - 3 * p2[k] + p3[k]) * u3);
        pos[k] = (float)v;
    }
    target[0] = (float)(ext * 0.5);
    target[1] = (float)(s * d->height_base);
    target[2] = (float)(ext * 0.5);
    return VXR_OK;
}

}  // namespace vxr
