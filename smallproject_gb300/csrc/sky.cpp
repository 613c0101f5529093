// sky.cpp - host side of the sky dome: World::UpdateSkylights with World::SampleSky
// (template/world.cpp:876-922), which integrate the sky texture into the six sky-light
// colours that shading uses for the axis normals.
#include <cmath>
#include <cstdint>

#include "internal.hpp"
#include "vxr.h"

namespace {

struct V3 {
    float x, y, z;
};

V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }

// World::SampleSky: bilinear lookup of direction D in the z-up texture (theta from +z,
// phi around it), texel rows wrapping at the end of the image
V3 sample_sky(const float* t, int iw, int ih, V3 D) {
    const float PI = 3.14159265358979323846264f;
    const float INV2PI = 0.15915494309189533576888f, INVPI = 0.31830988618379067153777f;
    const float theta = (float)std::acos((double)std::fmin(std::fmax(D.z, -1.0f), 1.0f));
    float phi = (float)std::atan2((double)D.y, (double)D.x);
    if (phi < 0.0f) phi += 2.0f * PI;
    const float u = ((float)iw * phi) * INV2PI - 0.5f, v = ((float)ih * theta) * INVPI - 0.5f;
    const float fu = u - std::floor(u), fv = v - std::floor(v);
    const int iu = (int)u, iv = (int)v, n = iw * ih;
    const float* a = t + 4 * (size_t)((iu + iv * iw) % n);
    const float* b = t + 4 * (size_t)((iu + 1 + iv * iw) % n);
    const float* c = t + 4 * (size_t)((iu + (iv + 1) * iw) % n);
    const float* d = t + 4 * (size_t)((iu + 1 + (iv + 1) * iw) % n);
    const float gu = 1.0f - fu, gv = 1.0f - fv;
    V3 r;
    float* o = &r.x;
    for (int k = 0; k < 3; k++) o[k] = (((a[k] * gu) * gv + (b[k] * fu) * gv) + (c[k] * gu) * fv) + (d[k] * fu) * fv;
    return r;
}

// DiffuseReflectionCosWeighted: cosine-weighted direction around N
V3 cos_weighted(float r0, float r1, V3 N) {
    V3 T = cross(N, std::fabs(N.y) > 0.99f ? V3{1, 0, 0} : V3{0, 1, 0});
    const float inv = 1.0f / std::sqrt(T.x * T.x + T.y * T.y + T.z * T.z);
    T = {T.x * inv, T.y * inv, T.z * inv};
    const V3 B = cross(T, N);
    const float term1 = 6.28318530717958647692528f * r0, term2 = std::sqrt(1.0f - r1);
    const float ct = (float)std::cos((double)term1) * term2, st = (float)std::sin((double)term1) * term2;
    const float sr = std::sqrt(r1);
    return {(ct * T.x + st * B.x) + sr * N.x, (ct * T.y + st * B.y) + sr * N.y, (ct * T.z + st * B.z) + sr * N.z};
}

float rnd(uint32_t& s) {   // xorshift32, as the reference's RandomFloat
    s ^= s << 13;
    s ^= s >> 17;
    s ^= s << 5;
    return (float)s * 2.3283064365387e-10f;
}

}  // namespace

extern "C" int vxr_sky_lights(const float* rgba, uint32_t w, uint32_t h, uint32_t seed, float sky_light[24]) {
    VXR_CHECK_ARG(rgba && sky_light, "vxr_sky_lights: null argument");
    VXR_CHECK_ARG(w >= 1 && h >= 1 && w <= 65536 && h <= 65536 && (uint64_t)w * h < (1ull << 31),
                  "vxr_sky_lights: size out of range");
    // the six normals of skyLight, in its order
    static const V3 N[6] = {{-1, 0, 0}, {1, 0, 0}, {0, 0, -1}, {0, 0, 1}, {0, -1, 0}, {0, 1, 0}};
    uint32_t s = seed ? seed : 0x9E3779B9u;   // xorshift32 never leaves 0
    for (int i = 0; i < 6; i++) {
        float sum[3] = {0.0f, 0.0f, 0.0f};
        for (int j = 0; j < 4096; j++) {
            const float sx = (float)(j & 15) * 0.0625f, sy = (float)((j >> 4) & 15) * 0.0625f;   // 256 strata
            const float r0 = rnd(s) * 0.0625f + sx, r1 = rnd(s) * 0.0625f + sy;
            const V3 c = sample_sky(rgba, (int)w, (int)h, cos_weighted(r0, r1, N[i]));
            sum[0] += c.x;
            sum[1] += c.y;
            sum[2] += c.z;
        }
        for (int k = 0; k < 3; k++) sky_light[4 * i + k] = sum[k] * (1.0f / 4096.0f);
        sky_light[4 * i + 3] = 0.0f;
    }
    return VXR_OK;
}
