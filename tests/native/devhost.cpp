// devhost.cpp - compiles the product's device header (device.cuh) for the host CPU so
// its DDA traversal (recursive and resumable forms) and its sin/cos can be compared
// with the oracle without a GPU. Test infrastructure only.
//
// Host stand-ins for the CUDA intrinsics device.cuh uses; each has the semantics the
// device instruction has (round-toward-zero saturating conversions, raw bit casts).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

static inline unsigned __float2uint_rz(float f) {
    if (!(f > 0.0f)) return 0u;
    if (f >= 4294967296.0f) return 0xFFFFFFFFu;
    return (unsigned)f;
}
static inline int __float2int_rz(float f) {
    if (f != f) return 0;
    if (f >= 2147483648.0f) return 2147483647;
    if (f <= -2147483648.0f) return (int)0x80000000u;
    return (int)f;
}
static inline float __uint_as_float(unsigned u) { float f; std::memcpy(&f, &u, 4); return f; }
static inline unsigned __float_as_uint(float f) { unsigned u; std::memcpy(&u, &f, 4); return u; }
static inline float __uint2float_rn(unsigned u) { return (float)u; }
static inline float __int_as_float(int i) { float f; std::memcpy(&f, &i, 4); return f; }
template <class T> static inline T __ldg(const T* p) { return *p; }
static inline unsigned atomicAdd(unsigned* p, unsigned v) { const unsigned o = *p; *p = o + v; return o; }
using std::isinf;
using std::isnan;
using std::max;
using std::min;
#ifndef __noinline__
#define __noinline__ __attribute__((noinline))
#endif

#include "device.cuh"

using namespace vxr::dev;

static World make_world(const uint32_t* grid, const uint8_t* uber, const uint32_t* bricks) {
    World w;
    w.grid = grid; w.uber = uber; w.bricks = bricks; w.bbox = nullptr; w.bbox0 = nullptr; w.ubox0 = nullptr; w.lgeom = nullptr; w.lemit = nullptr; w.nlights = 0;
    return w;
}

// The per-face form of the area-light sample (RandomPointOnVoxel, tools.cl:499-577) that
// the GPU path used before its per-axis form, kept here as a second restatement to
// check the per-axis form against, bit for bit (the GPU parity tests pin both to the
// oracle through whole frames).
__device__ __forceinline__ float3 face_point_perface(float4 g, uint32_t face, float r0, float r1) {
    // N = normals[face], T = normals[(face / 3) * 3 + (face + 1) % 3], B = ... + (face + 2) % 3
    const float size = g.w, h = 0.5f * size;
    const float s = face < 3 ? 1.0f : -1.0f;
    const uint32_t an = face % 3, at = (an + 1) % 3, ab = (an + 2) % 3;
    float c[3] = {g.x, g.y, g.z}, p[3];
    p[an] = c[an] + h * s;                                // center + 0.5*size*N
    p[at] = (c[at] - h * s) + (r0 * size) * s;            // - 0.5*size*T + r0*size*T
    p[ab] = (c[ab] - h * s) + (r1 * size) * s;            // - 0.5*size*B + r1*size*B
    return f3(p[0], p[1], p[2]);
}

__device__ __forceinline__ float3 sample_area_light_perface(float4 g, float3 spo, uint32_t& seed, float* invp, uint32_t* ncode) {
    const uint32_t seed0 = seed;
    float sa[6];
    float total = 0.0f;
    const float area = g.w * g.w, h = 0.5f * g.w;
#pragma unroll
    for (int f = 0; f < 6; f++) {
        const float r0 = rnd(seed), r1 = rnd(seed);
        const float s = f < 3 ? 1.0f : -1.0f;
        const uint32_t an = f % 3;
        const float pa = comp(f3(g.x, g.y, g.z), an) + h * s;
        sa[f] = 0.0f;
        if (s * (comp(spo, an) - pa) > 0.0f) {       // dot(N, -L) > 0 <=> s * R[an] < 0
            const float3 P = face_point_perface(g, f, r0, r1);
            const float3 R = sub(P, spo);
            const float dd = dot3(R, R);
            const float inv = 1.0f / sqrtf(dd);
            const float nl = -(s * (comp(R, an) * inv));
            const float d = fmaxf(1e-5f, dd);
            sa[f] = (nl * area) / d;
            total += sa[f];
        }
    }
    const float r2 = rnd(seed);
    uint32_t index = 0;
    float pdf;
    if (total == 0.0f) {
        pdf = __int_as_float(0x7fffffff);   // 0/0: NaN -> weight 0
    } else {
        pdf = sa[0] / total;
        float cdf = pdf;
        if (cdf < r2) {
            for (int i = 1; i < 6; i++) {
                const float p = sa[i] / total;
                cdf = cdf + p;
                index = i;
                if (cdf >= r2) break;
            }
            pdf = sa[index] / total;
        }
    }
    float wgt = 1.0f / pdf;
    if (isinf(wgt) || isnan(wgt)) wgt = 0.0f;
    *invp = wgt;
    *ncode = index;
    // regenerate the two draws of the chosen face
    uint32_t s2 = seed0;
    for (uint32_t i = 0; i < 2 * index; i++) xs32(s2);
    const float r0 = rnd(s2), r1 = rnd(s2);
    return face_point_perface(g, index, r0, r1);
}


extern "C" {

uint32_t dh_trace(int mode, const uint32_t* grid, const uint8_t* uber, const uint32_t* bricks, const float* O,
                  const float* D, int steps, uint32_t through, uint32_t mask, float* dist, uint32_t* side) {
    const World w = make_world(grid, uber, bricks);
    float d = 0.0f;
    uint32_t s = 0;
    uint32_t v;
    if (mode == 0) v = trace<0>(w, O[0], O[1], O[2], D[0], D[1], D[2], steps, through, mask, &d, &s);
    else if (mode == 1) v = trace<1>(w, O[0], O[1], O[2], D[0], D[1], D[2], steps, through, mask, &d, &s);
    else v = trace<2>(w, O[0], O[1], O[2], D[0], D[1], D[2], steps, through, mask, &d, &s);
    *dist = d;
    *side = s;
    return v;
}

// trace<mode> with brick skipping (bbox: opaque-voxel boxes, bbox0: non-zero-voxel boxes)
// and uber-cell skipping for budget-free primary rays (ubox0, or null)
uint32_t dh_trace_skip(int mode, const uint32_t* grid, const uint8_t* uber, const uint32_t* bricks,
                       const uint32_t* bbox, const uint32_t* bbox0, const uint32_t* ubox0, const float* O,
                       const float* D, int steps, uint32_t through, uint32_t mask, float* dist, uint32_t* side) {
    World w = make_world(grid, uber, bricks);
    w.bbox = bbox;
    w.bbox0 = bbox0;
    w.ubox0 = ubox0;
    float d = 0.0f;
    uint32_t s = 0;
    uint32_t v;
    if (mode == 0) v = trace<0>(w, O[0], O[1], O[2], D[0], D[1], D[2], steps, through, mask, &d, &s);
    else if (mode == 1) v = trace<1>(w, O[0], O[1], O[2], D[0], D[1], D[2], steps, through, mask, &d, &s);
    else v = trace<2>(w, O[0], O[1], O[2], D[0], D[1], D[2], steps, through, mask, &d, &s);
    *dist = d;
    *side = s;
    return v;
}

// resumable walker run to completion; *status: 1 hit, 2 miss; *visits: cells visited
uint32_t dh_walk(const uint32_t* grid, const uint8_t* uber, const uint32_t* bricks, const float* O, const float* D,
                 int steps, float* dist, uint32_t* side, int* status, int* visits) {
    const World w = make_world(grid, uber, bricks);
    Walker k;
    int st = walk_init(k, w, O[0], O[1], O[2], D[0], D[1], D[2], steps);
    int n = 0;
    while (st == WALK_CONTINUE) {
        st = walk_step(k, w);
        n++;
    }
    *status = st;
    *visits = n;
    if (st == WALK_HIT) {
        *dist = k.dist;
        *side = k.side;
        return k.voxel;
    }
    *dist = 0.0f;
    *side = 0;
    return 0u;
}

// the walker run in bursts of `burst` visits (the shadow tracer's form)
uint32_t dh_walk_burst(const uint32_t* grid, const uint8_t* uber, const uint32_t* bricks, const float* O,
                       const float* D, int steps, int burst, float* dist, uint32_t* side, int* status) {
    const World w = make_world(grid, uber, bricks);
    Walker k;
    int st = walk_init(k, w, O[0], O[1], O[2], D[0], D[1], D[2], steps);
    while (st == WALK_CONTINUE) {
        for (int i = 0; i < burst && st == WALK_CONTINUE; i++) st = walk_step(k, w);
    }
    *status = st;
    if (st == WALK_HIT) {
        *dist = k.dist;
        *side = k.side;
        return k.voxel;
    }
    *dist = 0.0f;
    *side = 0;
    return 0u;
}

// the walker with brick skipping (bbox: per brick the packed box of its opaque voxels);
// *visits: cells visited
int dh_walk_skip(const uint32_t* grid, const uint8_t* uber, const uint32_t* bricks, const uint32_t* bbox,
                 const float* O, const float* D, int steps, float* dist, uint32_t* side, int* visits) {
    World w = make_world(grid, uber, bricks);
    w.bbox = bbox;
    Walker k;
    int st = walk_init(k, w, O[0], O[1], O[2], D[0], D[1], D[2], steps);
    int n = 0;
    while (st == WALK_CONTINUE) {
        st = walk_step(k, w);
        n++;
    }
    *dist = st == WALK_HIT ? k.dist : 0.0f;
    *side = st == WALK_HIT ? k.side : 0u;
    *visits = n;
    return st;
}

// a shadow ray through the walker (brick skipping when bbox is given) as the persistent
// tracer runs it, with or without the visibility early-out towards the emitter cube
// [pos, pos + size); returns 1 when the visibility test passes (hit voxel in the cube),
// *visits: cells visited
int dh_shadow(const uint32_t* grid, const uint8_t* uber, const uint32_t* bricks, const uint32_t* bbox, const float* O,
              const float* D, uint32_t pos, uint32_t size, int early, int* visits) {
    World w = make_world(grid, uber, bricks);
    w.bbox = bbox;
    Walker k;
    int st = walk_init(k, w, O[0], O[1], O[2], D[0], D[1], D[2], 128);
    if (early && st == WALK_CONTINUE) walk_target(k, pos, size);
    int n = 0;
    while (st == WALK_CONTINUE) {
        st = early ? walk_step<kWalkEarly>(k, w) : walk_step(k, w);
        n++;
    }
    *visits = n;
    const float d2 = st == WALK_HIT ? k.dist : 0.0f;
    const uint32_t s2 = st == WALK_HIT ? k.side : 0u;
    const float3 L = f3(D[0], D[1], D[2]);
    const float ns = side_sign(s2, L);
    const float hx = L.x * d2 + O[0], hy = L.y * d2 + O[1], hz = L.z * d2 + O[2];
    const uint32_t vx = f2u(hx - (s2 == 0 ? ns * 0.1f : 0.0f));
    const uint32_t vy = f2u(hy - (s2 == 1 ? ns * 0.1f : 0.0f));
    const uint32_t vz = f2u(hz - (s2 == 2 ? ns * 0.1f : 0.0f));
    const uint32_t ey = pos / (1024u * 1024u), ez = (pos / 1024u) % 1024u, ex = pos % 1024u;
    return ex <= vx && ex + size > vx && ey <= vy && ey + size > vy && ez <= vz && ez + size > vz;
}

void dh_sincos(float a, float* s, float* c) { sincos_vx(a, s, c); }

// area-light sample, per-axis form (device.cuh) and per-face form (above); out = point xyz, inv, face, seed
void dh_area_sample(int which, const float* lg, const float* spo, uint32_t seed, float* out) {
    const float4 g = make_float4(lg[0], lg[1], lg[2], lg[3]);
    const float3 p = f3(spo[0], spo[1], spo[2]);
    float inv = 0.0f;
    uint32_t nc = 0;
    const float3 q = which ? sample_area_light_perface(g, p, seed, &inv, &nc) : sample_area_light(g, p, seed, &inv, &nc);
    out[0] = q.x; out[1] = q.y; out[2] = q.z; out[3] = inv;
    std::memcpy(out + 4, &nc, 4);
    std::memcpy(out + 5, &seed, 4);
}

}  // extern "C"
