// device.cuh - device-side building blocks of the Voxel ReSTIR render path (sm_103a).
//
// Arithmetic contract (shared with the CPU oracle, which checks it bit for bit):
// every float operation is an IEEE-754 binary32 op with round-to-nearest and no
// contraction (this translation unit builds with --fmad=false, IEEE div/sqrt),
// evaluated in the order the reference kernels write them. That makes the DDA hit
// (voxel, distance bits, side) and every reservoir field reproducible exactly.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace vxr {
namespace dev {

// ---- world as seen by the kernels ----------------------------------------------------
// Light table: per light two float4, built once per upload by build_light_table:
//   geom = (cx, cy, cz, size)      centre = coords + 0.5*size      (tools.cl:606-607)
//   emit = (er, eg, eb, bits(pos)) rgb/15 * strength * 1/pi        (phat.cl:8-12)
struct World {
    const uint32_t* __restrict__ grid;    // 128^3 cells, x + z*128 + y*16384
    const uint8_t* __restrict__ uber;     // 32^3 occupancy, x + z*32 + y*1024
    const uint32_t* __restrict__ bricks;  // nbricks * 512 voxels
    // per brick, or null: the box of its opaque voxels (type 15), corners in voxels from
    // the brick's corner: low x, y, z in bits 0-2, 3-5, 6-8, high x, y, z (inclusive) in
    // bits 9-11, 12-14, 15-17; kNoOpaque when the brick has no opaque voxel
    const uint32_t* __restrict__ bbox;
    // the same for the non-zero voxels (what stops a primary ray), or null
    const uint32_t* __restrict__ bbox0;
    // per uber cell (x + z*32 + y*1024), or null: the box of its non-zero voxels, 5 bits
    // per corner coordinate in voxels from the cell's corner (low x, y, z in bits 0-14,
    // high, inclusive, in bits 15-29), kNoOpaque when the cell is empty
    const uint32_t* __restrict__ ubox0;
    const float4* __restrict__ lgeom;
    const float4* __restrict__ lemit;
    uint32_t nlights;
    // shadow tracer's brick cache (walk_step<1> only): an open-addressed table of 2^bcLog2
    // keys (brick << 11 | slot, kNoKey empty) and per slot the brick's 512-bit opacity mask
    // (16 words), both in shared memory; bcCount (calibration, global): per brick the
    // number of brick walks, or null
    const uint32_t* bcKeys = nullptr;
    const uint32_t* bcMask = nullptr;
    uint32_t* bcCount = nullptr;
    int bcLog2 = 0;
};

// Sky dome in device memory: World::LoadSky / UpdateSkylights (world.cpp:803-923) and
// the RenderParams sky fields (common.h:105-112).
struct Sky {
    const float4* tex;            // w * h texels, row by row
    const uint32_t* blueNoise;    // blue-noise tables, 327,680 words (world.cpp:180-189)
    uint32_t w, h;
    float lightScale;             // skyLightScale
    float4 light[6];              // skyLight: integrated sky per axis normal
};

// Frame constants (kernel parameter, by value; mirrors RenderParams, common.h:100-118)
struct Frame {
    float3 E, p0, dx, dy;        // dx = p1 - p0, dy = p2 - p0 (the kernel's own subtractions)
    float oorx, oory;
    float4 Nl, Nr, Nt, Nb;
    uint32_t R0, framecount, restirtemporalframe;
    uint32_t frame;              // frame counter (the path tracer's stratum, kernels.cl:219-220)
    int32_t spatial, temporal, accumulate;
    uint32_t nlights, ncand;     // ncand = min(numberOfLights, numberOfCandidates) (ris.cl:48)
    uint32_t maxTemporal, radius, taps;
    int32_t W, H;
    const Sky* sky;               // null: skyDomeSampling 0
};

// ---- small float3 helpers (each op one IEEE rounding) ---------------------------------
__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 add(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 sub(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 mul(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 mulv(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float comp(float3 v, uint32_t i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
// normalize = v * (1 / sqrt(dot(v, v))): the reference's own definition (precomp.h:283,656)
__device__ __forceinline__ float3 normalize3(float3 v) {
    const float inv = 1.0f / sqrtf(dot3(v, v));
    return mul(v, inv);
}

// float -> uint, round toward zero, saturating, NaN -> 0 (convert_uint semantics on GPU)
__device__ __forceinline__ uint32_t f2u(float f) { return __float2uint_rz(f); }
__device__ __forceinline__ int32_t f2i(float f) { return __float2int_rz(f); }

// ---- RNG (tools.cl:17-19) ------------------------------------------------------------
__device__ __forceinline__ uint32_t wang_hash(uint32_t s) {
    s = (s ^ 61u) ^ (s >> 16);
    s *= 9u;
    s = s ^ (s >> 4);
    s *= 0x27d4eb2du;
    s = s ^ (s >> 15);
    return s;
}
__device__ __forceinline__ uint32_t xs32(uint32_t& s) {
    s ^= s << 13;
    s ^= s >> 17;
    s ^= s << 5;
    return s;
}
__device__ __forceinline__ float rnd(uint32_t& s) { return __uint2float_rn(xs32(s)) * 2.3283064365387e-10f; }

// ---- voxel payload (tools.cl:294-322, common.h:203-211) --------------------------------
__device__ __forceinline__ float3 to_rgb(uint32_t v) {
    return f3((float)((v >> 8) & 15u) * (1.0f / 15.0f), (float)((v >> 4) & 15u) * (1.0f / 15.0f),
              (float)(v & 15u) * (1.0f / 15.0f));
}
__device__ __forceinline__ float alphaf(uint32_t v) { return (float)((v & 0xf000u) >> 12) / 15.0f; }
__device__ __forceinline__ float strength(uint32_t v) { return (float)((v & 0xff0000u) >> 16); }
__device__ __forceinline__ bool emitter(uint32_t v) { return ((v >> 16) & 255u) > 0; }
__device__ __forceinline__ uint32_t from_rgba(float3 c, float a, uint32_t m) {
    return (m << 16) + (f2u(a * 15.0f) << 12) + (f2u(c.x * 15.0f) << 8) + (f2u(c.y * 15.0f) << 4) + f2u(c.z * 15.0f);
}
// VoxelNormal (tools.cl:416-421): axis `side`, facing against the ray
__device__ __forceinline__ float side_sign(uint32_t side, float3 D) { return comp(D, side) > 0.0f ? -1.0f : 1.0f; }
__device__ __forceinline__ float3 side_normal(uint32_t side, float s) {
    return f3(side == 0 ? s : 0.0f, side == 1 ? s : 0.0f, side == 2 ? s : 0.0f);
}

// ---- camera ray (tools.cl:102-127, TAA = PANINI = 0) ------------------------------------
__device__ __forceinline__ float3 camera_ray(const Frame& k, int x, int y) {
    const float u = (float)x * k.oorx, v = (float)y * k.oory;
    const float3 P = f3((k.p0.x + k.dx.x * u) + k.dy.x * v, (k.p0.y + k.dx.y * u) + k.dy.y * v,
                        (k.p0.z + k.dx.z * u) + k.dy.z * v);
    return normalize3(sub(P, k.E));
}

// ---- area-light sample (RandomPointOnVoxel, tools.cl:499-577) ---------------------------
// One random point per face of the emitter cube (two draws per face, faces in the order
// +x +y +z -x -y -z, all twelve draws always taken), faces weighted by the solid angle
// they subtend from the shading point, a CDF pick with one more draw, weight = 1/pdf.
// A face contributes only when its outward normal points toward the shading point, and
// along each axis at most one of the two faces does: the point is beyond the +a face or
// beyond the -a face or between them. So the solid angles are computed once per axis for
// that axis' facing face, with the same operations the per-face form uses; faces that do
// not face the point have solid angle +0, and adding +0 to the running total (which is
// never -0) changes nothing.
__device__ __forceinline__ float rnd_of(uint32_t u) { return __uint2float_rn(u) * 2.3283064365387e-10f; }

// point on face `face` at (r0, r1): center + 0.5 size N - 0.5 size T - 0.5 size B + r0 size T
// + r1 size B, with T, B the two following axes (tools.cl:502-515, 540-546)
__device__ __forceinline__ float3 face_point(float4 g, uint32_t face, float r0, float r1) {
    const float size = g.w, h = 0.5f * size;
    const float s = face < 3 ? 1.0f : -1.0f;
    const uint32_t an = face % 3, at = (an + 1) % 3, ab = (an + 2) % 3;
    float c[3] = {g.x, g.y, g.z}, p[3];
    p[an] = c[an] + h * s;
    p[at] = (c[at] - h * s) + (r0 * size) * s;
    p[ab] = (c[ab] - h * s) + (r1 * size) * s;
    return f3(p[0], p[1], p[2]);
}

// lg = (centre, size); spo = offset shading point. Returns the point, *invp = 1/pdf
// (NaN/Inf -> 0), *ncode = face index (Nlight = normals[face]).
__device__ __forceinline__ float3 sample_area_light(float4 g, float3 spo, uint32_t& seed, float* invp, uint32_t* ncode) {
    uint32_t u[12];
#pragma unroll
    for (int i = 0; i < 12; i++) u[i] = xs32(seed);
    const float size = g.w, h = 0.5f * size, area = size * size;
    const float c[3] = {g.x, g.y, g.z}, sp[3] = {spo.x, spo.y, spo.z};
    float sa[6], va[3];
    bool fa[6];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int at = (a + 1) % 3, ab = (a + 2) % 3;
        const bool plus = (sp[a] - (c[a] + h)) > 0.0f;      // s (sp - (c + h s)) > 0, s = +1
        const bool minus = -(sp[a] - (c[a] + (-h))) > 0.0f;  // s = -1
        const float s = plus ? 1.0f : -1.0f;
        const float r0 = rnd_of(plus ? u[2 * a] : u[2 * a + 6]), r1 = rnd_of(plus ? u[2 * a + 1] : u[2 * a + 7]);
        float P[3];
        P[a] = c[a] + h * s;
        P[at] = (c[at] - h * s) + (r0 * size) * s;
        P[ab] = (c[ab] - h * s) + (r1 * size) * s;
        const float3 R = f3(P[0] - spo.x, P[1] - spo.y, P[2] - spo.z);
        const float dd = dot3(R, R);
        const float inv = 1.0f / sqrtf(dd);
        const float nl = -(s * (comp(R, a) * inv));
        const float d = fmaxf(1e-5f, dd);
        const float val = (nl * area) / d;
        sa[a] = plus ? val : 0.0f;
        sa[a + 3] = minus ? val : 0.0f;
        va[a] = val;
        fa[a] = plus;
        fa[a + 3] = minus;
    }
    float total = 0.0f;
#pragma unroll
    for (int f = 0; f < 6; f++) total += sa[f];
    const float r2 = rnd(seed);
    uint32_t index = 0;
    float pdf;
    if (total == 0.0f) {
        pdf = __int_as_float(0x7fffffff);   // 0/0: NaN -> weight 0
    } else if (total > 0.0f && total < __int_as_float(0x7f800000)) {
        // finite total: a face's share is +0 when its solid angle is +0 and its solid
        // angle over the total otherwise; only the facing face of each axis can be
        // non-zero, so the three divisions are taken up front with the same operands
        float q[3];
#pragma unroll
        for (int a = 0; a < 3; a++) q[a] = __float_as_uint(va[a]) == 0u ? 0.0f : va[a] / total;
        pdf = fa[0] ? q[0] : 0.0f;
        float cdf = pdf;
        if (cdf < r2) {
#pragma unroll
            for (int i = 1; i < 6; i++) {
                const float p = fa[i] ? q[i % 3] : 0.0f;
                cdf = cdf + p;
                index = i;
                pdf = p;
                if (cdf >= r2) break;
            }
        }
    } else {
        // +0 / a positive finite total is +0: skip those divisions
        const bool fin = total > 0.0f && total < __int_as_float(0x7f800000);
        pdf = (fin && __float_as_uint(sa[0]) == 0u) ? 0.0f : sa[0] / total;
        float cdf = pdf;
        if (cdf < r2) {
#pragma unroll
            for (int i = 1; i < 6; i++) {
                const float p = (fin && __float_as_uint(sa[i]) == 0u) ? 0.0f : sa[i] / total;
                cdf = cdf + p;
                index = i;
                pdf = p;
                if (cdf >= r2) break;
            }
        }
    }
    float wgt = 1.0f / pdf;
    if (isinf(wgt) || isnan(wgt)) wgt = 0.0f;
    *invp = wgt;
    *ncode = index;
    // the two draws of the chosen face
    uint32_t d0 = u[0], d1 = u[1];
#pragma unroll
    for (int i = 1; i < 6; i++)
        if (index == (uint32_t)i) { d0 = u[2 * i]; d1 = u[2 * i + 1]; }
    return face_point(g, index, rnd_of(d0), rnd_of(d1));
}

// ---- sin/cos for the spatial tap offsets (spatialSampling.cl:24-27) -----------------
// OpenCL leaves cos/sin accuracy to the implementation; the oracle fixes this one:
// Cody-Waite reduction by pi/2 (three-part constant, exact products for |q| <= 4) and
// Taylor polynomials on [-pi/4, pi/4] in Horner form, every op a separate IEEE
// rounding. Within 2 ulp of the correctly rounded values on [0, 2pi].
__device__ __forceinline__ void sincos_vx(float a, float* s, float* c) {
    const float q = rintf(a * 0.636619772367581343f);
    const int qi = (int)q;
    const float r = ((a - q * 1.5703125f) - q * 4.83751296997070312e-4f) - q * 7.54978995489188216e-8f;
    const float r2 = r * r;
    const float ps = r + (r * r2) * (-1.0f / 6.0f + r2 * (1.0f / 120.0f + r2 * (-1.0f / 5040.0f + r2 * (1.0f / 362880.0f))));
    const float pc = 1.0f + r2 * (-0.5f + r2 * (1.0f / 24.0f + r2 * (-1.0f / 720.0f + r2 * (1.0f / 40320.0f + r2 * (-1.0f / 3628800.0f)))));
    switch (qi & 3) {
    case 0: *s = ps; *c = pc; break;
    case 1: *s = pc; *c = -ps; break;
    case 2: *s = -ps; *c = -pc; break;
    default: *s = -pc; *c = ps; break;
    }
}

// ---- brick-grid DDA ------------------------------------------------------------------
// Three nested levels: 32^3 uber cells (32 voxels), 128^3 grid cells (8 voxels), 8^3
// bricks. Same visiting order, step budget and float arithmetic as the reference's
// TraceRay/TraceOpaqueRay/TraceThrough (trace.cl:121-362): `steps` loses 4 per uber
// step and 1 per grid step, bricks are free; multi-axis steps when t ties; `side` is
// the last axis stepped. Levels keep integer coordinates instead of packed bitfields.
// MODE 0: first non-zero voxel. MODE 1: first opaque voxel (alpha 0xF). MODE 2: first
// voxel whose masked value differs from `through` (empty space included).
// dist/side are written only when a voxel is returned (reference behaviour).
// Brick skipping. A brick walk that ends without a hit leaves the walk exactly where
// skipping the brick would: the grid-level crossings saved at the descent are restored
// and the grid step follows, and brick visits cost no budget. So a brick may be skipped
// (treated as an empty grid cell) when none of the voxels the DDA could visit in it is
// opaque. The DDA visits only voxels within a few hundredths of a voxel of the ray's
// line (its crossing times follow the line up to float rounding), so a brick is skipped
// when the line misses the box of its opaque voxels grown by kBrickSlack = 0.1 voxel on
// every side (a slab test; its own rounding is far below the slack). Primary rays
// (trace<0>) skip the same way with the box of the non-zero voxels, and, when their step
// budget cannot run out (kFreeBudget: more than any walk of the map can spend), also
// whole uber cells whose non-zero box they miss: with no budget to account, an uber
// cell without a reachable non-zero voxel is walked over like an empty one.
constexpr float kBrickSlack = 0.1f;
constexpr uint32_t kNoOpaque = 0xFFFFFFFFu;
constexpr int kFreeBudget = 4096;   // > 96 uber visits * 4 + 96 * 10 grid visits

// true when the ray a + v t (r = 1 / v) misses the box `box` (B bits per corner
// coordinate, low x, y, z then high x, y, z) of the cell (cx, cy, cz) of 2^SH voxels,
// grown by the slack
template <int SH, int B>
__device__ __forceinline__ bool box_clear(float ax, float ay, float az, float rx, float ry, float rz, int cx, int cy,
                                          int cz, uint32_t box) {
    if (box == kNoOpaque) return true;
    constexpr uint32_t M = (1u << B) - 1u;
    const float bx = (float)(cx << SH), by = (float)(cy << SH), bz = (float)(cz << SH);
    const float x0 = ((bx + (float)(box & M)) - kBrickSlack - ax) * rx;
    const float x1 = ((bx + (float)((box >> (3 * B)) & M)) + (1.0f + kBrickSlack) - ax) * rx;
    const float y0 = ((by + (float)((box >> B) & M)) - kBrickSlack - ay) * ry;
    const float y1 = ((by + (float)((box >> (4 * B)) & M)) + (1.0f + kBrickSlack) - ay) * ry;
    const float z0 = ((bz + (float)((box >> (2 * B)) & M)) - kBrickSlack - az) * rz;
    const float z1 = ((bz + (float)((box >> (5 * B)) & M)) + (1.0f + kBrickSlack) - az) * rz;
    const float tin = fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fminf(z0, z1));
    const float tout = fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fmaxf(z0, z1));
    return tin > tout;
}

template <int MODE>
__device__ __forceinline__ bool dda_hit(uint32_t v, uint32_t through, uint32_t mask) {
    if (MODE == 0) return v != 0u;
    if (MODE == 1) return ((v & 0xf000u) >> 12) == 15u;
    return (v & mask) != (through & mask);
}

template <int MODE>
__device__ __noinline__ uint32_t trace(const World& w, float ax, float ay, float az, float vx, float vy, float vz,
                                       int steps, uint32_t through, uint32_t mask, float* dist, uint32_t* side) {
    // FixZeroDeltas (trace.cl:37-43)
    if (fabsf(vx) < 1e-8f) vx = vx < 0.0f ? -1e-8f : 1e-8f;
    if (fabsf(vy) < 1e-8f) vy = vy < 0.0f ? -1e-8f : 1e-8f;
    if (fabsf(vz) < 1e-8f) vz = vz < 0.0f ? -1e-8f : 1e-8f;
    const float rx = 1.0f / vx, ry = 1.0f / vy, rz = 1.0f / vz;
    const int sx = vx > 0.0f ? 1 : -1, sy = vy > 0.0f ? 1 : -1, sz = vz > 0.0f ? 1 : -1;
    const int ox = vx > 0.0f ? 1 : 0, oy = vy > 0.0f ? 1 : 0, oz = vz > 0.0f ? 1 : 0;
    float to = 0.0f;
    uint32_t last = 0;
    if (ax < 0.0f || ay < 0.0f || az < 0.0f || ax > 1024.0f || ay > 1024.0f || az > 1024.0f) {
        // slab-clip the origin against the map (trace.cl:139-153)
        const float tx1 = -ax * rx, tx2 = (1024.0f - ax) * rx;
        float tmin = fminf(tx1, tx2), tmax = fmaxf(tx1, tx2);
        const float ty1 = -ay * ry, ty2 = (1024.0f - ay) * ry;
        tmin = fmaxf(tmin, fminf(ty1, ty2));
        tmax = fminf(tmax, fmaxf(ty1, ty2));
        const float tz1 = -az * rz, tz2 = (1024.0f - az) * rz;
        tmin = fmaxf(tmin, fminf(tz1, tz2));
        tmax = fminf(tmax, fmaxf(tz1, tz2));
        if (tmax < tmin || tmax <= 0.0f) return 0u;
        ax = ax + tmin * vx;
        ay = ay + tmin * vy;
        az = az + tmin * vz;
        to = tmin;
        const float hi = 1024.0f - 1.01f;
        if (ay < 0.01f || ay > hi) last = 1;
        if (az < 0.01f || az > hi) last = 2;
    }
    int ux = (int)min(f2u(ax) >> 5, 31u), uy = (int)min(f2u(ay) >> 5, 31u), uz = (int)min(f2u(az) >> 5, 31u);
    float tmx = ((float)(uint32_t)(ux + ox) - ax * 0.03125f) * rx;
    float tmy = ((float)(uint32_t)(uy + oy) - ay * 0.03125f) * ry;
    float tmz = ((float)(uint32_t)(uz + oz) - az * 0.03125f) * rz;
    const float tdx = (float)sx * rx, tdy = (float)sy * ry, tdz = (float)sz * rz;
    float t = 0.0f;
    uint32_t o = __ldg(w.uber + ux + uz * 32 + uy * 1024);
    const bool nobudget = w.ubox0 && steps > kFreeBudget;
    while (true) {
        if ((steps -= 4) <= 0) break;
        if (MODE == 2 ? (o != 0u || through != 0u)
                      : (o != 0u && !(MODE == 0 && nobudget && box_clear<5, 5>(ax, ay, az, rx, ry, rz, ux, uy, uz,
                                                                               __ldg(w.ubox0 + ux + uz * 32 + uy * 1024))))) {
            const float ux_m = tmx, uy_m = tmy, uz_m = tmz;
            t *= 4.0f;
            const uint32_t qx = f2u(0.125f * ax + vx * t), qy = f2u(0.125f * ay + vy * t), qz = f2u(0.125f * az + vz * t);
            int gx = (int)min(max(qx, (uint32_t)ux * 4u), (uint32_t)ux * 4u + 3u);
            int gy = (int)min(max(qy, (uint32_t)uy * 4u), (uint32_t)uy * 4u + 3u);
            int gz = (int)min(max(qz, (uint32_t)uz * 4u), (uint32_t)uz * 4u + 3u);
            tmx = ((float)(uint32_t)(gx + ox) - ax * 0.125f) * rx;
            tmy = ((float)(uint32_t)(gy + oy) - ay * 0.125f) * ry;
            tmz = ((float)(uint32_t)(gz + oz) - az * 0.125f) * rz;
            o = __ldg(w.grid + gx + gz * 128 + gy * 16384);
            while (true) {
                if (!--steps) break;
                if ((o & 1u) == 0u) {
                    const uint32_t v = o >> 1;
                    if (dda_hit<MODE>(v, through, mask)) {
                        *dist = t * 8.0f + to;
                        *side = last;
                        return v;
                    }
                } else if (!(MODE == 0 && w.bbox0 &&
                             box_clear<3, 3>(ax, ay, az, rx, ry, rz, gx, gy, gz, __ldg(w.bbox0 + (o >> 1))))) {
                    // (a skipped brick steps on as an empty cell: no hit, crossings unchanged)
                    const float gx_m = tmx, gy_m = tmy, gz_m = tmz;
                    t *= 8.0f;
                    const uint32_t px = f2u(ax + vx * t), py = f2u(ay + vy * t), pz = f2u(az + vz * t);
                    const uint32_t bx0 = (uint32_t)gx * 8u, by0 = (uint32_t)gy * 8u, bz0 = (uint32_t)gz * 8u;
                    const uint32_t cx = min(max(px, bx0), bx0 + 7u), cy = min(max(py, by0), by0 + 7u),
                                   cz = min(max(pz, bz0), bz0 + 7u);
                    tmx = ((float)(cx + (uint32_t)ox) - ax) * rx;
                    tmy = ((float)(cy + (uint32_t)oy) - ay) * ry;
                    tmz = ((float)(cz + (uint32_t)oz) - az) * rz;
                    int lx = (int)(cx & 7u), ly = (int)(cy & 7u), lz = (int)(cz & 7u);
                    const uint32_t* br = w.bricks + (size_t)(o >> 1) * 512u;
#pragma unroll 1
                    for (int i = 0; i < 24; i++) {
                        const uint32_t v = __ldg(br + lx + ly * 8 + lz * 64);
                        if (dda_hit<MODE>(v, through, mask)) {
                            *dist = t + to;
                            *side = last;
                            return v;
                        }
                        t = fminf(tmx, fminf(tmy, tmz));
                        last = 0;
                        if (t == tmx) { tmx += tdx; lx += sx; }
                        if (t == tmy) { tmy += tdy; ly += sy; last = 1; }
                        if (t == tmz) { tmz += tdz; lz += sz; last = 2; }
                        if ((lx | ly | lz) & ~7) break;
                    }
                    tmx = gx_m; tmy = gy_m; tmz = gz_m;
                }
                t = fminf(tmx, fminf(tmy, tmz));
                last = 0;
                if (t == tmx) { tmx += tdx; gx += sx; }
                if (t == tmy) { tmy += tdy; gy += sy; last = 1; }
                if (t == tmz) { tmz += tdz; gz += sz; last = 2; }
                if (((gx >> 2) != ux) | ((gy >> 2) != uy) | ((gz >> 2) != uz)) break;
                o = __ldg(w.grid + gx + gz * 128 + gy * 16384);
            }
            tmx = ux_m; tmy = uy_m; tmz = uz_m;
        }
        t = fminf(tmx, fminf(tmy, tmz));
        last = 0;
        if (t == tmx) { tmx += tdx; ux += sx; }
        if (t == tmy) { tmy += tdy; uy += sy; last = 1; }
        if (t == tmz) { tmz += tdz; uz += sz; last = 2; }
        if ((ux | uy | uz) & ~31) break;
        o = __ldg(w.uber + ux + uz * 32 + uy * 1024);
    }
    return 0u;
}

// ---- resumable DDA for shadow rays ----------------------------------------------------
// The same traversal as trace<1> (first opaque voxel), restated as a state machine that
// visits one cell per step() call, so a persistent kernel can hand a lane a new ray as
// soon as its current one ends instead of idling until the warp's longest ray is done.
// Every float op, the step budget accounting and the exit cascade (brick -> grid step
// -> uber step) follow trace<MODE> exactly; the oracle checks the two for equality.
//
// The three levels share one code for each action (visit, descent, DDA step, ascent,
// cell load): the current cell (cx, cy, cz) is in uber, grid or voxel units by level,
// and a lane is inside its parent cell while cell >> sh equals the parent (sh = 5 with
// parent 0 at the uber level: inside the map). Lanes of a warp at different levels then
// issue one instruction stream instead of one per level.
struct Walker {
    float ax, ay, az, vx, vy, vz, rx, ry, rz, to;
    float t, tmx, tmy, tmz;        // crossings of the current level
    float umx, umy, umz;           // saved uber-level crossings
    float gmx, gmy, gmz;           // saved grid-level crossings
    int cx, cy, cz;                // current cell
    int px, py, pz;                // parent of the current cell (0 at the uber level)
    int ux, uy, uz, gx, gy, gz;    // uber cell / grid cell being walked below
    int sh;                        // 5 (uber), 2 (grid), 3 (brick)
    int steps, level, cnt;         // cnt: brick steps left (a brick walk ends after 24)
    uint32_t o, brick, last;       // o: value of the current cell (uber byte, grid cell, voxel)
    int stx, sty, stz;             // axis steps (+-1)
    float dist;                    // result
    uint32_t side, voxel;
    uint32_t tlo, thi;             // grid cells (x | y << 10 | z << 20) of the cube a shadow ray must reach
    int guard;                     // the early-out is tested while steps < guard (0: no target)
    int cslot;                     // brick-cache slot of the current brick, or -1 (walk_step<1>)
    __device__ __forceinline__ int ox() const { return stx > 0 ? 1 : 0; }
    __device__ __forceinline__ int oy() const { return sty > 0 ? 1 : 0; }
    __device__ __forceinline__ int oz() const { return stz > 0 ? 1 : 0; }
};
enum : int { WALK_CONTINUE = 0, WALK_HIT = 1, WALK_MISS = 2 };
constexpr int kWalkNoCap = 1 << 30;   // cnt above the brick level: never runs out
constexpr uint32_t kNoTarget = 0xFFFFFFFFu;

constexpr uint32_t kNoKey = 0xFFFFFFFFu;

// value of the current cell at the current level; CACHE: a voxel of a cached brick is
// read from its opacity mask as 0xF000 (opaque) or 0 - all a shadow ray's walk reads of it
// (the hit test; the voxel value of a shadow hit is never used)
template <int CACHE = 0>
__device__ __forceinline__ void walk_load(Walker& k, const World& w) {
    if (k.level == 0) {
        k.o = __ldg(w.uber + k.cx + k.cz * 32 + k.cy * 1024);
    } else if (k.level == 1) {
        k.o = __ldg(w.grid + k.cx + k.cz * 128 + k.cy * 16384);
    } else {
        const uint32_t vi = (uint32_t)((k.cx & 7) | ((k.cy & 7) << 3) | ((k.cz & 7) << 6));
        if (CACHE && k.cslot >= 0)
            k.o = ((w.bcMask[k.cslot * 16 + (vi >> 5)] >> (vi & 31u)) & 1u) ? 0xF000u : 0u;
        else
            k.o = __ldg(w.bricks + (size_t)k.brick * 512u + vi);
    }
}

// slot of `brick` in the brick cache, or -1 (at most 4 probes)
__device__ __forceinline__ int brick_cache_slot(const World& w, uint32_t brick) {
    const uint32_t n = 1u << w.bcLog2;
    uint32_t h = (brick * 2654435761u) >> (32 - w.bcLog2);
#pragma unroll
    for (int p = 0; p < 4; p++) {
        const uint32_t key = w.bcKeys[(h + p) & (n - 1u)];
        if ((key >> 11) == brick && key != kNoKey) return (int)(key & 2047u);
        if (key == kNoKey) return -1;
    }
    return -1;
}

// TraceOpaqueRay prologue (trace.cl:219-243); returns WALK_MISS when the ray misses the map
__device__ __forceinline__ int walk_init(Walker& k, const World& w, float ax, float ay, float az, float vx, float vy,
                                         float vz, int steps) {
    if (fabsf(vx) < 1e-8f) vx = vx < 0.0f ? -1e-8f : 1e-8f;
    if (fabsf(vy) < 1e-8f) vy = vy < 0.0f ? -1e-8f : 1e-8f;
    if (fabsf(vz) < 1e-8f) vz = vz < 0.0f ? -1e-8f : 1e-8f;
    k.vx = vx; k.vy = vy; k.vz = vz;
    k.rx = 1.0f / vx; k.ry = 1.0f / vy; k.rz = 1.0f / vz;
    k.stx = vx > 0.0f ? 1 : -1;
    k.sty = vy > 0.0f ? 1 : -1;
    k.stz = vz > 0.0f ? 1 : -1;
    k.to = 0.0f;
    k.last = 0;
    if (ax < 0.0f || ay < 0.0f || az < 0.0f || ax > 1024.0f || ay > 1024.0f || az > 1024.0f) {
        const float tx1 = -ax * k.rx, tx2 = (1024.0f - ax) * k.rx;
        float tmin = fminf(tx1, tx2), tmax = fmaxf(tx1, tx2);
        const float ty1 = -ay * k.ry, ty2 = (1024.0f - ay) * k.ry;
        tmin = fmaxf(tmin, fminf(ty1, ty2));
        tmax = fminf(tmax, fmaxf(ty1, ty2));
        const float tz1 = -az * k.rz, tz2 = (1024.0f - az) * k.rz;
        tmin = fmaxf(tmin, fminf(tz1, tz2));
        tmax = fminf(tmax, fmaxf(tz1, tz2));
        if (tmax < tmin || tmax <= 0.0f) return WALK_MISS;
        ax = ax + tmin * vx;
        ay = ay + tmin * vy;
        az = az + tmin * vz;
        k.to = tmin;
        const float hi = 1024.0f - 1.01f;
        if (ay < 0.01f || ay > hi) k.last = 1;
        if (az < 0.01f || az > hi) k.last = 2;
    }
    k.ax = ax; k.ay = ay; k.az = az;
    k.cx = (int)min(f2u(ax) >> 5, 31u);
    k.cy = (int)min(f2u(ay) >> 5, 31u);
    k.cz = (int)min(f2u(az) >> 5, 31u);
    k.tmx = ((float)(uint32_t)(k.cx + k.ox()) - ax * 0.03125f) * k.rx;
    k.tmy = ((float)(uint32_t)(k.cy + k.oy()) - ay * 0.03125f) * k.ry;
    k.tmz = ((float)(uint32_t)(k.cz + k.oz()) - az * 0.03125f) * k.rz;
    k.t = 0.0f;
    k.px = k.py = k.pz = 0;
    k.sh = 5;
    k.steps = steps;
    k.level = 0;
    k.cnt = kWalkNoCap;
    k.tlo = k.thi = kNoTarget;
    k.guard = 0;
    k.cslot = -1;
    walk_load(k, w);
    return WALK_CONTINUE;
}

// Visibility early-out for a shadow ray towards the emitter cube [pos, pos + size)
// (packed x + z * 1024 + y * 1024^2, the Light record). Every uber-cell visit costs 4 of
// the step budget and moves the walk at most 4 grid cells along each axis; every grid-cell
// visit costs 1 and moves it at most 1 (brick walks cost nothing and stay in their grid
// cell; a brick exit is followed by a grid visit). So once the budget left after a visit
// is below the Chebyshev distance, in grid cells, between the current cell and the cube's
// cells, no cell within one grid cell of the cube can be visited before the budget runs
// out: the walk cannot hit the cube, nor a voxel whose rounded hit point could fall in it,
// and ends as occluded whichever way it ends. The walk then stops as a miss, which the
// visibility test reads as occluded (the origin is outside the cube: its cell is at least
// one grid cell away, or the distance would be 0).
// The ray heads for a point on the cube, so along each axis its grid cell approaches the
// cube's cells until it gets there: the distance never exceeds the one of the starting
// grid cell, and the test can wait until the budget drops below that (`guard`; the test
// itself is exact whatever guard holds).
__device__ __forceinline__ void walk_target(Walker& k, uint32_t pos, uint32_t size) {
    const uint32_t ex = pos % 1024u, ez = (pos / 1024u) % 1024u, ey = pos / (1024u * 1024u);
    const uint32_t s1 = size > 0u ? size - 1u : 0u;
    const int lx = (int)(ex >> 3), ly = (int)(ey >> 3), lz = (int)(ez >> 3);
    const int hx = (int)(min(ex + s1, 1023u) >> 3), hy = (int)(min(ey + s1, 1023u) >> 3), hz = (int)(min(ez + s1, 1023u) >> 3);
    k.tlo = (uint32_t)lx | ((uint32_t)ly << 10) | ((uint32_t)lz << 20);
    k.thi = (uint32_t)hx | ((uint32_t)hy << 10) | ((uint32_t)hz << 20);
    const int gx = (int)min(f2u(k.ax) >> 3, 127u), gy = (int)min(f2u(k.ay) >> 3, 127u), gz = (int)min(f2u(k.az) >> 3, 127u);
    const int dx = max(max(lx - gx, gx - hx), 0), dy = max(max(ly - gy, gy - hy), 0), dz = max(max(lz - gz, gz - hz), 0);
    k.guard = max(dx, max(dy, dz)) + 1;
}

// Chebyshev distance in grid cells between the current cell (level 0: its 4^3 grid cells)
// and the target cube's grid cells
__device__ __forceinline__ int walk_target_distance(const Walker& k) {
    const int s2 = k.level == 0 ? 2 : 0, span = (1 << s2) - 1;
    const int lx = k.cx << s2, ly = k.cy << s2, lz = k.cz << s2;
    const int dx = max(max((int)(k.tlo & 1023u) - (lx + span), lx - (int)(k.thi & 1023u)), 0);
    const int dy = max(max((int)((k.tlo >> 10) & 1023u) - (ly + span), ly - (int)((k.thi >> 10) & 1023u)), 0);
    const int dz = max(max((int)(k.tlo >> 20) - (lz + span), lz - (int)(k.thi >> 20)), 0);
    return max(dx, max(dy, dz));
}

// One cell visit at the current level, then one action: the hit or the budget miss,
// a descent into the cell (uber -> grid, trace.cl:262-273; grid -> brick, GRIDSTEP,
// trace.cl:85-104), or a DDA step (BRICKSTEP / GRIDSTEP tail / uber loop,
// trace.cl:66-80, 105-110, 274-279) that climbs a level each time it leaves the parent
// cell and ends as a miss when it leaves the map. FLAGS (shadow tracer options, 0 for the
// plain walk): kWalkCache - brick walks count into w.bcCount when it is set, and read cached
// bricks' opacity masks from w.bcKeys / w.bcMask when bcLog2 > 0; kWalkEarly - the
// visibility early-out of walk_target.
constexpr int kWalkCache = 1, kWalkEarly = 2;
template <int FLAGS = 0>
__device__ __forceinline__ int walk_step(Walker& k, const World& w) {
    constexpr int CACHE = FLAGS & kWalkCache;
    const int lv = k.level;
    // a grid step with the budget exhausted always ends as a miss (the uber loop
    // re-checks the budget before any further cell is visited)
    k.steps -= lv == 0 ? 4 : (lv == 1 ? 1 : 0);
    if (lv < 2 && k.steps <= 0) return WALK_MISS;
    if ((FLAGS & kWalkEarly) && lv < 2 && k.steps < k.guard && k.steps < walk_target_distance(k)) return WALK_MISS;
    // uber: descend into a non-empty cell; grid: descend into a brick, hit an opaque
    // brick-less cell; brick: hit an opaque voxel
    const uint32_t hv = lv == 1 ? k.o >> 1 : k.o;
    const bool brickcell = lv == 1 && (k.o & 1u);
    bool desc = lv == 0 ? k.o != 0u : brickcell;
    const bool hit = lv != 0 && !brickcell && ((hv & 0xf000u) >> 12) == 15u;
    if (brickcell && w.bbox &&
        box_clear<3, 3>(k.ax, k.ay, k.az, k.rx, k.ry, k.rz, k.cx, k.cy, k.cz, __ldg(w.bbox + (k.o >> 1))))
        desc = false;   // a brick the ray cannot stop in: step on as over an empty cell
    if (hit) {
        k.dist = (lv == 1 ? k.t * 8.0f : k.t) + k.to;
        k.side = k.last;
        k.voxel = hv;
        return WALK_HIT;
    }
    if (desc) {
        // uber -> grid: t in grid units (x4), entry cell from 0.125 * a + v * t;
        // grid -> brick: t in voxel units (x8), entry voxel from a + v * t
        const bool top = lv == 0;
        const float S = top ? 4.0f : 8.0f, K = top ? 0.125f : 1.0f;
        const uint32_t W = top ? 2u : 3u;
        if (top) {
            k.umx = k.tmx; k.umy = k.tmy; k.umz = k.tmz;
            k.ux = k.cx; k.uy = k.cy; k.uz = k.cz;
        } else {
            k.gmx = k.tmx; k.gmy = k.tmy; k.gmz = k.tmz;
            k.gx = k.cx; k.gy = k.cy; k.gz = k.cz;
            k.brick = k.o >> 1;
            if (CACHE) {
                if (w.bcCount) atomicAdd(w.bcCount + k.brick, 1u);
                k.cslot = w.bcLog2 > 0 ? brick_cache_slot(w, k.brick) : -1;
            }
        }
        k.t *= S;
        const uint32_t qx = f2u(K * k.ax + k.vx * k.t), qy = f2u(K * k.ay + k.vy * k.t),
                       qz = f2u(K * k.az + k.vz * k.t);
        const uint32_t lx = (uint32_t)k.cx << W, ly = (uint32_t)k.cy << W, lz = (uint32_t)k.cz << W;
        const uint32_t span = (1u << W) - 1u;
        k.px = k.cx; k.py = k.cy; k.pz = k.cz;
        k.cx = (int)min(max(qx, lx), lx + span);
        k.cy = (int)min(max(qy, ly), ly + span);
        k.cz = (int)min(max(qz, lz), lz + span);
        k.tmx = ((float)(uint32_t)(k.cx + k.ox()) - k.ax * K) * k.rx;
        k.tmy = ((float)(uint32_t)(k.cy + k.oy()) - k.ay * K) * k.ry;
        k.tmz = ((float)(uint32_t)(k.cz + k.oz()) - k.az * K) * k.rz;
        k.sh = (int)W;
        k.cnt = top ? kWalkNoCap : 24;
        k.level = lv + 1;
    } else {
        while (true) {
            k.t = fminf(k.tmx, fminf(k.tmy, k.tmz));
            k.last = 0;
            if (k.t == k.tmx) { k.tmx += fabsf(k.rx); k.cx += k.stx; }
            if (k.t == k.tmy) { k.tmy += fabsf(k.ry); k.cy += k.sty; k.last = 1; }
            if (k.t == k.tmz) { k.tmz += fabsf(k.rz); k.cz += k.stz; k.last = 2; }
            const bool inside = ((k.cx >> k.sh) == k.px) & ((k.cy >> k.sh) == k.py) & ((k.cz >> k.sh) == k.pz);
            if (inside && --k.cnt != 0) break;
            if (k.level == 0) return WALK_MISS;
            if (k.level == 2) {
                k.tmx = k.gmx; k.tmy = k.gmy; k.tmz = k.gmz;
                k.cx = k.gx; k.cy = k.gy; k.cz = k.gz;
                k.px = k.ux; k.py = k.uy; k.pz = k.uz;
                k.sh = 2;
                k.cnt = kWalkNoCap;
            } else {
                k.tmx = k.umx; k.tmy = k.umy; k.tmz = k.umz;
                k.cx = k.ux; k.cy = k.uy; k.cz = k.uz;
                k.px = k.py = k.pz = 0;
                k.sh = 5;
            }
            k.level--;
        }
    }
    walk_load<CACHE>(k, w);
    return WALK_CONTINUE;
}

// ---- reservoirs --------------------------------------------------------------------
// In HBM a reservoir is 32 bytes in two SoA planes:
//   a = (lightIndex, M | nlight << 29, bits(sumOfWeights), bits(pHat))
//   b = (positionOnVoxel.xyz, invPositionProbability)
// nlight: 0..5 = Nlight is one of the six face normals (+x,+y,+z,-x,-y,-z, the order of
// tools.cl:502-510); 6 = zero vector. W is not stored: every producer ends with
// AdjustWeight(res, res.pHat) or zeroes both W and sumOfWeights, so
// W = sumOfWeights / max(1e-5, pHat * M) reproduces the stored value exactly.
struct Res {
    float sumW;
    uint32_t M;
    uint32_t idx;
    float pHat;
    float3 pos;
    float inv;
    uint32_t ncode;
};
__device__ __forceinline__ float res_W(const Res& r) { return r.sumW / fmaxf(1e-5f, r.pHat * (float)r.M); }
__device__ __forceinline__ Res res_load(const uint4* __restrict__ a, const float4* __restrict__ b, size_t i) {
    const uint4 qa = __ldg(a + i);
    const float4 qb = __ldg(b + i);
    Res r;
    r.idx = qa.x;
    r.M = qa.y & 0x1FFFFFFFu;
    r.ncode = qa.y >> 29;
    r.sumW = __uint_as_float(qa.z);
    r.pHat = __uint_as_float(qa.w);
    r.pos = f3(qb.x, qb.y, qb.z);
    r.inv = qb.w;
    return r;
}
__device__ __forceinline__ void res_store(uint4* a, float4* b, size_t i, const Res& r) {
    a[i] = make_uint4(r.idx, (r.M & 0x1FFFFFFFu) | (r.ncode << 29), __float_as_uint(r.sumW), __float_as_uint(r.pHat));
    b[i] = make_float4(r.pos.x, r.pos.y, r.pos.z, r.inv);
}
__device__ __forceinline__ Res res_zero() {
    Res r;
    r.sumW = 0.0f; r.M = 0; r.idx = 0; r.pHat = 0.0f; r.pos = f3(0.0f, 0.0f, 0.0f); r.inv = 0.0f; r.ncode = 6;
    return r;
}

// UpdateReservoir (reservoir.cl:3-15)
__device__ __forceinline__ void res_update(Res& r, float weight, float pHat, uint32_t idx, float r0, float3 pos,
                                           float inv, uint32_t ncode) {
    r.M += 1u;
    r.sumW = r.sumW + weight;
    if (r0 < weight / fmaxf(1e-5f, r.sumW)) {
        r.idx = idx;
        r.pos = pos;
        r.inv = inv;
        r.ncode = ncode;
        r.pHat = pHat;
    }
}
// ReWeighSumOfWeights (reservoir.cl:22-28) applied to a stored reservoir with weight W
__device__ __forceinline__ void res_reweigh(Res& r, float W, float newPHat, uint32_t M) {
    r.sumW = (W * (float)M) * newPHat;
    r.M = M;
    r.pHat = newPHat;
}
// CombineReservoir (reservoir.cl:30-38)
__device__ __forceinline__ void res_combine(Res& r, const Res& o, float r0) {
    const uint32_t m1 = r.M, m2 = o.M;
    res_update(r, o.sumW, o.pHat, o.idx, r0, o.pos, o.inv, o.ncode);
    r.M = m1 + m2;
}

}  // namespace dev
}  // namespace vxr
