// kernels.cu - the per-frame stage kernels of Voxel ReSTIR on sm_103a, plus the
// one-time world kernels (uber grid, light table).
//
// Memory layout in HBM (per view):
//   G-buffer   vd[2]  uint2  (voxel | side << 24, bits(dist))   current / previous frame
//              seed   uint32 per-pixel xorshift32 state
//   reservoirs C, H   uint4 + float4 planes (see Res in device.cuh), 32 B/pixel each:
//              C = candidate+temporal output, H = spatial output = temporal history
//   frame      float4 (rgb, dist); accum float4 (running mean, the output image)
// and per batch of views (a single view holds two sets and takes the other one as each
// frame begins, so its candidate passes can run beside the previous frame's shading):
//   hits       uint32 list of (view << 27 | pixel) whose primary ray hit a voxel
//   queue      float4 x 2 per entry: shadow-ray requests (origin | entry, dir | light)
//   counters   uint32[kCounters]: list lengths and work-queue cursors (kernels.hpp)
// The reference cycles two 80-byte reservoir buffers through three roles per frame
// (world.cpp:2209-2219) and copies the shaded reservoir at the end of shading
// (ris.cl:412). Here the spatial pass writes H in place of the previous history,
// which the candidate pass has finished reading, and shading patches H on a failed
// visibility test; H is then next frame's history without any copy.
//
// Work decomposition: the reference runs one work item per pixel through each whole
// kernel, so sky pixels idle beside terrain pixels and every warp waits for its
// longest shadow ray. Here every stage is one launch over a table of views (one view,
// or a batch of up to 16 independent views with their own worlds, resolutions and
// light models): pixel stages are persistent blocks pulling screen tiles from a work queue;
// the candidate loop, the temporal step and the shading request run over a compacted
// list of hit pixels; and every shadow ray goes through one persistent tracer whose
// lanes take a new ray as soon as theirs ends. Each pixel's arithmetic is unchanged,
// so results are the same bit for bit whatever order pixels and rays are processed in.
#include <algorithm>
#include <cstdint>
#include <map>
#include <mutex>
#include <cuda_runtime.h>

#include "device.cuh"
#include "kernels.hpp"
#include "proposal.hpp"

namespace vxr {
namespace dev {

__device__ __forceinline__ void raise_error(uint32_t* err, uint32_t code) { atomicOr(err, code); }

// Light centre/emission from the reference records (tools.cl:600-607, phat.cl:8-12).
__global__ void build_light_table_kernel(const uint4* __restrict__ raw, uint32_t n, float4* geom, float4* emit) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint4 l = raw[i];  // (position, voxel, size, 0)
    const uint32_t y = l.x / (1024u * 1024u), z = (l.x / 1024u) % 1024u, x = l.x % 1024u;
    const float size = (float)l.z;
    const float half = 0.5f * size;
    geom[i] = make_float4((float)x + half, (float)y + half, (float)z + half, size);
    const float3 c = to_rgb(l.y);
    const float m = strength(l.y);
    const float INVPI = 0.31830988618379067153777f;
    emit[i] = make_float4((c.x * m) * INVPI, (c.y * m) * INVPI, (c.z * m) * INVPI, __uint_as_float(l.x));
}

// updateUberGrid (kernels.cl:498-513): 1 when any of the 4^3 grid cells is non-empty.
__global__ void build_uber_kernel(const uint32_t* __restrict__ grid, uint8_t* uber) {
    const int task = blockIdx.x * blockDim.x + threadIdx.x;
    if (task >= 32 * 32 * 32) return;
    const int x = task & 31, z = (task >> 5) & 31, y = task >> 10;
    bool empty = true;
    for (int a = 0; a < 4 && empty; a++)
        for (int b = 0; b < 4 && empty; b++)
            for (int c = 0; c < 4; c++) {
                const int gx = x * 4 + a, gy = y * 4 + b, gz = z * 4 + c;
                if (grid[gx + gz * 128 + gy * 16384]) { empty = false; break; }
            }
    uber[x + z * 32 + y * 1024] = empty ? 0 : 1;
}

// Per brick the boxes of its opaque voxels (type nibble 15) and of its non-zero voxels,
// packed as World::bbox describes: one warp per brick, 16 voxels a lane, min / max
// reductions over the warp.
__device__ __forceinline__ uint32_t warp_box(bool any, const uint32_t lo[3], const uint32_t hi[3]) {
    const bool anyw = __any_sync(0xffffffffu, any);
    uint32_t box = 0u;
    for (int a = 0; a < 3; a++) {
        box |= __reduce_min_sync(0xffffffffu, lo[a]) << (3 * a);
        box |= __reduce_max_sync(0xffffffffu, hi[a]) << (9 + 3 * a);
    }
    return anyw ? box : kNoOpaque;
}
// (list: the bricks to do, or null for bricks 0 .. n - 1)
__global__ void build_brick_boxes_kernel(const uint32_t* __restrict__ bricks, const uint32_t* __restrict__ list,
                                         uint32_t n, uint32_t* __restrict__ bbox, uint32_t* __restrict__ bbox0) {
    const size_t item = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (item >= n) return;   // whole warps leave together (blockDim a multiple of 32)
    const size_t brick = list ? (size_t)__ldg(list + item) : item;
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t lo[3] = {7u, 7u, 7u}, hi[3] = {0u, 0u, 0u}, lo0[3] = {7u, 7u, 7u}, hi0[3] = {0u, 0u, 0u};
    bool any = false, any0 = false;
    for (uint32_t i = 0; i < 16; i++) {
        const uint32_t e = i * 32u + lane;   // coalesced: a warp reads 32 consecutive voxels
        const uint32_t v = __ldg(bricks + brick * 512u + e);
        const uint32_t c[3] = {e & 7u, (e >> 3) & 7u, e >> 6};
        if (((v & 0xf000u) >> 12) == 15u) {
            for (int a = 0; a < 3; a++) { lo[a] = min(lo[a], c[a]); hi[a] = max(hi[a], c[a]); }
            any = true;
        }
        if (v != 0u) {
            for (int a = 0; a < 3; a++) { lo0[a] = min(lo0[a], c[a]); hi0[a] = max(hi0[a], c[a]); }
            any0 = true;
        }
    }
    const uint32_t box = warp_box(any, lo, hi), box0 = warp_box(any0, lo0, hi0);
    if (lane == 0u) {
        bbox[brick] = box;
        bbox0[brick] = box0;
    }
}

// commit (kernels.cl:448-477): staged brick i (512 voxels after the index list) to its
// place in the pool; one block of 128 threads per brick, 16 bytes a thread
__global__ void commit_bricks_kernel(const uint32_t* __restrict__ list, const uint32_t* __restrict__ voxels,
                                     uint32_t* __restrict__ bricks) {
    const uint32_t b = __ldg(list + blockIdx.x);
    const uint4 v = __ldg(reinterpret_cast<const uint4*>(voxels + (size_t)blockIdx.x * 512u) + threadIdx.x);
    reinterpret_cast<uint4*>(bricks + (size_t)b * 512u)[threadIdx.x] = v;
}

// Per uber cell the box of its non-zero voxels (World::ubox0): brick-less non-zero grid
// cells count whole, bricks with their non-zero box (bbox0, built before).
__global__ void build_uber_boxes_kernel(const uint32_t* __restrict__ grid, const uint32_t* __restrict__ bbox0,
                                        uint32_t* __restrict__ ubox0) {
    const int task = blockIdx.x * blockDim.x + threadIdx.x;
    if (task >= 32 * 32 * 32) return;
    const int x = task & 31, z = (task >> 5) & 31, y = task >> 10;
    uint32_t lo[3] = {31u, 31u, 31u}, hi[3] = {0u, 0u, 0u};
    bool any = false;
    for (int b = 0; b < 64; b++) {
        const uint32_t cx = b & 3, cz = (b >> 2) & 3, cy = b >> 4;
        const uint32_t c = __ldg(grid + (x * 4 + cx) + (z * 4 + cz) * 128 + (y * 4 + cy) * 16384);
        if (c == 0u) continue;
        uint32_t l[3] = {0u, 0u, 0u}, h[3] = {7u, 7u, 7u};
        if (c & 1u) {
            const uint32_t bb = __ldg(bbox0 + (c >> 1));
            if (bb == kNoOpaque) continue;
            for (int a = 0; a < 3; a++) { l[a] = (bb >> (3 * a)) & 7u; h[a] = (bb >> (9 + 3 * a)) & 7u; }
        }
        const uint32_t base[3] = {cx * 8u, cy * 8u, cz * 8u};
        for (int a = 0; a < 3; a++) { lo[a] = min(lo[a], base[a] + l[a]); hi[a] = max(hi[a], base[a] + h[a]); }
        any = true;
    }
    uint32_t box = 0u;
    for (int a = 0; a < 3; a++) box |= (lo[a] << (5 * a)) | (hi[a] << (15 + 5 * a));
    ubox0[task] = any ? box : kNoOpaque;
}


// ---- work distribution --------------------------------------------------------------------
// VARIANT of a launch: 0 one view with area lights, 1 one view with point lights (the
// view is read from the kernel parameter), 2 a table of views in device memory, light
// model per view.
constexpr uint32_t kPixMask = (1u << 27) - 1u;

template <int VARIANT>
__device__ __forceinline__ const ViewDev* view_of(const BatchDev& bd, uint32_t v) {
    if (VARIANT < 2) return &bd.one;
    return bd.views + v;
}
// pixel of a hit-list or request entry (a single view's entries are the bare pixel index,
// so a single view may hold more than 2^27 pixels)
template <int VARIANT>
__device__ __forceinline__ uint32_t pix_of(uint32_t e) {
    return VARIANT < 2 ? e : (e & kPixMask);
}
template <int VARIANT>
__device__ __forceinline__ bool point_of(const ViewDev* V) {
    return VARIANT == 1 || (VARIANT == 2 && V->point);
}

// warp-aggregated append to a list: one atomic per group of lanes that call it together
__device__ __forceinline__ uint32_t append_slot(uint32_t* counter) {
    const unsigned m = __activemask();
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(m));
    base = __shfl_sync(m, base, leader);
    return base + (uint32_t)__popc(m & ((1u << lane) - 1u));
}

// Block-aggregated append: one atomic per block and call instead of one per warp, so a
// list filled by a short kernel is not serialised on its counter. Every thread of the
// block calls it (flag = this thread appends); returns this thread's slot when flag.
__device__ __forceinline__ uint32_t block_append(uint32_t* counter, bool flag) {
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_base;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (int)((blockDim.x + 31) >> 5);
    const unsigned m = __ballot_sync(0xffffffffu, flag);
    if (lane == 0) s_warp[warp] = (uint32_t)__popc(m);
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t tot = 0;
        for (int w = 0; w < nw; w++) {
            const uint32_t c = s_warp[w];
            s_warp[w] = tot;
            tot += c;
        }
        s_base = tot ? atomicAdd(counter, tot) : 0u;
    }
    __syncthreads();
    const uint32_t slot = s_base + s_warp[warp] + (uint32_t)__popc(m & ((1u << lane) - 1u));
    __syncthreads();   // the shared words are reused by the next call
    return slot;
}

// Next tile of the batch for this block: with bd.persistent, resident blocks pull tiles
// from the queue cursor `ctr` until it is drained; otherwise the launch has one block per
// tile and the hardware block scheduler balances them. `round` counts calls (starts at 0).
__device__ __forceinline__ bool next_tile(const BatchDev& bd, uint32_t* ctr, uint32_t* tile, uint32_t& round) {
    if (!bd.persistent) {
        *tile = blockIdx.x;
        return round++ == 0;
    }
    __shared__ uint32_t s_tile;
    __syncthreads();
    if (threadIdx.x == 0) s_tile = atomicAdd(ctr, 1u);
    __syncthreads();
    *tile = s_tile;
    return s_tile < bd.totalTiles;
}

// view of a batch tile and the pixel of this thread in it
template <int VARIANT>
__device__ __forceinline__ const ViewDev* tile_pixel(const BatchDev& bd, uint32_t tile, int* x, int* y) {
    uint32_t v = 0;
    if (VARIANT == 2)
        while (v + 1 < bd.nviews && bd.views[v + 1].tileBase <= tile) v++;
    const ViewDev* V = view_of<VARIANT>(bd, v);
    const uint32_t lt = tile - V->tileBase;
    const uint32_t tx = lt % V->tilesX, ty = lt / V->tilesX;
    *x = (int)(tx * (uint32_t)bd.tx + threadIdx.x % (uint32_t)bd.tx);
    *y = (int)(ty * (uint32_t)bd.ty + threadIdx.x / (uint32_t)bd.tx);
    return V;
}

// ---- stage 1: primary rays / G-buffer (renderAlbedo, ris.cl:295-389) --------------------
__device__ __forceinline__ void albedo_px(const World& w, const Frame& k, uint2* __restrict__ vd, uint32_t* __restrict__ seeds,
                                          int x, int y) {
    const uint32_t seed = wang_hash((uint32_t)x * 171u + (uint32_t)y * 1773u + k.R0);
    const float3 D = camera_ray(k, x, y);
    uint32_t side = 0;
    float dist = 0.0f;
    uint32_t voxel = trace<0>(w, k.E.x, k.E.y, k.E.z, D.x, D.y, D.z, 999999, 0u, 0u, &dist, &side);
    float alpha = alphaf(voxel);
    float3 outc = mul(to_rgb(voxel), alpha);
    float total = 0.0f;
    // translucency: continue through non-opaque voxels (ris.cl:321-377)
    float remvis = 1.0f - alphaf(voxel);
    int iteration = 0;
    uint32_t prevSide = 0, prevHit = 0;
    while (prevHit != voxel && remvis > 0.0f) {
        prevHit = voxel;
        prevSide = side;
        total += dist + 0.01f;
        const float3 o = f3(k.E.x + total * D.x, k.E.y + total * D.y, k.E.z + total * D.z);
        voxel = trace<2>(w, o.x, o.y, o.z, D.x, D.y, D.z, 999999, voxel, 0x00FFFFu, &dist, &side);
        const float3 c = to_rgb(voxel);
        alpha = alphaf(voxel);
        outc = add(outc, mul(mul(c, remvis), alpha));
        remvis = remvis * (1.0f - alpha);
        if (++iteration == 25) remvis = 0.0f;
        if (dist <= 0.001f) break;
    }
    if (voxel != 0u) total += dist;
    else side = prevSide;
    const uint32_t enc = from_rgba(outc, 1.0f - remvis, (uint32_t)strength(voxel));
    const size_t i = (size_t)y * k.W + x;
    vd[i] = make_uint2(enc | (side << 24), __float_as_uint(total));
    seeds[i] = seed;
}

template <int VARIANT>
__global__ void __launch_bounds__(kMaxTileThreads) albedo_kernel(const __grid_constant__ BatchDev bd) {
    uint32_t tile, round = 0;
    while (next_tile(bd, bd.counters + kCtrAlbedo, &tile, round)) {
        int x, y;
        const ViewDev* V = tile_pixel<VARIANT>(bd, tile, &x, &y);
        const Frame& k = V->k;
        if (x < k.W && y < k.H) {
            const World w = V->w;
            albedo_px(w, k, V->b.vd[V->cur], V->b.seed, x, y);
        }
    }
}

// ---- ground truth: renderPathTracer / render_di_gfxexp (kernels.cl:177-260, GFXEXP 1) ----
// One-bounce estimate of the direct light: the primary hit's own emission plus the
// emission met along one uniform hemisphere direction (stratified on a 16 x 16 grid by the
// frame counter), weighted by 2 pi N.L and the BRDF, into the frame buffer as (rgb,
// distance); no hit: (0, 0, 0, 1e20). Sky sampling is off (no sky texture). cos and sin
// are the correctly rounded FP64 results rounded to FP32, the oracle's choice for the
// implementation-defined OpenCL builtins.
__device__ __forceinline__ float3 uniform_sample_hemisphere(float r1, float r2, float3 N) {   // tools.cl:31-51
    float3 Nt;
    if (fabsf(N.x) > fabsf(N.y)) {
        const float l = sqrtf(N.x * N.x + N.z * N.z);
        Nt = f3(N.z / l, 0.0f / l, -N.x / l);
    } else {
        const float l = sqrtf(N.y * N.y + N.z * N.z);
        Nt = f3(0.0f / l, -N.z / l, N.y / l);
    }
    const float3 Nb = f3(N.y * Nt.z - N.z * Nt.y, N.z * Nt.x - N.x * Nt.z, N.x * Nt.y - N.y * Nt.x);
    const float sinTheta = sqrtf(1.0f - r1 * r1);
    const float phi = 6.28318530717958647692528f * r2;
    double sd, cd;
    sincos((double)phi, &sd, &cd);            // one argument reduction for both
    const float x = sinTheta * (float)cd;
    const float z = sinTheta * (float)sd;
    return f3((x * Nb.x + r1 * N.x) + z * Nt.x, (x * Nb.y + r1 * N.y) + z * Nt.y, (x * Nb.z + r1 * N.z) + z * Nt.z);
}

__device__ __forceinline__ float4 path_trace_px(const World& w, const Frame& k, int x, int y) {
    uint32_t seed = wang_hash((uint32_t)x * 171u + (uint32_t)y * 1773u + k.R0);
    const float3 D = camera_ray(k, x, y);
    float dist = 0.0f;
    uint32_t side = 0;
    const uint32_t voxel = trace<0>(w, k.E.x, k.E.y, k.E.z, D.x, D.y, D.z, 999999, 0u, 0u, &dist, &side);
    if (voxel == 0u) return make_float4(0.0f, 0.0f, 0.0f, 1e20f);
    const float INVPI = 0.31830988618379067153777f;
    const float3 rgb = to_rgb(voxel);
    const float es = (float)((voxel & 0xff0000u) >> 16);
    const float3 contribution = mul(mul(rgb, es), INVPI);
    const float3 brdf = f3(INVPI * rgb.x, INVPI * rgb.y, INVPI * rgb.z);
    const float3 I = f3(k.E.x + D.x * dist, k.E.y + D.y * dist, k.E.z + D.z * dist);
    const int sx = (int)(k.frame & 15u), sy = (int)(k.frame >> 4);
    const float r0 = (float)sx * 0.0625f + rnd(seed) * 0.0625f;
    const float r1 = (float)sy * 0.0625f + rnd(seed) * 0.0625f;
    const float s = side_sign(side, D);
    const float3 N = side_normal(side, s);
    const float3 R = uniform_sample_hemisphere(r0, r1, N);
    const float NdotL = fmaxf(0.0f, (N.x * R.x + N.y * R.y) + N.z * R.z);
    float dist2 = 0.0f;
    uint32_t side2 = 0;
    const uint32_t voxel2 = trace<0>(w, I.x + 0.1f * N.x, I.y + 0.1f * N.y, I.z + 0.1f * N.z, R.x, R.y, R.z, 128, 0u, 0u,
                                     &dist2, &side2);
    const float3 sampleL = mul(mul(to_rgb(voxel2), (float)((voxel2 & 0xff0000u) >> 16)), INVPI);
    const float TWOPI = 6.28318530717958647692528f;
    return make_float4(((sampleL.x * TWOPI) * NdotL) * brdf.x + contribution.x,
                       ((sampleL.y * TWOPI) * NdotL) * brdf.y + contribution.y,
                       ((sampleL.z * TWOPI) * NdotL) * brdf.z + contribution.z, dist);
}

__global__ void __launch_bounds__(kMaxTileThreads) path_trace_kernel(const __grid_constant__ BatchDev bd) {
    uint32_t tile, round = 0;
    while (next_tile(bd, bd.counters + kCtrAlbedo, &tile, round)) {
        int x, y;
        const ViewDev* V = tile_pixel<0>(bd, tile, &x, &y);
        const Frame& k = V->k;
        if (x < k.W && y < k.H) V->b.frame[(size_t)y * k.W + x] = path_trace_px(V->w, k, x, y);
    }
}

// Hit list of the frame over every view (blockIdx.y = view); pixels without a hit get
// the empty reservoir (ris.cl:34,123).
template <int VARIANT>
__global__ void __launch_bounds__(256) compact_hits_kernel(const __grid_constant__ BatchDev bd) {
    const ViewDev* V = view_of<VARIANT>(bd, blockIdx.y);
    const uint32_t n = (uint32_t)V->k.W * (uint32_t)V->k.H;
    const uint2* vd = V->b.vd[V->cur];
    uint4* cA = V->b.cA;
    float4* cB = V->b.cB;
    // every thread of a block runs the same iterations (block_append needs all of them)
    for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < n; i0 += gridDim.x * blockDim.x) {
        const uint32_t i = i0 + threadIdx.x;
        const bool in = i < n;
        const bool hit = in && (vd[i].x & 0x00FFFFFFu) != 0u;
        const uint32_t slot = block_append(bd.counters + kCtrHits, hit);
        if (hit) {
            bd.hits[slot] = (blockIdx.y << 27) | i;
        } else if (in) {
            cA[i] = make_uint4(0u, 6u << 29, 0u, 0u);
            cB[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
    }
}

// ---- target function (phat.cl:2-41) ------------------------------------------------------
// length(brdf * Le/pi * cos(theta) * cos(theta_l) * size^2 / d^2), NaN/Inf -> 0.
// The zero cases are decided from signs before any division: N is an axis normal, so
// dot(N, L) = sN * L[side] and sign(L[a]) = sign(R[a]); a non-positive cosine makes the
// product exactly (+/-)0, whose length is +0.
template <bool POINT>
__device__ __forceinline__ float3 phat_full(float3 pos, uint32_t ncode, float3 sp, uint32_t nside, float nsign,
                                            float3 brdf, float4 em, float size, bool* zero) {
    const float3 R = sub(pos, sp);
    *zero = true;
    if (!(nsign * comp(R, nside) > 0.0f)) return f3(0.0f, 0.0f, 0.0f);
    float lsign = 0.0f;
    uint32_t laxis = 0;
    if (!POINT) {
        if (ncode >= 6) return f3(0.0f, 0.0f, 0.0f);
        laxis = ncode % 3;
        lsign = ncode < 3 ? 1.0f : -1.0f;
        if (!(-(lsign * comp(R, laxis)) > 0.0f)) return f3(0.0f, 0.0f, 0.0f);
    }
    *zero = false;
    const float dd = dot3(R, R);
    const float inv = 1.0f / sqrtf(dd);
    const float3 L = mul(R, inv);
    const float ndotl = fmaxf(nsign * comp(L, nside), 0.0f);
    const float distsq = fmaxf(1e-5f, dd);
    const float area = size * size;
    const float nldotl = POINT ? 1.0f : fmaxf(-(lsign * comp(L, laxis)), 0.0f);
    const float solid = (nldotl * area) / distsq;
    return f3(((brdf.x * em.x) * ndotl) * solid, ((brdf.y * em.y) * ndotl) * solid, ((brdf.z * em.z) * ndotl) * solid);
}
template <bool POINT>
__device__ __forceinline__ float phat(float3 pos, uint32_t ncode, float3 sp, uint32_t nside, float nsign, float3 brdf,
                                      float4 em, float size) {
    bool zero;
    const float3 c = phat_full<POINT>(pos, ncode, sp, nside, nsign, brdf, em, size, &zero);
    if (zero) return 0.0f;
    const float r = sqrtf(dot3(c, c));
    if (isnan(r) || isinf(r)) return 0.0f;
    return r;
}

// ---- visibility (isLightOccluded, ris.cl:1-17) -----------------------------------------
// Persistent shadow tracer over the batch's request queue. Requests:
// qA = (origin, bits(view << 27 | pixel)), qB = (dir, bits(light)). Budget GRIDWIDTH = 128
// steps (ris.cl:10); a miss leaves dist/side at 0 (the fixed convention for the
// reference's uninitialised locals); visible iff the hit voxel (hit point - 0.1 N,
// truncated) lies in the emitter cube [pos, pos + size) (GridCoordinatesFromHit /
// Uint3CubeEquals, tools.cl:452-472). An occluded request zeroes sumOfWeights of its
// pixel in reservoir plane C (plane 0) or H (plane 1) of its view (W follows:
// ris.cl:79-80, 248-250). Lanes refill from the queue as soon as enough are idle. A walk
// stops early, as occluded, once its budget cannot reach the emitter (walk_target).
__device__ __forceinline__ void shadow_finish(const World& w, int st, const Walker& wk, float3 o, float3 L, uint32_t* plane,
                                              uint32_t pix, uint32_t li) {
    const float d2 = st == WALK_HIT ? wk.dist : 0.0f;
    const uint32_t s2 = st == WALK_HIT ? wk.side : 0u;
    const float ns = side_sign(s2, L);
    const float hx = L.x * d2 + o.x, hy = L.y * d2 + o.y, hz = L.z * d2 + o.z;
    const uint32_t vx = f2u(hx - (s2 == 0 ? ns * 0.1f : 0.0f));
    const uint32_t vy = f2u(hy - (s2 == 1 ? ns * 0.1f : 0.0f));
    const uint32_t vz = f2u(hz - (s2 == 2 ? ns * 0.1f : 0.0f));
    const uint32_t pos = __float_as_uint(__ldg(&w.lemit[li].w));
    const uint32_t size = (uint32_t)__ldg(&w.lgeom[li].w);
    const uint32_t ey = pos / (1024u * 1024u), ez = (pos / 1024u) % 1024u, ex = pos % 1024u;
    const bool inside = ex <= vx && ex + size > vx && ey <= vy && ey + size > vy && ez <= vz && ez + size > vz;
    if (!inside) plane[(size_t)pix * 4u + 2u] = 0u;
}

// MINB > 0 caps registers so that MINB blocks of 128 threads fit on an SM (more warps to
// hide L2 latency, at the price of a few spills); chosen by the launch tuning.
// CACHE = 1 (single views): blocks of 512 threads, brick walks through the cache walk: with
// a brick cache (bd.bcLog2 > 0) every block first copies the table and the opacity masks
// into shared memory; with bd.bcCount set they count brick walks (calibration).
// EARLY = 1: walks stop as occluded once their budget cannot reach the emitter.
template <int VARIANT, int MINB, int CACHE, int EARLY>
__global__ void __launch_bounds__(CACHE ? 512 : 128, CACHE ? 1 : MINB) shadow_kernel(const __grid_constant__ BatchDev bd,
                                                                                    int countIdx, int fetchIdx,
                                                                                    int planeSel) {
    const int refill = bd.refill, burst = bd.burst, schedule = bd.schedule;
    const uint32_t n = bd.counters[countIdx];
    uint32_t* fetch = bd.counters + fetchIdx;
    const int lane = threadIdx.x & 31;
    Walker wk;
    World wt;   // a table batch: the world of this lane's ray; one view: the parameter's
    if (CACHE) {
        extern __shared__ __align__(16) uint32_t bcs[];
        wt = bd.one.w;
        wt.bcCount = bd.bcCount;
        wt.bcLog2 = bd.bcLog2;
        if (bd.bcLog2 > 0) {
            const uint32_t nk = 1u << bd.bcLog2, nm = (nk >> 1) * 16u;
            for (uint32_t i = threadIdx.x; i < nk; i += blockDim.x) bcs[i] = __ldg(bd.bcKeys + i);
            for (uint32_t i = threadIdx.x; i < nm / 4u; i += blockDim.x)
                reinterpret_cast<uint4*>(bcs + nk)[i] = __ldg(reinterpret_cast<const uint4*>(bd.bcMask) + i);
            wt.bcKeys = bcs;
            wt.bcMask = bcs + nk;
        }
        __syncthreads();
    }
    const World& w = (VARIANT < 2 && !CACHE) ? bd.one.w : wt;
    uint32_t* plane = nullptr;
    bool active = false, exhausted = false;
    float3 o = f3(0.0f, 0.0f, 0.0f), L = f3(0.0f, 0.0f, 0.0f);
    uint32_t pix = 0, li = 0;
    while (true) {
        const unsigned idle = __ballot_sync(0xffffffffu, !active);
        if (!exhausted && (idle == 0xffffffffu || __popc(idle) >= refill)) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(fetch, (uint32_t)__popc(idle));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base + (uint32_t)__popc(idle) >= n) exhausted = true;
            if (!active) {
                const uint32_t r = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
                if (r < n) {
                    const float4 a = __ldg(bd.qA + r), b = __ldg(bd.qB + r);
                    o = f3(a.x, a.y, a.z);
                    L = f3(b.x, b.y, b.z);
                    const uint32_t e = __float_as_uint(a.w);
                    const ViewDev* V = view_of<VARIANT>(bd, e >> 27);
                    pix = pix_of<VARIANT>(e);
                    li = __float_as_uint(b.w);
                    if (VARIANT == 2) wt = V->w;
                    plane = reinterpret_cast<uint32_t*>(planeSel ? V->b.hA : V->b.cA);
                    const int st = walk_init(wk, w, o.x, o.y, o.z, L.x, L.y, L.z, 128);
                    if (st == WALK_CONTINUE) {
                        if (EARLY)
                            walk_target(wk, __float_as_uint(__ldg(&w.lemit[li].w)), (uint32_t)__ldg(&w.lgeom[li].w));
                        active = true;
                    } else {
                        shadow_finish(w, st, wk, o, L, plane, pix, li);
                    }
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) {
            if (exhausted) break;
            continue;
        }
        // schedule 1: only the lanes at the DDA level most lanes are at take this round
        // (one level's code per round instead of all three), and stop when they leave it
        int sel = -1;
        if (schedule) {
            const int n2 = __popc(__ballot_sync(0xffffffffu, active && wk.level == 2));
            const int n1 = __popc(__ballot_sync(0xffffffffu, active && wk.level == 1));
            const int n0 = __popc(__ballot_sync(0xffffffffu, active && wk.level == 0));
            sel = n2 >= n1 ? (n2 >= n0 ? 2 : 0) : (n1 >= n0 ? 1 : 0);
        }
        if (active && (sel < 0 || wk.level == sel)) {
#pragma unroll 1
            for (int s = 0; s < burst; s++) {
                const int st = walk_step<(CACHE ? kWalkCache : 0) | (EARLY ? kWalkEarly : 0)>(wk, w);
                if (st != WALK_CONTINUE) {
                    shadow_finish(w, st, wk, o, L, plane, pix, li);
                    active = false;
                    break;
                }
                if (sel >= 0 && wk.level != sel) break;
            }
        }
    }
}

// ---- stage 2a: candidates (perPixelInitialSampling, ris.cl:20-82) ---------------------------
// Over the hit list. Ends with AdjustWeight(res, res.pHat) (implied by the stored
// sumW, pHat, M) and a shadow-ray request for the selected sample when sumW > 0 (when
// sumW == 0 the discard of ris.cl:79-80 changes nothing).
// LEARNED: the light index and its source pdf p come from the learned proposal (drawn
// by the inference kernel) instead of GenerateLightCandidate's uniform 1 / N.
template <bool POINT, bool LEARNED>
__device__ __forceinline__ void ris_item(const BatchDev& bd, const ViewDev* V, uint32_t e, uint32_t i, uint32_t j) {
    const World w = V->w;
    const Frame& k = V->k;
    const int x = (int)(i % (uint32_t)k.W), y = (int)(i / (uint32_t)k.W);
    const uint2 g = V->b.vd[V->cur][i];
    const uint32_t voxel = g.x & 0x00FFFFFFu, side = g.x >> 24;
    const float dist = __uint_as_float(g.y);
    Res res = res_zero();
    uint32_t seed = V->b.seed[i];
    const float3 D = camera_ray(k, x, y);
    const float nsign = side_sign(side, D);
    const float3 brdf = mul(to_rgb(voxel), 0.31830988618379067153777f);
    const float3 sp = f3(D.x * dist + k.E.x, D.y * dist + k.E.y, D.z * dist + k.E.z);
    const float3 spo = f3(sp.x + (side == 0 ? 0.1f * nsign : 0.0f), sp.y + (side == 1 ? 0.1f * nsign : 0.0f),
                          sp.z + (side == 2 ? 0.1f * nsign : 0.0f));
    const uint32_t nL = k.nlights;
    const float puni = 1.0f / (float)nL;
    // x / (1 / N) is exactly x * N when N is a power of two (1 / N is then exact, and both
    // are the rounding of the same real number)
    const bool pow2 = !LEARNED && (nL & (nL - 1u)) == 0u;
    const float nLf = (float)nL;
    for (uint32_t c = 0; c < k.ncand; c++) {
        int li;
        float p = puni;
        if (LEARNED) {
            const uint2 cq = __ldg(V->ll.cand + (size_t)c * V->ll.stride + j);
            li = (int)cq.x;
            p = __uint_as_float(cq.y);
            // an entry the inference did not write (it gave up and raised its error flag):
            // a uniform candidate instead, so no index leaves the light table
            if (cq.x >= nL || !(p > 0.0f && p <= 1.0f)) {
                li = min(max(f2i(rnd(seed) * (float)nL), 0), (int)nL - 1);
                p = puni;
            }
        } else {
            // GenerateLightCandidate (tools.cl:593-598)
            li = min(max(f2i(rnd(seed) * (float)nL), 0), (int)nL - 1);
        }
        const float4 lg = __ldg(w.lgeom + li);
        const float4 le = __ldg(w.lemit + li);
        float3 pos;
        float inv;
        uint32_t nc;
        if (POINT) {
            pos = f3(lg.x, lg.y, lg.z);
            inv = 1.0f;
            nc = 6;
        } else {
            pos = sample_area_light(lg, spo, seed, &inv, &nc);
        }
        const float ph = phat<POINT>(pos, nc, sp, side, nsign, brdf, le, lg.w) * inv;
        res_update(res, pow2 ? ph * nLf : ph / p, ph, (uint32_t)li, rnd(seed), pos, inv, nc);
    }
    if (k.ncand > 0 && res.sumW > 0.0f) {
        const float3 L = normalize3(sub(res.pos, spo));
        const uint32_t slot = append_slot(bd.counters + kCtrQ1);
        bd.qA[slot] = make_float4(spo.x, spo.y, spo.z, __uint_as_float(e));
        bd.qB[slot] = make_float4(L.x, L.y, L.z, __uint_as_float(res.idx));
    }
    res_store(V->b.cA, V->b.cB, i, res);
    V->b.seed[i] = seed;
}

template <int VARIANT, bool LEARNED, int MINB>
__global__ void __launch_bounds__(128, MINB) ris_kernel(const __grid_constant__ BatchDev bd) {
    const uint32_t nh = bd.counters[kCtrHits];
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < nh; j += gridDim.x * blockDim.x) {
        const uint32_t e = bd.hits[j];
        const ViewDev* V = view_of<VARIANT>(bd, e >> 27);
        if (point_of<VARIANT>(V)) ris_item<true, LEARNED>(bd, V, e, pix_of<VARIANT>(e), j);
        else ris_item<false, LEARNED>(bd, V, e, pix_of<VARIANT>(e), j);
    }
}

// ---- stage 2c: temporal reuse (ris.cl:84-119) over the hit list, after visibility ------------
template <bool POINT>
__device__ __forceinline__ void temporal_item(const ViewDev* V, uint32_t i) {
    const Frame& k = V->k;
    if (!(k.restirtemporalframe > 0 && k.temporal)) return;
    // loads are issued as early as their addresses are known (before the tests that may
    // make them unneeded), so the item waits for three rounds of memory instead of five
    const uint4 ca = __ldg(V->b.cA + i);
    const float4 cb = __ldg(V->b.cB + i);
    const uint32_t seed0 = V->b.seed[i];
    const int x = (int)(i % (uint32_t)k.W), y = (int)(i / (uint32_t)k.W);
    const uint2 g = V->b.vd[V->cur][i];
    const uint32_t voxel = g.x & 0x00FFFFFFu, side = g.x >> 24;
    const float dist = __uint_as_float(g.y);
    const float3 D = camera_ray(k, x, y);
    const float3 sp = f3(D.x * dist + k.E.x, D.y * dist + k.E.y, D.z * dist + k.E.z);
    const float dl = ((sp.x * k.Nl.x + sp.y * k.Nl.y) + sp.z * k.Nl.z) - k.Nl.w;
    const float dr = ((sp.x * k.Nr.x + sp.y * k.Nr.y) + sp.z * k.Nr.z) - k.Nr.w;
    const float dt = ((sp.x * k.Nt.x + sp.y * k.Nt.y) + sp.z * k.Nt.z) - k.Nt.w;
    const float db = ((sp.x * k.Nb.x + sp.y * k.Nb.y) + sp.z * k.Nb.z) - k.Nb.w;
    const float up = (float)k.W * (dl / (dl + dr));
    const float vp = (float)k.H * (dt / (dt + db));
    const float ru = roundf(up), rv = roundf(vp);
    if (!(ru == ru && rv == rv)) return;
    const int px = f2i(ru), py = f2i(rv);
    if (px < 0 || py < 0 || px >= k.W || py >= k.H) return;
    const size_t jp = (size_t)py * k.W + px;
    const uint2 pg = __ldg(V->b.vd[V->cur ^ 1] + jp);
    Res prev = res_load(V->b.hA, V->b.hB, jp);
    const float pdist = __uint_as_float(pg.y);
    if ((pg.x >> 24) != side || !(fabsf(dist - pdist) <= 0.1f * dist)) return;
    const uint32_t pm = min(k.maxTemporal * k.ncand, prev.M);
    if (pm == 0u) return;
    uint32_t pli = prev.idx;
    if (pli >= k.nlights) { raise_error(V->b.err, 2u); pli = 0; }
    const float nsign = side_sign(side, D);
    const float3 brdf = mul(to_rgb(voxel), 0.31830988618379067153777f);
    const float4 pg4 = __ldg(V->w.lgeom + pli), pe4 = __ldg(V->w.lemit + pli);
    const float pph = phat<POINT>(prev.pos, prev.ncode, sp, side, nsign, brdf, pe4, pg4.w) * prev.inv;
    const float W = res_W(prev);
    res_reweigh(prev, W, pph, pm);
    Res res;
    res.idx = ca.x;
    res.M = ca.y & 0x1FFFFFFFu;
    res.ncode = ca.y >> 29;
    res.sumW = __uint_as_float(ca.z);
    res.pHat = __uint_as_float(ca.w);
    res.pos = f3(cb.x, cb.y, cb.z);
    res.inv = cb.w;
    uint32_t seed = seed0;
    res_combine(res, prev, rnd(seed));
    // AdjustWeight(res, pHat of the selected sample here) equals res.pHat
    res_store(V->b.cA, V->b.cB, i, res);
    V->b.seed[i] = seed;
}

template <int VARIANT>
__global__ void __launch_bounds__(128) temporal_kernel(const __grid_constant__ BatchDev bd) {
    const uint32_t nh = bd.counters[kCtrHits];
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < nh; j += gridDim.x * blockDim.x) {
        const uint32_t e = bd.hits[j];
        const ViewDev* V = view_of<VARIANT>(bd, e >> 27);
        if (point_of<VARIANT>(V)) temporal_item<true>(V, pix_of<VARIANT>(e));
        else temporal_item<false>(V, pix_of<VARIANT>(e));
    }
}

// ---- stage 3: spatial reuse (perPixelSpatialResampling, ris.cl:126-151,
//      spatialSampling.cl:2-66) -------------------------------------------------------
template <bool POINT>
__device__ __forceinline__ void spatial_px(const ViewDev* V, int x, int y) {
    const Frame& k = V->k;
    const size_t i = (size_t)y * k.W + x;
    const uint4* cA = V->b.cA;
    const float4* cB = V->b.cB;
    const uint2* vd = V->b.vd[V->cur];
    Res res = res_load(cA, cB, i);
    const uint2 g = vd[i];
    const uint32_t voxel = g.x & 0x00FFFFFFu;
    if (voxel != 0u && k.spatial) {
        const uint32_t side = g.x >> 24;
        const float dist = __uint_as_float(g.y);
        uint32_t seed = V->b.seed[i];
        const float3 D = camera_ray(k, x, y);
        const float nsign = side_sign(side, D);
        const float3 brdf = mul(to_rgb(voxel), 0.31830988618379067153777f);
        const float3 sp = f3(D.x * dist + k.E.x, D.y * dist + k.E.y, D.z * dist + k.E.z);
        const float rad = (float)(k.radius - 1u);
        for (uint32_t t = 0; t < k.taps; t++) {
            const float angle = rnd(seed) * 6.28318530717958647692528f;
            const float radius = rad * sqrtf(rnd(seed)) + 1.0f;
            float sn, cs;
            sincos_vx(angle, &sn, &cs);
            const int nx = x + f2i(cs * radius), ny = y + f2i(sn * radius);
            if ((nx == x && ny == y) || nx < 0 || ny < 0 || nx >= k.W || ny >= k.H) continue;
            const size_t j = (size_t)ny * k.W + nx;
            Res nb = res_load(cA, cB, j);
            const uint2 ng = __ldg(vd + j);
            // the light record is fetched with the tests still pending (it is needed when
            // they pass), one round of memory fewer per combined tap
            const uint32_t nli = nb.idx < k.nlights ? nb.idx : 0u;
            const float4 lg = __ldg(V->w.lgeom + nli), le = __ldg(V->w.lemit + nli);
            if (nb.M > 0u) {
                const float ndist = __uint_as_float(ng.y);
                if ((ng.x >> 24) == side && fabsf(dist - ndist) <= 0.1f * dist) {
                    if (nb.idx >= k.nlights) raise_error(V->b.err, 4u);
                    const float ph = phat<POINT>(nb.pos, nb.ncode, sp, side, nsign, brdf, le, lg.w) * nb.inv;
                    const float W = res_W(nb);
                    res_reweigh(nb, W, ph, nb.M);
                    res_combine(res, nb, rnd(seed));
                }
            }
        }
        // AdjustWeight(res, res.pHat): implied by the stored (sumW, pHat, M)
        V->b.seed[i] = seed;
    }
    res_store(V->b.hA, V->b.hB, i, res);
}

template <int VARIANT>
__global__ void __launch_bounds__(kMaxTileThreads) spatial_kernel(const __grid_constant__ BatchDev bd) {
    uint32_t tile, round = 0;
    while (next_tile(bd, bd.counters + kCtrSpatial, &tile, round)) {
        int x, y;
        const ViewDev* V = tile_pixel<VARIANT>(bd, tile, &x, &y);
        if (x < V->k.W && y < V->k.H) {
            if (point_of<VARIANT>(V)) spatial_px<true>(V, x, y);
            else spatial_px<false>(V, x, y);
        }
    }
}

// ---- stage 4: shading (renderRIS / render_di_ris, ris.cl:155-293, 391-413) ------------------
// 4a: a shadow-ray request for every hit pixel whose reservoir has W > 0 and M > 0.
template <int VARIANT>
__global__ void __launch_bounds__(128) shade_request_kernel(const __grid_constant__ BatchDev bd) {
    const uint32_t nh = bd.counters[kCtrHits];
    // every thread of a block runs the same iterations (block_append needs all of them)
    for (uint32_t j0 = blockIdx.x * blockDim.x; j0 < nh; j0 += gridDim.x * blockDim.x) {
        const uint32_t j = j0 + threadIdx.x;
        bool want = false;
        float4 ra = make_float4(0.0f, 0.0f, 0.0f, 0.0f), rb = ra;
        if (j < nh) {
            const uint32_t e = bd.hits[j];
            const ViewDev* V = view_of<VARIANT>(bd, e >> 27);
            const Frame& k = V->k;
            const uint32_t i = pix_of<VARIANT>(e);
            const uint4 qa = V->b.hA[i];
            const uint32_t M = qa.y & 0x1FFFFFFFu;
            const float W = __uint_as_float(qa.z) / fmaxf(1e-5f, __uint_as_float(qa.w) * (float)M);
            if (W > 0.0f && M > 0u) {
                const int x = (int)(i % (uint32_t)k.W), y = (int)(i / (uint32_t)k.W);
                const uint2 g = V->b.vd[V->cur][i];
                const uint32_t side = g.x >> 24;
                const float dist = __uint_as_float(g.y);
                const float3 D = camera_ray(k, x, y);
                const float nsign = side_sign(side, D);
                const float3 sp = f3(D.x * dist + k.E.x, D.y * dist + k.E.y, D.z * dist + k.E.z);
                const float3 spo = f3(sp.x + (side == 0 ? 0.1f * nsign : 0.0f), sp.y + (side == 1 ? 0.1f * nsign : 0.0f),
                                      sp.z + (side == 2 ? 0.1f * nsign : 0.0f));
                uint32_t li = qa.x;
                if (li >= k.nlights) { raise_error(V->b.err, 8u); li = 0; }
                const float4 qb = __ldg(V->b.hB + i);
                const float3 L = normalize3(sub(f3(qb.x, qb.y, qb.z), spo));
                ra = make_float4(spo.x, spo.y, spo.z, __uint_as_float(e));
                rb = make_float4(L.x, L.y, L.z, __uint_as_float(li));
                want = true;
            }
        }
        const uint32_t slot = block_append(bd.counters + kCtrQ2, want);
        if (want) {
            bd.qA[slot] = ra;
            bd.qB[slot] = rb;
        }
    }
}

// ---- sky dome (tools.cl:6-15, 21-28, 54-70, 130-144) --------------------------------
// acos, atan2, sin and cos are the correctly rounded binary32 values (through double).

// SampleSky with SphericalTheta / SphericalPhi: bilinear lookup of direction (tx, ty, tz)
// in the z-up sky texture
__device__ __forceinline__ float3 sample_sky(const Sky& s, float tx, float ty, float tz) {
    const float PI = 3.14159265358979323846264f;
    const float INV2PI = 0.15915494309189533576888f, INVPI = 0.31830988618379067153777f;
    const float theta = (float)acos((double)fminf(fmaxf(tz, -1.0f), 1.0f));
    float phi = (float)atan2((double)ty, (double)tx);
    phi = phi < 0.0f ? phi + 2.0f * PI : phi;
    const float u = ((float)s.w * phi) * INV2PI - 0.5f;
    const float v = ((float)s.h * theta) * INVPI - 0.5f;
    const float fu = u - floorf(u), fv = v - floorf(v);
    const uint32_t iu = (uint32_t)f2i(u), iv = (uint32_t)f2i(v), n = s.w * s.h;
    const float4 a = __ldg(s.tex + (iu + iv * s.w) % n), b = __ldg(s.tex + (iu + 1u + iv * s.w) % n);
    const float4 c = __ldg(s.tex + (iu + (iv + 1u) * s.w) % n), d = __ldg(s.tex + (iu + 1u + (iv + 1u) * s.w) % n);
    const float gu = 1.0f - fu, gv = 1.0f - fv;
    return f3((((a.x * gu) * gv + (b.x * fu) * gv) + (c.x * gu) * fv) + (d.x * fu) * fv,
              (((a.y * gu) * gv + (b.y * fu) * gv) + (c.y * gu) * fv) + (d.y * fu) * fv,
              (((a.z * gu) * gv + (b.z * fu) * gv) + (c.z * gu) * fv) + (d.z * fu) * fv);
}

// blueNoiseSampler: E. Heitz's ranked, scrambled sequence, sample `idx`, dimension `dim`
__device__ __forceinline__ float blue_noise(const uint32_t* bn, int x, int y, int idx, int dim) {
    x &= 127, y &= 127, idx &= 255, dim &= 255;
    const int ranked = (idx ^ (int)__ldg(bn + dim + (x + y * 128) * 8 + 65536 * 3)) & 255;
    int value = (int)__ldg(bn + dim + ranked * 256);
    value ^= (int)__ldg(bn + (dim & 7) + (x + y * 128) * 8 + 65536);
    float r = (0.5f + (float)value) * (1.0f / 256.0f);
    if (r >= 1.0f) r -= 1.0f;
    return r;
}

// DiffuseReflectionCosWeighted: cosine-weighted direction around N
__device__ __forceinline__ float3 cos_weighted(float r0, float r1, float3 N) {
    const float3 T = normalize3(cross3(N, fabsf(N.y) > 0.99f ? f3(1.0f, 0.0f, 0.0f) : f3(0.0f, 1.0f, 0.0f)));
    const float3 B = cross3(T, N);
    const float term1 = 6.28318530717958647692528f * r0, term2 = sqrtf(1.0f - r1);
    double sd, cd;
    sincos((double)term1, &sd, &cd);          // one argument reduction for both
    const float c = (float)cd, s = (float)sd;
    const float ct = c * term2, st = s * term2, sr = sqrtf(r1);
    return f3((ct * T.x + st * B.x) + sr * N.x, (ct * T.y + st * B.y) + sr * N.y, (ct * T.z + st * B.z) + sr * N.z);
}

// skyLight entry of an axis normal (ris.cl:279-285: the last matching test wins)
__device__ __forceinline__ float4 sky_light(const Sky& s, float3 M) {
    float4 l = s.light[0];
    if (M.x > 0.9f) l = s.light[1];
    if (M.y < -0.9f) l = s.light[2];
    if (M.y > 0.9f) l = s.light[3];
    if (M.z < -0.9f) l = s.light[4];
    if (M.z > 0.9f) l = s.light[5];
    return l;
}

// accumulatorFinalizer (kernels.cl:304-326): running mean over `framecount` frames
__device__ __forceinline__ void accumulate_px(const ViewDev* V, size_t i, float4 px) {
    const Frame& k = V->k;
    const int n = (int)k.framecount * k.accumulate;
    float4 prev = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (n > 0) prev = V->b.accum[i];
    const float cw = 1.0f / (float)(1 + n);
    V->b.accum[i] = make_float4((1.0f - cw) * prev.x + cw * px.x, (1.0f - cw) * prev.y + cw * px.y,
                                (1.0f - cw) * prev.z + cw * px.z, 1.0f);
}

// 4c: colour per pixel once visibility has zeroed the occluded reservoirs; optionally
// fused with the accumulator. SKY: the frame may carry a sky dome (the sky-less
// instantiation keeps the common case's registers).
template <bool POINT, bool SKY>
__device__ __forceinline__ void shade_finish_px(const ViewDev* V, int x, int y, int fuse) {
    const Frame& k = V->k;
    const size_t i = (size_t)y * k.W + x;
    const uint2 g = V->b.vd[V->cur][i];
    const uint32_t voxel = g.x & 0x00FFFFFFu;
    const float dist = __uint_as_float(g.y);
    const float INVPI = 0.31830988618379067153777f;
    float3 color = f3(0.0f, 0.0f, 0.0f);
    const Sky* sky = SKY ? k.sky : nullptr;
    if (sky && voxel == 0u) {
        // background (ris.cl:197-202); the sky-light term adds its incoming light times a
        // zero BRDF, which leaves non-negative sums as they are
        const float3 D = camera_ray(k, x, y);
        color = sample_sky(*sky, D.x, D.z, D.y);
        const float4 l = sky_light(*sky, side_normal(g.x >> 24, side_sign(g.x >> 24, D)));
        color = add(color, f3((0.0f + sky->lightScale * l.x) * 0.0f, (0.0f + sky->lightScale * l.y) * 0.0f,
                              (0.0f + sky->lightScale * l.z) * 0.0f));
    }
    if (voxel != 0u) {
        float3 skyC = f3(0.0f, 0.0f, 0.0f);   // sky seen through a translucent voxel (ris.cl:206-211)
        if (sky && ((voxel & 0xf000u) >> 12) != 15u) {
            const float3 D = camera_ray(k, x, y);
            skyC = sample_sky(*sky, D.x, D.z, D.y);
        }
        if (emitter(voxel)) {
            const float3 c = to_rgb(voxel);
            const float m = strength(voxel);
            color = add(color, f3((c.x * m) * INVPI, (c.y * m) * INVPI, (c.z * m) * INVPI));
        }
        const uint4 qa = V->b.hA[i];
        const uint32_t M = qa.y & 0x1FFFFFFFu;
        const float W = __uint_as_float(qa.z) / fmaxf(1e-5f, __uint_as_float(qa.w) * (float)M);
        if (W > 0.0f && M > 0u) {   // visible: occluded reservoirs were zeroed by the tracer
            const uint32_t side = g.x >> 24;
            const float4 qb = __ldg(V->b.hB + i);
            const float3 D = camera_ray(k, x, y);
            const float nsign = side_sign(side, D);
            const float3 sp = f3(D.x * dist + k.E.x, D.y * dist + k.E.y, D.z * dist + k.E.z);
            const uint32_t li = qa.x < k.nlights ? qa.x : 0u;
            const float4 lg = __ldg(V->w.lgeom + li), le = __ldg(V->w.lemit + li);
            const float3 brdf = mul(to_rgb(voxel), INVPI);
            bool zero;
            const float3 inc = phat_full<POINT>(f3(qb.x, qb.y, qb.z), qa.y >> 29, sp, side, nsign, brdf, le, lg.w, &zero);
            color = add(color, f3((inc.x * W) * qb.w, (inc.y * W) * qb.w, (inc.z * W) * qb.w));
        }
        const float a = alphaf(voxel);
        color = f3(color.x + ((a * color.x) + ((1.0f - a) * skyC.x)), color.y + ((a * color.y) + ((1.0f - a) * skyC.y)),
                   color.z + ((a * color.z) + ((1.0f - a) * skyC.z)));
        if (sky) {
            // sky light (ris.cl:258-290): one cosine-weighted ray, 10 steps, opaque voxels
            // only; lit by the sky light of the normal it ends on
            const uint32_t side = g.x >> 24;
            const float3 D = camera_ray(k, x, y);
            const float3 N = side_normal(side, side_sign(side, D));
            const float r0 = blue_noise(sky->blueNoise, x, y, (int)k.frame, 0);
            const float r1 = blue_noise(sky->blueNoise, x, y, (int)k.frame, 1);
            const float3 R = cos_weighted(r0, r1, N);
            const float3 sp = f3(D.x * dist + k.E.x, D.y * dist + k.E.y, D.z * dist + k.E.z);
            float dist2 = 0.0f;
            uint32_t side2 = 0;
            const uint32_t voxel2 = trace<1>(V->w, sp.x + 0.1f * N.x, sp.y + 0.1f * N.y, sp.z + 0.1f * N.z, R.x, R.y, R.z,
                                             10 /* GRIDWIDTH / 12 */, 0u, 0u, &dist2, &side2);
            float3 toAdd = f3(sky->lightScale, sky->lightScale, sky->lightScale), M = N;
            if (voxel2 != 0u) {
                const float3 c2 = to_rgb(voxel2);
                toAdd = f3(toAdd.x * (INVPI * c2.x), toAdd.y * (INVPI * c2.y), toAdd.z * (INVPI * c2.z));
                M = side_normal(side2, side_sign(side2, R));
            }
            const float4 l = sky_light(*sky, M);
            const float3 inc = f3(0.0f + toAdd.x * l.x, 0.0f + toAdd.y * l.y, 0.0f + toAdd.z * l.z);
            const float3 brdf = mul(to_rgb(voxel), INVPI);
            color = add(color, mulv(inc, brdf));
        }
    }
    const float4 px = make_float4(color.x, color.y, color.z, dist);
    V->b.frame[i] = px;
    if (fuse) accumulate_px(V, i, px);
}

template <int VARIANT, bool SKY>
__global__ void __launch_bounds__(kMaxTileThreads) shade_finish_kernel(const __grid_constant__ BatchDev bd) {
    uint32_t tile, round = 0;
    while (next_tile(bd, bd.counters + kCtrFinish, &tile, round)) {
        int x, y;
        const ViewDev* V = tile_pixel<VARIANT>(bd, tile, &x, &y);
        if (x < V->k.W && y < V->k.H) {
            if (point_of<VARIANT>(V)) shade_finish_px<true, SKY>(V, x, y, bd.fuse);
            else shade_finish_px<false, SKY>(V, x, y, bd.fuse);
        }
    }
}

// stage 5 on its own
template <int VARIANT>
__global__ void __launch_bounds__(kMaxTileThreads) accumulate_kernel(const __grid_constant__ BatchDev bd) {
    uint32_t tile, round = 0;
    while (next_tile(bd, bd.counters + kCtrAccum, &tile, round)) {
        int x, y;
        const ViewDev* V = tile_pixel<VARIANT>(bd, tile, &x, &y);
        if (x < V->k.W && y < V->k.H) {
            const size_t i = (size_t)y * V->k.W + x;
            accumulate_px(V, i, V->b.frame[i]);
        }
    }
}

}  // namespace dev
}  // namespace vxr

// ---- launchers -------------------------------------------------------------------------
namespace vxr {

static int g_sms = 0;
static int sm_count() {
    if (!g_sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_sms <= 0) g_sms = 1;
    }
    return g_sms;
}
// grid-stride kernels over a list of at most n items
static unsigned list_blocks(size_t n, int threads, int per_sm) {
    const size_t need = (n + threads - 1) / threads;
    const size_t cap = (size_t)sm_count() * per_sm;
    return (unsigned)std::max<size_t>(1, std::min(need, cap));
}
// Persistent kernels: as many blocks as fit on the machine at once (occupancy query per
// kernel and block size, cached), never more than there are tiles.
static unsigned resident_blocks(const void* kernel, int threads) {
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, int> cache;
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find({kernel, threads});
    if (it == cache.end()) {
        int per = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, 0) != cudaSuccess || per < 1) per = 1;
        it = cache.emplace(std::make_pair(kernel, threads), per).first;
    }
    return (unsigned)(sm_count() * it->second);
}
// brackets one kernel launch with the attached timer's events
struct Timed {
    const BatchDev& bd;
    int id;
    cudaStream_t s;
    Timed(const BatchDev& b, int i, cudaStream_t st) : bd(b), id(i), s(st) {
        if (bd.timer) bd.timer->mark(id, false, s);
    }
    ~Timed() {
        if (bd.timer) bd.timer->mark(id, true, s);
    }
};

template <class K>
static void launch_tiles(K kernel, const BatchDev& bd, int ctr, cudaStream_t s, int id) {
    const int threads = bd.tx * bd.ty;
    unsigned nb = std::max(1u, bd.totalTiles);
    if (bd.persistent) {
        cudaMemsetAsync(bd.counters + ctr, 0, sizeof(uint32_t), s);
        nb = std::max(1u, std::min(resident_blocks((const void*)kernel, threads), bd.totalTiles));
    }
    Timed tm(bd, id, s);
    kernel<<<nb, threads, 0, s>>>(bd);
}

void apply_tuning(BatchDev& bd, const Tuning& tu) {
    bd.tx = tu.bx;
    bd.ty = tu.by;
    bd.persistent = tu.persistent;
    bd.refill = tu.refill;
    bd.burst = tu.burst;
    bd.listPerSm = tu.listPerSm;
    bd.occupancy = tu.occupancy;
    bd.schedule = tu.schedule;
    bd.earlyOut = tu.earlyOut;
}

BatchDev single_batch(const dev::World& w, const dev::Frame& k, const ViewBuffers& b, int cur, bool point, const Tuning& tu) {
    BatchDev bd;
    bd.one.w = w;
    bd.one.k = k;
    bd.one.b = b;
    bd.one.cur = cur;
    bd.one.point = point ? 1 : 0;
    bd.one.tileBase = 0;
    bd.one.tilesX = (uint32_t)((k.W + tu.bx - 1) / tu.bx);
    bd.nviews = 1;
    bd.sky = k.sky != nullptr ? 1 : 0;
    bd.totalPixels = (uint32_t)k.W * (uint32_t)k.H;
    bd.totalTiles = bd.one.tilesX * (uint32_t)((k.H + tu.by - 1) / tu.by);
    apply_tuning(bd, tu);
    bd.hits = b.hits;
    bd.qA = b.qA;
    bd.qB = b.qB;
    bd.counters = b.counters;
    return bd;
}

void launch_build_light_table(const uint4* raw, uint32_t n, float4* geom, float4* emit, cudaStream_t s) {
    if (n == 0) return;
    dev::build_light_table_kernel<<<(n + 255) / 256, 256, 0, s>>>(raw, n, geom, emit);
}

void launch_build_uber(const uint32_t* grid, uint8_t* uber, cudaStream_t s) {
    dev::build_uber_kernel<<<(32 * 32 * 32 + 255) / 256, 256, 0, s>>>(grid, uber);
}

void launch_build_brick_boxes(const uint32_t* bricks, const uint32_t* list, uint32_t n, uint32_t* bbox, uint32_t* bbox0,
                              cudaStream_t s) {
    const size_t threads = (size_t)n * 32u;
    if (threads)
        dev::build_brick_boxes_kernel<<<(unsigned)((threads + 255u) / 256u), 256, 0, s>>>(bricks, list, n, bbox, bbox0);
}

void launch_commit_bricks(const uint32_t* list, const uint32_t* voxels, uint32_t n, uint32_t* bricks, cudaStream_t s) {
    if (n) dev::commit_bricks_kernel<<<n, 128, 0, s>>>(list, voxels, bricks);
}

void launch_build_uber_boxes(const uint32_t* grid, const uint32_t* bbox0, uint32_t* ubox0, cudaStream_t s) {
    dev::build_uber_boxes_kernel<<<(32 * 32 * 32 + 255) / 256, 256, 0, s>>>(grid, bbox0, ubox0);
}

void launch_path_trace(const BatchDev& bd, cudaStream_t s) {
    BatchDev b = bd;
    b.timer = nullptr;
    launch_tiles(dev::path_trace_kernel, b, kCtrAlbedo, s, K_ALBEDO);
}

void launch_batch_albedo(const BatchDev& bd, int variant, cudaStream_t s) {
    if (variant == 2) launch_tiles(dev::albedo_kernel<2>, bd, kCtrAlbedo, s, K_ALBEDO);
    else launch_tiles(dev::albedo_kernel<0>, bd, kCtrAlbedo, s, K_ALBEDO);
}

template <int VARIANT, int MINB, int EARLY>
static void launch_shadow_k(const BatchDev& bd, int countIdx, int planeSel, cudaStream_t s) {
    const size_t rb = resident_blocks((const void*)dev::shadow_kernel<VARIANT, MINB, 0, EARLY>, 128);
    const unsigned nb = (unsigned)std::max<size_t>(1, std::min<size_t>(rb, ((size_t)bd.totalPixels + 127) / 128));
    Timed tm(bd, planeSel ? K_SHADOW_SHADE : K_SHADOW_CAND, s);
    dev::shadow_kernel<VARIANT, MINB, 0, EARLY><<<nb, 128, 0, s>>>(bd, countIdx, countIdx + 1, planeSel);
}
// shared memory of the brick-cache variant: 2^log2 keys and 2^(log2 - 1) masks of 64 bytes
size_t brick_cache_smem(int log2) { return log2 > 0 ? ((size_t)4 << log2) + ((size_t)64 << (log2 - 1)) : 0; }
template <int EARLY>
static void launch_shadow_cached(const BatchDev& bd, int countIdx, int planeSel, cudaStream_t s) {
    const void* fn = (const void*)dev::shadow_kernel<0, 0, 1, EARLY>;
    const size_t sm = brick_cache_smem(bd.bcLog2);
    if (sm > 48 * 1024) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, 512, sm);
    const size_t rb = (size_t)std::max(per, 1) * (size_t)sm_count();
    const unsigned nb = (unsigned)std::max<size_t>(1, std::min<size_t>(rb, ((size_t)bd.totalPixels + 511) / 512));
    Timed tm(bd, planeSel ? K_SHADOW_SHADE : K_SHADOW_CAND, s);
    dev::shadow_kernel<0, 0, 1, EARLY><<<nb, 512, sm, s>>>(bd, countIdx, countIdx + 1, planeSel);
}
template <int VARIANT>
static void launch_shadow(const BatchDev& bd, int countIdx, int planeSel, cudaStream_t s) {
    const bool early = bd.earlyOut != 0;
    if (VARIANT < 2 && (bd.bcLog2 > 0 || bd.bcCount)) {
        if (early) launch_shadow_cached<1>(bd, countIdx, planeSel, s);
        else launch_shadow_cached<0>(bd, countIdx, planeSel, s);
    } else if (bd.occupancy) {
        if (early) launch_shadow_k<VARIANT, 8, 1>(bd, countIdx, planeSel, s);
        else launch_shadow_k<VARIANT, 8, 0>(bd, countIdx, planeSel, s);
    } else {
        if (early) launch_shadow_k<VARIANT, 0, 1>(bd, countIdx, planeSel, s);
        else launch_shadow_k<VARIANT, 0, 0>(bd, countIdx, planeSel, s);
    }
}
template <int VARIANT, bool LEARNED>
static void launch_ris(const BatchDev& bd, unsigned nb, cudaStream_t s) {
    Timed tm(bd, K_RIS, s);
    if (bd.occupancy) dev::ris_kernel<VARIANT, LEARNED, 7><<<nb, 128, 0, s>>>(bd);
    else dev::ris_kernel<VARIANT, LEARNED, 0><<<nb, 128, 0, s>>>(bd);
}

template <int VARIANT>
static void candidates_v(const BatchDev& bd, const LearnedHook* learned, cudaStream_t s, cudaStream_t tail,
                         cudaEvent_t ev) {
    const size_t n = bd.totalPixels;
    cudaMemsetAsync(bd.counters + kCtrHits, 0, 3 * sizeof(uint32_t), s);   // hits, q1 requests, q1 fetch
    uint32_t maxPx = VARIANT < 2 ? bd.totalPixels : 0;
    if (VARIANT == 2) maxPx = (uint32_t)(n / bd.nviews + 1);
    {
        Timed tm(bd, K_COMPACT, s);
        dev::compact_hits_kernel<VARIANT><<<dim3(list_blocks(maxPx, 256, 8), bd.nviews), 256, 0, s>>>(bd);
    }
    const unsigned nb = list_blocks(n, 128, bd.listPerSm);
    bool learnedDone = false;
    if constexpr (VARIANT < 2) {
        if (learned) {
            BatchDev lb = bd;
            lb.one.ll.cand = learned->cand;
            lb.one.ll.stride = (uint32_t)n;
            prop::InferArgs ia = learned->infer;
            ia.k = bd.one.k;
            ia.vd = bd.one.b.vd[bd.one.cur];
            ia.hits = bd.hits;
            ia.count = bd.counters + kCtrHits;
            ia.ncand = bd.one.k.ncand;
            ia.cand = learned->cand;
            ia.clOff = learned->clOff;
            ia.clMembers = learned->clMembers;
            ia.lightCluster = learned->lightCluster;
            ia.nlights = bd.one.k.nlights;
            ia.candStride = (uint32_t)n;
            ia.err = bd.one.b.err;
            ia.samples = nullptr;
            ia.probs = nullptr;
            if (bd.one.k.ncand > 0) {
                Timed tm(bd, K_INFER, s);
                if (learned->rows) {
                    cudaMemsetAsync(learned->rowCount, 0, sizeof(uint32_t), s);
                    prop::launch_pair_rows(ia.k, ia.vd, ia.hits, ia.count, (uint32_t)n, learned->group,
                                           learned->pairDist, learned->rows, learned->rowCount, s);
                    ia.rows = learned->rows;
                    ia.rowCount = learned->rowCount;
                }
                prop::launch_infer(ia, (uint32_t)n, s);
            }
            launch_ris<VARIANT, true>(lb, nb, s);
            learnedDone = true;
        }
    }
    if (!learnedDone) launch_ris<VARIANT, false>(bd, nb, s);
    launch_shadow<VARIANT < 2 ? 0 : 2>(bd, kCtrQ1, 0, s);
    if (tail && tail != s) {
        cudaEventRecord(ev, s);
        cudaStreamWaitEvent(tail, ev, 0);
        s = tail;
    }
    // a single view without temporal reuse this frame skips the launch (a table checks per view)
    if (VARIANT == 2 || (bd.one.k.restirtemporalframe > 0 && bd.one.k.temporal)) {
        Timed tm(bd, K_TEMPORAL, s);
        dev::temporal_kernel<VARIANT><<<nb, 128, 0, s>>>(bd);
    }
}

void launch_batch_candidates(const BatchDev& bd, int variant, const LearnedHook* learned, cudaStream_t s,
                             cudaStream_t tail, cudaEvent_t ev) {
    if (variant == 0) candidates_v<0>(bd, learned, s, tail, ev);
    else if (variant == 1) candidates_v<1>(bd, learned, s, tail, ev);
    else candidates_v<2>(bd, nullptr, s, tail, ev);
}

void launch_batch_spatial(const BatchDev& bd, int variant, cudaStream_t s) {
    if (variant == 0) launch_tiles(dev::spatial_kernel<0>, bd, kCtrSpatial, s, K_SPATIAL);
    else if (variant == 1) launch_tiles(dev::spatial_kernel<1>, bd, kCtrSpatial, s, K_SPATIAL);
    else launch_tiles(dev::spatial_kernel<2>, bd, kCtrSpatial, s, K_SPATIAL);
}

template <int VARIANT>
static void shade_v(const BatchDev& bd, cudaStream_t s) {
    cudaMemsetAsync(bd.counters + kCtrQ2, 0, 2 * sizeof(uint32_t), s);   // q2 requests, q2 fetch
    {
        Timed tm(bd, K_SHADE_REQ, s);
        dev::shade_request_kernel<VARIANT < 2 ? 0 : 2><<<list_blocks(bd.totalPixels, 128, bd.listPerSm), 128, 0, s>>>(bd);
    }
    launch_shadow<VARIANT < 2 ? 0 : 2>(bd, kCtrQ2, 1, s);
    if (bd.sky) launch_tiles(dev::shade_finish_kernel<VARIANT, true>, bd, kCtrFinish, s, K_SHADE_FINISH);
    else launch_tiles(dev::shade_finish_kernel<VARIANT, false>, bd, kCtrFinish, s, K_SHADE_FINISH);
}

void launch_batch_shade(const BatchDev& bd, int variant, cudaStream_t s) {
    if (variant == 0) shade_v<0>(bd, s);
    else if (variant == 1) shade_v<1>(bd, s);
    else shade_v<2>(bd, s);
}

void launch_batch_accumulate(const BatchDev& bd, int variant, cudaStream_t s) {
    if (variant == 2) launch_tiles(dev::accumulate_kernel<2>, bd, kCtrAccum, s, K_ACCUM);
    else launch_tiles(dev::accumulate_kernel<0>, bd, kCtrAccum, s, K_ACCUM);
}

}  // namespace vxr

// ---- converged reference and error metric ----------------------------------------------
namespace vxr {
namespace dev {

// FP64 running sum of the shaded frame's rgb (converged reference render).
__global__ void __launch_bounds__(256) sum64_add_kernel(const float4* __restrict__ frame, double* __restrict__ sum,
                                                        uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 f = frame[i];
        sum[3 * (size_t)i + 0] += (double)f.x;
        sum[3 * (size_t)i + 1] += (double)f.y;
        sum[3 * (size_t)i + 2] += (double)f.z;
    }
}

// CalculateMSE / CalculateRMAE (mse.cpp:33-65): the ground truth is the FP64 mean
// rounded to float (the reference compares float images); per pixel the squared and
// absolute channel errors are summed in float as mse.cpp does, then accumulated in FP64.
__global__ void __launch_bounds__(256) error_kernel(const float4* __restrict__ img, const double* __restrict__ sum,
                                                    double inv_count, uint32_t n, double* out) {
    double se = 0.0, ae = 0.0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 x = img[i];
        const float gx = (float)(sum[3 * (size_t)i + 0] * inv_count);
        const float gy = (float)(sum[3 * (size_t)i + 1] * inv_count);
        const float gz = (float)(sum[3 * (size_t)i + 2] * inv_count);
        const float dx = gx - x.x, dy = gy - x.y, dz = gz - x.z;
        se += (double)((dx * dx + dy * dy) + dz * dz);
        ae += (double)((fabsf(dx) + fabsf(dy)) + fabsf(dz));
    }
    for (int o = 16; o > 0; o >>= 1) {
        se += __shfl_down_sync(0xffffffffu, se, o);
        ae += __shfl_down_sync(0xffffffffu, ae, o);
    }
    __shared__ double s_se[8], s_ae[8];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { s_se[warp] = se; s_ae[warp] = ae; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) { a += s_se[i]; b += s_ae[i]; }
        atomicAdd(&out[0], a);
        atomicAdd(&out[1], b);
    }
}

}  // namespace dev

void launch_sum64_add(const float4* frame, double* sum, uint32_t n, cudaStream_t s) {
    dev::sum64_add_kernel<<<list_blocks(n, 256, 8), 256, 0, s>>>(frame, sum, n);
}

void launch_error(const float4* img, const double* sum, double inv_count, uint32_t n, double* out, cudaStream_t s) {
    dev::error_kernel<<<list_blocks(n, 256, 4), 256, 0, s>>>(img, sum, inv_count, n, out);
}

}  // namespace vxr
