// kernels.cu - the five per-frame stage kernels of Voxel ReSTIR on sm_103a, plus the
// one-time world kernels (uber grid, light table).
//
// One thread per pixel on 2D tiles. Memory layout in HBM (per view):
//   G-buffer   vd[2]  uint2  (voxel | side << 24, bits(dist))   current / previous frame
//              seed   uint32 per-pixel xorshift32 state
//   reservoirs C, H   uint4 + float4 planes (see Res in device.cuh), 32 B/pixel each:
//              C = candidate+temporal output, H = spatial output = temporal history
//   frame      float4 (rgb, dist); accum float4 (running mean, the output image)
// The reference cycles two 80-byte reservoir buffers through three roles per frame
// (world.cpp:2209-2219) and copies the shaded reservoir at the end of shading
// (ris.cl:412). Here the spatial pass writes H in place of the previous history,
// which the candidate pass has finished reading, and shading patches H on a failed
// visibility test; H is then next frame's history without any copy.
#include <cstdint>
#include <cuda_runtime.h>

#include "device.cuh"
#include "kernels.hpp"

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

// ---- stage 1: primary rays / G-buffer (renderAlbedo, ris.cl:295-389) --------------------
__global__ void __launch_bounds__(128) albedo_kernel(World w, Frame k, uint2* __restrict__ vd, uint32_t* __restrict__ seeds) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= k.W || y >= k.H) return;
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

// ---- visibility (isLightOccluded, ris.cl:1-17) ---------------------------------------
// Shadow ray with the reference's budget of GRIDWIDTH (128) steps; a miss leaves
// dist/side at 0 (the oracle's fixed convention for the reference's uninitialised
// locals); visible iff the hit voxel lies in the emitter cube [pos, pos + size).
__device__ __forceinline__ bool occluded(const World& w, float4 geom, float4 em, float3 o, float3 L) {
    float d2 = 0.0f;
    uint32_t s2 = 0;
    trace<1>(w, o.x, o.y, o.z, L.x, L.y, L.z, 128, 0u, 0u, &d2, &s2);
    const float ns = side_sign(s2, L);
    const float hx = L.x * d2 + o.x, hy = L.y * d2 + o.y, hz = L.z * d2 + o.z;
    const uint32_t vx = f2u(hx - (s2 == 0 ? ns * 0.1f : 0.0f));
    const uint32_t vy = f2u(hy - (s2 == 1 ? ns * 0.1f : 0.0f));
    const uint32_t vz = f2u(hz - (s2 == 2 ? ns * 0.1f : 0.0f));
    const uint32_t pos = __float_as_uint(em.w);
    const uint32_t ey = pos / (1024u * 1024u), ez = (pos / 1024u) % 1024u, ex = pos % 1024u;
    const uint32_t size = (uint32_t)geom.w;
    const bool inside = ex <= vx && ex + size > vx && ey <= vy && ey + size > vy && ez <= vz && ez + size > vz;
    return !inside;
}

// Area-light sample (RandomPointOnVoxel, tools.cl:499-577): one random point per face
// (2 draws each, all six faces always drawn), faces weighted by their solid angle,
// CDF pick with one more draw, weight = 1/pdf. Only faces whose normal points toward
// the shading point get a non-zero solid angle, so only those are normalised.
__device__ __forceinline__ float3 face_point(float4 g, uint32_t face, float r0, float r1) {
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

__device__ __forceinline__ float3 sample_area_light(float4 g, float3 spo, uint32_t& seed, float* invp, uint32_t* ncode) {
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
            const float3 P = face_point(g, f, r0, r1);
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
    return face_point(g, index, r0, r1);
}

// ---- stage 2: candidates + visibility + temporal (perPixelInitialSampling, ris.cl:20-124) ----
template <bool POINT>
__global__ void __launch_bounds__(128) candidates_kernel(World w, Frame k, const uint2* __restrict__ vd,
                                                         const uint2* __restrict__ vdPrev, uint32_t* __restrict__ seeds,
                                                         const uint4* __restrict__ hA, const float4* __restrict__ hB,
                                                         uint4* __restrict__ cA, float4* __restrict__ cB, uint32_t* err) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= k.W || y >= k.H) return;
    const size_t i = (size_t)y * k.W + x;
    const uint2 g = vd[i];
    const uint32_t voxel = g.x & 0x00FFFFFFu, side = g.x >> 24;
    const float dist = __uint_as_float(g.y);
    Res res = res_zero();
    if (voxel != 0u) {
        uint32_t seed = seeds[i];
        const float3 D = camera_ray(k, x, y);
        const float nsign = side_sign(side, D);
        const float3 brdf = mul(to_rgb(voxel), 0.31830988618379067153777f);
        const float3 sp = f3(D.x * dist + k.E.x, D.y * dist + k.E.y, D.z * dist + k.E.z);
        const float3 spo = f3(sp.x + (side == 0 ? 0.1f * nsign : 0.0f), sp.y + (side == 1 ? 0.1f * nsign : 0.0f),
                              sp.z + (side == 2 ? 0.1f * nsign : 0.0f));
        const uint32_t nL = k.nlights;
        const float p = 1.0f / (float)nL;
        for (uint32_t c = 0; c < k.ncand; c++) {
            // GenerateLightCandidate (tools.cl:593-598)
            const int li = min(max(f2i(rnd(seed) * (float)nL), 0), (int)nL - 1);
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
            res_update(res, ph / p, ph, (uint32_t)li, rnd(seed), pos, inv, nc);
        }
        // AdjustWeight with the selected pHat; visibility of the selected sample
        if (k.ncand > 0) {
            const uint32_t li = res.idx;
            const float4 lg = __ldg(w.lgeom + li), le = __ldg(w.lemit + li);
            const float3 L = normalize3(sub(res.pos, spo));
            if (occluded(w, lg, le, spo, L)) res.sumW = 0.0f;   // W = 0 follows from sumW = 0
        }
        // temporal reuse (ris.cl:84-119)
        if (k.restirtemporalframe > 0 && k.temporal) {
            const float dl = ((sp.x * k.Nl.x + sp.y * k.Nl.y) + sp.z * k.Nl.z) - k.Nl.w;
            const float dr = ((sp.x * k.Nr.x + sp.y * k.Nr.y) + sp.z * k.Nr.z) - k.Nr.w;
            const float dt = ((sp.x * k.Nt.x + sp.y * k.Nt.y) + sp.z * k.Nt.z) - k.Nt.w;
            const float db = ((sp.x * k.Nb.x + sp.y * k.Nb.y) + sp.z * k.Nb.z) - k.Nb.w;
            const float up = (float)k.W * (dl / (dl + dr));
            const float vp = (float)k.H * (dt / (dt + db));
            const float ru = roundf(up), rv = roundf(vp);
            if (ru == ru && rv == rv) {
                const int px = f2i(ru), py = f2i(rv);
                if (px >= 0 && py >= 0 && px < k.W && py < k.H) {
                    const size_t j = (size_t)py * k.W + px;
                    const uint2 pg = __ldg(vdPrev + j);
                    const uint32_t pside = pg.x >> 24;
                    const float pdist = __uint_as_float(pg.y);
                    if (pside == side && fabsf(dist - pdist) <= 0.1f * dist) {
                        Res prev = res_load(hA, hB, j);
                        const uint32_t pm = min(k.maxTemporal * k.ncand, prev.M);
                        if (pm > 0u) {
                            uint32_t pli = prev.idx;
                            if (pli >= nL) { raise_error(err, 2u); pli = 0; }
                            const float4 pg4 = __ldg(w.lgeom + pli), pe4 = __ldg(w.lemit + pli);
                            const float pph = phat<POINT>(prev.pos, prev.ncode, sp, side, nsign, brdf, pe4, pg4.w) * prev.inv;
                            const float W = res_W(prev);
                            res_reweigh(prev, W, pph, pm);
                            res_combine(res, prev, rnd(seed));
                            // AdjustWeight(res, pHat of the selected sample here) equals res.pHat
                        }
                    }
                }
            }
        }
        seeds[i] = seed;
    }
    res_store(cA, cB, i, res);
}

// ---- stage 3: spatial reuse (perPixelSpatialResampling, ris.cl:126-151,
//      spatialSampling.cl:2-66) -------------------------------------------------------

template <bool POINT>
__global__ void __launch_bounds__(128) spatial_kernel(World w, Frame k, const uint2* __restrict__ vd,
                                                      uint32_t* __restrict__ seeds, const uint4* __restrict__ cA,
                                                      const float4* __restrict__ cB, uint4* __restrict__ hA,
                                                      float4* __restrict__ hB, uint32_t* err) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= k.W || y >= k.H) return;
    const size_t i = (size_t)y * k.W + x;
    Res res = res_load(cA, cB, i);
    const uint2 g = vd[i];
    const uint32_t voxel = g.x & 0x00FFFFFFu;
    if (voxel != 0u && k.spatial) {
        const uint32_t side = g.x >> 24;
        const float dist = __uint_as_float(g.y);
        uint32_t seed = seeds[i];
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
            if (nb.M > 0u) {
                const uint2 ng = __ldg(vd + j);
                const float ndist = __uint_as_float(ng.y);
                if ((ng.x >> 24) == side && fabsf(dist - ndist) <= 0.1f * dist) {
                    uint32_t nli = nb.idx;
                    if (nli >= k.nlights) { raise_error(err, 4u); nli = 0; }
                    const float4 lg = __ldg(w.lgeom + nli), le = __ldg(w.lemit + nli);
                    const float ph = phat<POINT>(nb.pos, nb.ncode, sp, side, nsign, brdf, le, lg.w) * nb.inv;
                    const float W = res_W(nb);
                    res_reweigh(nb, W, ph, nb.M);
                    res_combine(res, nb, rnd(seed));
                }
            }
        }
        // AdjustWeight(res, res.pHat): implied by the stored (sumW, pHat, M)
        seeds[i] = seed;
    }
    res_store(hA, hB, i, res);
}

// ---- stage 4+5: shading (renderRIS / render_di_ris, ris.cl:155-293, 391-413) fused with
//      accumulation (accumulatorFinalizer, kernels.cl:304-326) -----------------------------
template <bool POINT>
__global__ void __launch_bounds__(128) shade_kernel(World w, Frame k, const uint2* __restrict__ vd,
                                                    uint4* __restrict__ hA, const float4* __restrict__ hB,
                                                    float4* __restrict__ frame, float4* __restrict__ accum,
                                                    int fuse_accumulate, uint32_t* err) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= k.W || y >= k.H) return;
    const size_t i = (size_t)y * k.W + x;
    const uint2 g = vd[i];
    const uint32_t voxel = g.x & 0x00FFFFFFu;
    const float dist = __uint_as_float(g.y);
    float3 color = f3(0.0f, 0.0f, 0.0f);
    if (voxel != 0u) {
        const float INVPI = 0.31830988618379067153777f;
        if (emitter(voxel)) {
            const float3 c = to_rgb(voxel);
            const float m = strength(voxel);
            color = add(color, f3((c.x * m) * INVPI, (c.y * m) * INVPI, (c.z * m) * INVPI));
        }
        const uint4 qa = hA[i];
        const float sumW = __uint_as_float(qa.z), pH = __uint_as_float(qa.w);
        const uint32_t M = qa.y & 0x1FFFFFFFu;
        const float W = sumW / fmaxf(1e-5f, pH * (float)M);
        if (W > 0.0f && M > 0u) {
            const uint32_t side = g.x >> 24;
            const float4 qb = __ldg(hB + i);
            const float3 D = camera_ray(k, x, y);
            const float nsign = side_sign(side, D);
            const float3 sp = f3(D.x * dist + k.E.x, D.y * dist + k.E.y, D.z * dist + k.E.z);
            const float3 spo = f3(sp.x + (side == 0 ? 0.1f * nsign : 0.0f), sp.y + (side == 1 ? 0.1f * nsign : 0.0f),
                                  sp.z + (side == 2 ? 0.1f * nsign : 0.0f));
            uint32_t li = qa.x;
            if (li >= k.nlights) { raise_error(err, 8u); li = 0; }
            const float4 lg = __ldg(w.lgeom + li), le = __ldg(w.lemit + li);
            const float3 pos = f3(qb.x, qb.y, qb.z);
            const float3 L = normalize3(sub(pos, spo));
            if (!occluded(w, lg, le, spo, L)) {
                const float3 brdf = mul(to_rgb(voxel), INVPI);
                bool zero;
                const float3 inc = phat_full<POINT>(pos, qa.y >> 29, sp, side, nsign, brdf, le, lg.w, &zero);
                color = add(color, f3((inc.x * W) * qb.w, (inc.y * W) * qb.w, (inc.z * W) * qb.w));
            } else {
                // discard: W = sumOfWeights = 0 written back into the history
                hA[i] = make_uint4(qa.x, qa.y, 0u, qa.w);
            }
        }
        const float a = alphaf(voxel);
        color = f3(color.x + ((a * color.x) + ((1.0f - a) * 0.0f)), color.y + ((a * color.y) + ((1.0f - a) * 0.0f)),
                   color.z + ((a * color.z) + ((1.0f - a) * 0.0f)));
    }
    const float4 px = make_float4(color.x, color.y, color.z, dist);
    frame[i] = px;
    if (fuse_accumulate) {
        const int n = (int)k.framecount * k.accumulate;
        float4 prev = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (n > 0) prev = accum[i];
        const float cw = 1.0f / (float)(1 + n);
        accum[i] = make_float4((1.0f - cw) * prev.x + cw * px.x, (1.0f - cw) * prev.y + cw * px.y,
                               (1.0f - cw) * prev.z + cw * px.z, 1.0f);
    }
}

// stage 5 on its own (accumulatorFinalizer, kernels.cl:304-326)
__global__ void __launch_bounds__(256) accumulate_kernel(Frame k, const float4* __restrict__ frame, float4* __restrict__ accum) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= k.W || y >= k.H) return;
    const size_t i = (size_t)y * k.W + x;
    const float4 px = frame[i];
    const int n = (int)k.framecount * k.accumulate;
    float4 prev = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (n > 0) prev = accum[i];
    const float cw = 1.0f / (float)(1 + n);
    accum[i] = make_float4((1.0f - cw) * prev.x + cw * px.x, (1.0f - cw) * prev.y + cw * px.y,
                           (1.0f - cw) * prev.z + cw * px.z, 1.0f);
}

}  // namespace dev
}  // namespace vxr

// ---- launchers -------------------------------------------------------------------------
namespace vxr {

static dim3 grid_for(const dev::Frame& k, LaunchShape sh) {
    return dim3((unsigned)((k.W + sh.bx - 1) / sh.bx), (unsigned)((k.H + sh.by - 1) / sh.by), 1);
}

void launch_build_light_table(const uint4* raw, uint32_t n, float4* geom, float4* emit, cudaStream_t s) {
    if (n == 0) return;
    dev::build_light_table_kernel<<<(n + 255) / 256, 256, 0, s>>>(raw, n, geom, emit);
}

void launch_build_uber(const uint32_t* grid, uint8_t* uber, cudaStream_t s) {
    dev::build_uber_kernel<<<(32 * 32 * 32 + 255) / 256, 256, 0, s>>>(grid, uber);
}

void launch_albedo(const dev::World& w, const dev::Frame& k, const ViewBuffers& b, int cur, LaunchShape sh, cudaStream_t s) {
    dev::albedo_kernel<<<grid_for(k, sh), dim3(sh.bx, sh.by), 0, s>>>(w, k, b.vd[cur], b.seed);
}

void launch_candidates(bool point, const dev::World& w, const dev::Frame& k, const ViewBuffers& b, int cur, LaunchShape sh,
                       cudaStream_t s) {
    if (point)
        dev::candidates_kernel<true><<<grid_for(k, sh), dim3(sh.bx, sh.by), 0, s>>>(w, k, b.vd[cur], b.vd[cur ^ 1], b.seed,
                                                                                  b.hA, b.hB, b.cA, b.cB, b.err);
    else
        dev::candidates_kernel<false><<<grid_for(k, sh), dim3(sh.bx, sh.by), 0, s>>>(w, k, b.vd[cur], b.vd[cur ^ 1], b.seed,
                                                                                   b.hA, b.hB, b.cA, b.cB, b.err);
}

void launch_spatial(bool point, const dev::World& w, const dev::Frame& k, const ViewBuffers& b, int cur, LaunchShape sh,
                    cudaStream_t s) {
    if (point)
        dev::spatial_kernel<true><<<grid_for(k, sh), dim3(sh.bx, sh.by), 0, s>>>(w, k, b.vd[cur], b.seed, b.cA, b.cB, b.hA,
                                                                               b.hB, b.err);
    else
        dev::spatial_kernel<false><<<grid_for(k, sh), dim3(sh.bx, sh.by), 0, s>>>(w, k, b.vd[cur], b.seed, b.cA, b.cB, b.hA,
                                                                                b.hB, b.err);
}

void launch_shade(bool point, const dev::World& w, const dev::Frame& k, const ViewBuffers& b, int cur, bool fuse_accumulate,
                  LaunchShape sh, cudaStream_t s) {
    if (point)
        dev::shade_kernel<true><<<grid_for(k, sh), dim3(sh.bx, sh.by), 0, s>>>(w, k, b.vd[cur], b.hA, b.hB, b.frame, b.accum,
                                                                             fuse_accumulate ? 1 : 0, b.err);
    else
        dev::shade_kernel<false><<<grid_for(k, sh), dim3(sh.bx, sh.by), 0, s>>>(w, k, b.vd[cur], b.hA, b.hB, b.frame,
                                                                              b.accum, fuse_accumulate ? 1 : 0, b.err);
}

void launch_accumulate(const dev::Frame& k, const ViewBuffers& b, LaunchShape sh, cudaStream_t s) {
    dev::accumulate_kernel<<<grid_for(k, sh), dim3(sh.bx, sh.by), 0, s>>>(k, b.frame, b.accum);
}

}  // namespace vxr
