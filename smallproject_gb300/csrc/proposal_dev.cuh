// proposal_dev.cuh - device helpers shared by the learned-proposal kernels (proposal.cu,
// train.cu): the hash-grid encoding, the network input row, and the BF16 mma.sync
// fragment helpers (m16n8k16, row.col, FP32 accumulation). No reference counterpart.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "device.cuh"
#include "proposal.cuh"

namespace vxr {
namespace prop {

// ---- hash-grid encoding ------------------------------------------------------------------
__device__ __forceinline__ uint32_t grid_hash(uint32_t x, uint32_t y, uint32_t z, uint32_t mask) {
    return (x ^ (y * 2654435761u) ^ (z * 805459861u)) & mask;
}

struct Corner {
    uint32_t idx[kLevels][8];
    float w[kLevels][8];
};

// corner table indices and trilinear weights of point p (map coordinates) on both levels
__device__ __forceinline__ void corners(const Dims& d, float px, float py, float pz, Corner& c) {
    const uint32_t mask = (1u << d.tableLog2) - 1u;
#pragma unroll
    for (int l = 0; l < kLevels; l++) {
        const int R = l == 0 ? d.res0 : d.res1;
        const float s = (float)R * (1.0f / 1024.0f);
        const float ux = fminf(fmaxf(px * s, 0.0f), (float)R), uy = fminf(fmaxf(py * s, 0.0f), (float)R),
                    uz = fminf(fmaxf(pz * s, 0.0f), (float)R);
        const int ix = min((int)ux, R - 1), iy = min((int)uy, R - 1), iz = min((int)uz, R - 1);
        const float fx = ux - (float)ix, fy = uy - (float)iy, fz = uz - (float)iz;
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const int ox = q & 1, oy = (q >> 1) & 1, oz = q >> 2;
            c.idx[l][q] = (uint32_t)l * (mask + 1u) + grid_hash((uint32_t)(ix + ox), (uint32_t)(iy + oy), (uint32_t)(iz + oz), mask);
            c.w[l][q] = (ox ? fx : 1.0f - fx) * (oy ? fy : 1.0f - fy) * (oz ? fz : 1.0f - fz);
        }
    }
}

// network input row: 16 encoding features, one-hot side (6), zeros
__device__ __forceinline__ void input_row(const float* __restrict__ enc, const Dims& d, float4 pin, float* x) {
    Corner c;
    corners(d, pin.x, pin.y, pin.z, c);
#pragma unroll
    for (int l = 0; l < kLevels; l++) {
        float a[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const float4* e = reinterpret_cast<const float4*>(enc + (size_t)c.idx[l][q] * kFeat);
            const float4 e0 = __ldg(e), e1 = __ldg(e + 1);
            const float w = c.w[l][q];
            a[0] += w * e0.x; a[1] += w * e0.y; a[2] += w * e0.z; a[3] += w * e0.w;
            a[4] += w * e1.x; a[5] += w * e1.y; a[6] += w * e1.z; a[7] += w * e1.w;
        }
#pragma unroll
        for (int f = 0; f < 8; f++) x[l * 8 + f] = a[f];
    }
    const uint32_t code = __float_as_uint(pin.w);
#pragma unroll
    for (int s = 0; s < 6; s++) x[16 + s] = (code == (uint32_t)s) ? 1.0f : 0.0f;
#pragma unroll
    for (int s = 22; s < kIn; s++) x[s] = 0.0f;
}

// side code of a voxel face: axis * 2 + (normal points to negative axis)
__device__ __forceinline__ uint32_t side_code(uint32_t side, float nsign) { return side * 2u + (nsign < 0.0f ? 1u : 0u); }

// ---- tensor-core helpers (mma.sync m16n8k16, BF16 in, FP32 accumulate) ------------------
__device__ __forceinline__ void mma16816(float* c, const uint32_t* a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}

// one hidden layer on register fragments: out = relu(in * W^T + b); in/out are the A
// fragments of one m-tile (16 rows), H/16 k-tiles
template <int H>
__device__ __forceinline__ void hidden_layer(const uint32_t (&in)[H / 16][4], uint32_t (&out)[H / 16][4],
                                             const __nv_bfloat16* Ws, int ldw, const float* bs, int g, int t) {
    float c[H / 8][4];
#pragma unroll
    for (int nt = 0; nt < H / 8; nt++) {
        const float b0 = bs[nt * 8 + 2 * t], b1 = bs[nt * 8 + 2 * t + 1];
        c[nt][0] = b0; c[nt][1] = b1; c[nt][2] = b0; c[nt][3] = b1;
    }
#pragma unroll
    for (int kt = 0; kt < H / 16; kt++) {
#pragma unroll
        for (int nt = 0; nt < H / 8; nt++) {
            const __nv_bfloat16* row = Ws + (size_t)(nt * 8 + g) * ldw + kt * 16 + 2 * t;
            mma16816(c[nt], in[kt], *reinterpret_cast<const uint32_t*>(row), *reinterpret_cast<const uint32_t*>(row + 8));
        }
    }
#pragma unroll
    for (int kt = 0; kt < H / 16; kt++) {
        out[kt][0] = pack_bf16(fmaxf(c[2 * kt][0], 0.f), fmaxf(c[2 * kt][1], 0.f));
        out[kt][1] = pack_bf16(fmaxf(c[2 * kt][2], 0.f), fmaxf(c[2 * kt][3], 0.f));
        out[kt][2] = pack_bf16(fmaxf(c[2 * kt + 1][0], 0.f), fmaxf(c[2 * kt + 1][1], 0.f));
        out[kt][3] = pack_bf16(fmaxf(c[2 * kt + 1][2], 0.f), fmaxf(c[2 * kt + 1][3], 0.f));
    }
}

// the 8 hash-grid features of one level at point p (trilinear over the cell's corners)
__device__ __forceinline__ void level_features(const float* __restrict__ enc, const Dims& d, float px, float py, float pz,
                                               int l, float* a) {
    const uint32_t mask = (1u << d.tableLog2) - 1u;
    const int R = l == 0 ? d.res0 : d.res1;
    const float s = (float)R * (1.0f / 1024.0f);
    const float ux = fminf(fmaxf(px * s, 0.0f), (float)R), uy = fminf(fmaxf(py * s, 0.0f), (float)R),
                uz = fminf(fmaxf(pz * s, 0.0f), (float)R);
    const int ix = min((int)ux, R - 1), iy = min((int)uy, R - 1), iz = min((int)uz, R - 1);
    const float fx = ux - (float)ix, fy = uy - (float)iy, fz = uz - (float)iz;
#pragma unroll
    for (int f = 0; f < 8; f++) a[f] = 0.0f;
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const int ox = q & 1, oy = (q >> 1) & 1, oz = q >> 2;
        const uint32_t idx = (uint32_t)l * (mask + 1u) + grid_hash((uint32_t)(ix + ox), (uint32_t)(iy + oy), (uint32_t)(iz + oz), mask);
        const float w = (ox ? fx : 1.0f - fx) * (oy ? fy : 1.0f - fy) * (oz ? fz : 1.0f - fz);
        const float4* e = reinterpret_cast<const float4*>(enc + (size_t)idx * kFeat);
        const float4 e0 = __ldg(e), e1 = __ldg(e + 1);
        a[0] += w * e0.x; a[1] += w * e0.y; a[2] += w * e0.z; a[3] += w * e0.w;
        a[4] += w * e1.x; a[5] += w * e1.y; a[6] += w * e1.z; a[7] += w * e1.w;
    }
}

}  // namespace prop
}  // namespace vxr
