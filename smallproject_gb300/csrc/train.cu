// train.cu - one online training step of the learned proposal on the tensor cores
// (no reference counterpart; the proposal replaces the uniform source pdf of
// GenerateLightCandidate, tools.cl:593-598).
//
// The step minimises the weighted softmax cross-entropy of proposal.cuh over a batch of
// reservoir samples (position, voxel side, target cluster, weight W * pHat), with Adam on
// an FP32 master copy of the parameters. Tensor-core operands are BF16 and every product
// accumulates in FP32 (mma.sync.m16n8k16).
//
// Launches per step:
//   wsum_kernel          - the batch's weight sum as fixed per-block partial sums
//   train_kernel         - per warp, 16 samples at a time: hash-grid encoding, forward
//                          through the three hidden layers, the K logits twice (softmax
//                          statistics, then probabilities) and the backward pass through
//                          the layers to the network input, whose gradient goes straight
//                          to the hash tables (vector atomics). For the weight gradients
//                          dW = dY^T X it stores the operands, transposed in registers
//                          (movmatrix), as ready-made mma fragments: one 512-byte block per
//                          16 x 16 tile, lane-major, so every store and load is a
//                          coalesced 16-byte access.
//   wgrad_kernel         - the weight and bias gradients from those fragments: a CTA per
//                          (chunk of 16-sample tiles, 16 output rows of one layer), split-K
//                          over its warps, FP32 register accumulators, the warps' sums
//                          added in a fixed order, one row of a partial-gradient table per
//                          chunk (no atomics)
//   train_reduce_kernel  - sums the chunk rows, Adam on the MLP parameters, BF16 copies for
//                          the inference kernels
//   adam_enc_kernel      - Adam on the hash tables, clearing their gradient for the next step
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdint>

#include "proposal.hpp"
#include "proposal_dev.cuh"

namespace vxr {
namespace prop {

namespace {

constexpr int kTW = 8;          // warps per CTA
constexpr int kTrainCtasPerSm = 1;   // train_kernel: one CTA per SM (two, capped at 128 registers, spill and run slower)
constexpr int kTH = 64;         // hidden width handled by the fused step
constexpr int kLd1 = kIn + 8;   // padded row of W1 and X in shared memory (BF16 elements)
constexpr int kLdh = kTH + 8;   // padded row of W2, W3, W4 and H1
constexpr int kWsumBlocks = 256;
constexpr uint32_t kChunkTiles = 64;   // 16-sample tiles per row of the partial-gradient table

__device__ __forceinline__ uint32_t movT(uint32_t a) {
    uint32_t d;
    asm volatile("movmatrix.sync.aligned.m8n8.trans.b16 %0, %1;\n" : "=r"(d) : "r"(a));
    return d;
}

// four 8x8 BF16 matrices from shared memory, transposed (the B fragments of a row-major
// [k][n] operand)
__device__ __forceinline__ void ldsm4t(uint32_t (&r)[4], const __nv_bfloat16* p) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

__device__ __forceinline__ float keep_lo(uint32_t act, float x) { return (act & 0xFFFFu) ? x : 0.0f; }
__device__ __forceinline__ float keep_hi(uint32_t act, float x) { return (act >> 16) ? x : 0.0f; }

// online softmax statistics: running maximum m and sum s of exp(z - m)
__device__ __forceinline__ void online(float& m, float& s, float x, float y) {
    const float mn = fmaxf(m, fmaxf(x, y));
    s = s * __expf(m - mn) + __expf(x - mn) + __expf(y - mn);
    m = mn;
}
__device__ __forceinline__ void merge_quad(float& m, float& s) {
#pragma unroll
    for (int o = 1; o <= 2; o <<= 1) {
        const float mo = __shfl_xor_sync(0xffffffffu, m, o), so = __shfl_xor_sync(0xffffffffu, s, o);
        const float mn = fmaxf(m, mo);
        s = s * __expf(m - mn) + so * __expf(mo - mn);
        m = mn;
    }
}

// Fragment blocks of the weight-gradient operands, per 16-sample tile: A operands are
// dY^T (16 output rows x 16 samples), B operands X^T as pairs of 8-column n-tiles.
// Regions: 0 dZ^T (K/16 blocks), 1 H3 (4), 2 dH3^T (4), 3 H2 (4), 4 dH2^T (4), 5 H1 (4),
// 6 dH1^T (4), 7 X (2); region r holds ntiles * count(r) blocks of 32 uint4.
__host__ __device__ __forceinline__ int frag_count(int region, int kt4) {
    return region == 0 ? kt4 : (region == 7 ? 2 : 4);
}
// (frag_prefix(8, kt4): blocks per tile)
__host__ __device__ __forceinline__ int frag_prefix(int region, int kt4) {
    return region == 0 ? 0 : kt4 + 4 * (region - 1) - (region == 8 ? 2 : 0);
}
__device__ __forceinline__ size_t frag_at(int region, uint32_t tile, int j, uint32_t ntiles, int kt4) {
    return ((size_t)ntiles * frag_prefix(region, kt4) + (size_t)tile * frag_count(region, kt4) + j) * 32;
}

// the A fragment of dY^T for the 16 outputs of dya (rows = samples)
__device__ __forceinline__ uint4 dyt(const uint32_t (&dya)[4]) {
    return make_uint4(movT(dya[0]), movT(dya[2]), movT(dya[1]), movT(dya[3]));
}

// dIn = dOut W for W [out][in] row-major in shared memory (leading dimension ld): KT
// k-tiles of 16 outputs, NT n-tiles of 8 inputs (NT even)
template <int KT, int NT>
__device__ __forceinline__ void dgrad(const uint32_t (&dya)[KT][4], const __nv_bfloat16* Ws, int ld, float (&c)[NT][4],
                                      int lane) {
#pragma unroll
    for (int nt = 0; nt < NT; nt++) c[nt][0] = c[nt][1] = c[nt][2] = c[nt][3] = 0.0f;
    const int q = lane >> 3, rr = lane & 7;
#pragma unroll
    for (int kt = 0; kt < KT; kt++)
#pragma unroll
        for (int np = 0; np < NT / 2; np++) {
            uint32_t b[4];
            ldsm4t(b, Ws + (kt * 16 + (q & 1) * 8 + rr) * ld + (2 * np + (q >> 1)) * 8);
            mma16816(c[2 * np], dya[kt], b[0], b[1]);
            mma16816(c[2 * np + 1], dya[kt], b[2], b[3]);
        }
}

// ReLU backward: dH = dA * (H > 0) as A fragments
__device__ __forceinline__ void relu_back(const float (&c)[8][4], const uint32_t (&act)[4][4], uint32_t (&out)[4][4]) {
#pragma unroll
    for (int kt = 0; kt < 4; kt++)
#pragma unroll
        for (int hh = 0; hh < 2; hh++) {
            const int nt = 2 * kt + hh;
            const uint32_t top = act[kt][2 * hh], bot = act[kt][2 * hh + 1];
            out[kt][2 * hh] = pack_bf16(keep_lo(top, c[nt][0]), keep_hi(top, c[nt][1]));
            out[kt][2 * hh + 1] = pack_bf16(keep_lo(bot, c[nt][2]), keep_hi(bot, c[nt][3]));
        }
}

// store the B fragments (X^T pairs of n-tiles) of an activation held as A fragments
template <int KT>
__device__ __forceinline__ void store_xt(uint4* frag, int region, uint32_t tile, uint32_t ntiles, int kt4,
                                         const uint32_t (&act)[KT][4], int lane) {
#pragma unroll
    for (int kt = 0; kt < KT; kt++)
        frag[frag_at(region, tile, kt, ntiles, kt4) + lane] =
            make_uint4(movT(act[kt][0]), movT(act[kt][1]), movT(act[kt][2]), movT(act[kt][3]));
}

// logits of the n-tile nt (8 clusters) for the warp's 16 samples
__device__ __forceinline__ void logits_tile(float (&c)[4], const uint32_t (&h3)[4][4], const __nv_bfloat16* W4s,
                                            const float* b4, int nt, int g, int t) {
    const float b0 = b4[nt * 8 + 2 * t], b1 = b4[nt * 8 + 2 * t + 1];
    c[0] = b0; c[1] = b1; c[2] = b0; c[3] = b1;
#pragma unroll
    for (int kt = 0; kt < 4; kt++) {
        const __nv_bfloat16* row = W4s + (nt * 8 + g) * kLdh + kt * 16 + 2 * t;
        mma16816(c, h3[kt], *reinterpret_cast<const uint32_t*>(row), *reinterpret_cast<const uint32_t*>(row + 8));
    }
}

__global__ void wsum_kernel(const float* __restrict__ w, uint32_t B, float* __restrict__ part) {
    __shared__ float ws[8];
    float s = 0.0f;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < B; i += gridDim.x * blockDim.x) s += w[i];
#pragma unroll
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.0f;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) t += ws[k];
        part[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(kTW * 32, kTrainCtasPerSm) train_kernel(TrainArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ float s_inv;
    __shared__ float s_loss[kTW];
    const Dims d = a.dims;
    const int K = d.K, kt4 = K / 16;
    __nv_bfloat16* W1s = reinterpret_cast<__nv_bfloat16*>(smem);   // [64][40]
    __nv_bfloat16* W2s = W1s + kTH * kLd1;                           // [64][72]
    __nv_bfloat16* W3s = W2s + kTH * kLdh;
    __nv_bfloat16* W4s = W3s + kTH * kLdh;                           // [K][72]
    float* bs = reinterpret_cast<float*>(W4s + K * kLdh);            // b1 | b2 | b3 | b4
    unsigned char* wbase = reinterpret_cast<unsigned char*>(bs + 3 * kTH + K);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int r = lane & 15, half = lane >> 4;
    __nv_bfloat16* Xs = reinterpret_cast<__nv_bfloat16*>(wbase + warp * kTrainWarpBytes);   // [16][40]
    __nv_bfloat16* H1s = Xs + 16 * kLd1;                                                   // [16][72]
    float* dxs = reinterpret_cast<float*>(H1s + 16 * kLdh);                                // [16][16]
    {
        const __nv_bfloat16* wg = a.wbf;   // W1 [64][32] | W2 [64][64] | W3 [64][64] | W4 [K][64]
        for (int e = threadIdx.x; e < kTH * kIn; e += blockDim.x) W1s[(e / kIn) * kLd1 + e % kIn] = wg[e];
        wg += kTH * kIn;
        for (int e = threadIdx.x; e < kTH * kTH; e += blockDim.x) W2s[(e / kTH) * kLdh + e % kTH] = wg[e];
        wg += kTH * kTH;
        for (int e = threadIdx.x; e < kTH * kTH; e += blockDim.x) W3s[(e / kTH) * kLdh + e % kTH] = wg[e];
        wg += kTH * kTH;
        for (int e = threadIdx.x; e < K * kTH; e += blockDim.x) W4s[(e / kTH) * kLdh + e % kTH] = wg[e];
        const float* p = a.params;
        for (int e = threadIdx.x; e < kTH; e += blockDim.x) {
            bs[e] = p[a.L.b1 + e];
            bs[kTH + e] = p[a.L.b2 + e];
            bs[2 * kTH + e] = p[a.L.b3 + e];
        }
        for (int e = threadIdx.x; e < K; e += blockDim.x) bs[3 * kTH + e] = p[a.L.b4 + e];
        if (warp == 0) {
            // the batch's weight sum from the fixed partials, in the same order in every CTA
            float s = 0.0f;
            for (uint32_t i = lane; i < a.nwpart; i += 32) s += a.wpart[i];
#pragma unroll
            for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) s_inv = s > 0.0f ? 1.0f / s : 0.0f;
        }
    }
    __syncthreads();
    const float inv = s_inv;
    const float* enc = a.params + a.L.enc;
    float* encGrad = a.grads + a.L.enc;
    const uint32_t mask = (1u << d.tableLog2) - 1u;
    const uint32_t ntiles = (a.B + 15u) / 16u;
    uint4* frag = a.frag;
    float lossAcc = 0.0f;
    for (uint32_t tile = blockIdx.x * kTW + warp; tile < ntiles; tile += gridDim.x * kTW) {
        const uint32_t base = tile * 16u;
        // ---- input rows: lane (r, half) encodes level `half` of sample r
        const uint32_t j = base + (uint32_t)r;
        const bool valid = j < a.B;
        const float4 pin = valid ? a.samples[j] : make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(6u));
        {
            float f[8];
            level_features(enc, d, pin.x, pin.y, pin.z, half, f);
            __nv_bfloat16* xr = Xs + r * kLd1;
#pragma unroll
            for (int q = 0; q < 8; q += 2)
                *reinterpret_cast<uint32_t*>(xr + half * 8 + q) = valid ? pack_bf16(f[q], f[q + 1]) : 0u;
            if (half == 0) {
                const uint32_t code = __float_as_uint(pin.w);
#pragma unroll
                for (int q = 16; q < kIn; q += 2)
                    *reinterpret_cast<uint32_t*>(xr + q) =
                        valid ? pack_bf16(code == (uint32_t)(q - 16) ? 1.f : 0.f, code == (uint32_t)(q - 15) ? 1.f : 0.f)
                              : 0u;
            }
        }
        const uint32_t j0 = base + (uint32_t)g, j1 = j0 + 8u;
        const float w0 = j0 < a.B ? a.weight[j0] * inv : 0.0f;
        const float w1 = j1 < a.B ? a.weight[j1] * inv : 0.0f;
        const int t0 = j0 < a.B ? (int)a.target[j0] : -1;
        const int t1 = j1 < a.B ? (int)a.target[j1] : -1;
        __syncwarp();
        // ---- forward
        uint32_t xa[2][4];
#pragma unroll
        for (int kt = 0; kt < 2; kt++) {
            const __nv_bfloat16* r0 = Xs + g * kLd1 + kt * 16 + 2 * t;
            const __nv_bfloat16* r1 = r0 + 8 * kLd1;
            xa[kt][0] = *reinterpret_cast<const uint32_t*>(r0);
            xa[kt][1] = *reinterpret_cast<const uint32_t*>(r1);
            xa[kt][2] = *reinterpret_cast<const uint32_t*>(r0 + 8);
            xa[kt][3] = *reinterpret_cast<const uint32_t*>(r1 + 8);
        }
        store_xt<2>(frag, 7, tile, ntiles, kt4, xa, lane);
        uint32_t h1[4][4], h2[4][4], h3[4][4];
        {
            float c[8][4];
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                const float b0 = bs[nt * 8 + 2 * t], b1 = bs[nt * 8 + 2 * t + 1];
                c[nt][0] = b0; c[nt][1] = b1; c[nt][2] = b0; c[nt][3] = b1;
            }
#pragma unroll
            for (int kt = 0; kt < 2; kt++)
#pragma unroll
                for (int nt = 0; nt < 8; nt++) {
                    const __nv_bfloat16* row = W1s + (nt * 8 + g) * kLd1 + kt * 16 + 2 * t;
                    mma16816(c[nt], xa[kt], *reinterpret_cast<const uint32_t*>(row),
                             *reinterpret_cast<const uint32_t*>(row + 8));
                }
#pragma unroll
            for (int kt = 0; kt < 4; kt++) {
                h1[kt][0] = pack_bf16(fmaxf(c[2 * kt][0], 0.f), fmaxf(c[2 * kt][1], 0.f));
                h1[kt][1] = pack_bf16(fmaxf(c[2 * kt][2], 0.f), fmaxf(c[2 * kt][3], 0.f));
                h1[kt][2] = pack_bf16(fmaxf(c[2 * kt + 1][0], 0.f), fmaxf(c[2 * kt + 1][1], 0.f));
                h1[kt][3] = pack_bf16(fmaxf(c[2 * kt + 1][2], 0.f), fmaxf(c[2 * kt + 1][3], 0.f));
            }
        }
        hidden_layer<kTH>(h1, h2, W2s, kLdh, bs + kTH, g, t);
        store_xt<4>(frag, 5, tile, ntiles, kt4, h1, lane);
        hidden_layer<kTH>(h2, h3, W3s, kLdh, bs + 2 * kTH, g, t);
        store_xt<4>(frag, 3, tile, ntiles, kt4, h2, lane);
        store_xt<4>(frag, 1, tile, ntiles, kt4, h3, lane);
        // H1 waits in shared memory for its ReLU mask in the layer-2 backward pass
#pragma unroll
        for (int kt = 0; kt < 4; kt++) {
            __nv_bfloat16* r0 = H1s + g * kLdh + kt * 16 + 2 * t;
            *reinterpret_cast<uint32_t*>(r0) = h1[kt][0];
            *reinterpret_cast<uint32_t*>(r0 + 8 * kLdh) = h1[kt][1];
            *reinterpret_cast<uint32_t*>(r0 + 8) = h1[kt][2];
            *reinterpret_cast<uint32_t*>(r0 + 8 * kLdh + 8) = h1[kt][3];
        }
        // ---- softmax statistics of rows g (m0, s0) and g + 8 (m1, s1), target logits
        const float* b4 = bs + 3 * kTH;
        float m0 = -INFINITY, s0 = 0.0f, m1 = -INFINITY, s1 = 0.0f, z0 = 0.0f, z1 = 0.0f;
        for (int nt = 0; nt < K / 8; nt++) {
            float c[4];
            logits_tile(c, h3, W4s, b4, nt, g, t);
            online(m0, s0, c[0], c[1]);
            online(m1, s1, c[2], c[3]);
            const int col = nt * 8 + 2 * t;
            if (t0 == col) z0 = c[0];
            if (t0 == col + 1) z0 = c[1];
            if (t1 == col) z1 = c[2];
            if (t1 == col + 1) z1 = c[3];
        }
        merge_quad(m0, s0);
        merge_quad(m1, s1);
        z0 += __shfl_xor_sync(0xffffffffu, z0, 1);
        z0 += __shfl_xor_sync(0xffffffffu, z0, 2);
        z1 += __shfl_xor_sync(0xffffffffu, z1, 1);
        z1 += __shfl_xor_sync(0xffffffffu, z1, 2);
        if (t == 0) lossAcc += w0 * (m0 + logf(s0) - z0) + w1 * (m1 + logf(s1) - z1);
        const float is0 = 1.0f / s0, is1 = 1.0f / s1;
        // ---- output layer backward: dZ = w (softmax - onehot), dH3 = dZ W4
        float dh[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; nt++) dh[nt][0] = dh[nt][1] = dh[nt][2] = dh[nt][3] = 0.0f;
        {
            const int q = lane >> 3, rr = lane & 7;
            for (int kc = 0; kc < kt4; kc++) {
                float ca[4], cb[4];
                logits_tile(ca, h3, W4s, b4, 2 * kc, g, t);
                logits_tile(cb, h3, W4s, b4, 2 * kc + 1, g, t);
                const int cA = kc * 16 + 2 * t, cB = cA + 8;
                const uint32_t dz[4] = {
                    pack_bf16(w0 * (__expf(ca[0] - m0) * is0 - (t0 == cA ? 1.0f : 0.0f)),
                              w0 * (__expf(ca[1] - m0) * is0 - (t0 == cA + 1 ? 1.0f : 0.0f))),
                    pack_bf16(w1 * (__expf(ca[2] - m1) * is1 - (t1 == cA ? 1.0f : 0.0f)),
                              w1 * (__expf(ca[3] - m1) * is1 - (t1 == cA + 1 ? 1.0f : 0.0f))),
                    pack_bf16(w0 * (__expf(cb[0] - m0) * is0 - (t0 == cB ? 1.0f : 0.0f)),
                              w0 * (__expf(cb[1] - m0) * is0 - (t0 == cB + 1 ? 1.0f : 0.0f))),
                    pack_bf16(w1 * (__expf(cb[2] - m1) * is1 - (t1 == cB ? 1.0f : 0.0f)),
                              w1 * (__expf(cb[3] - m1) * is1 - (t1 == cB + 1 ? 1.0f : 0.0f)))};
#pragma unroll
                for (int np = 0; np < 4; np++) {
                    uint32_t b[4];
                    ldsm4t(b, W4s + (kc * 16 + (q & 1) * 8 + rr) * kLdh + (2 * np + (q >> 1)) * 8);
                    mma16816(dh[2 * np], dz, b[0], b[1]);
                    mma16816(dh[2 * np + 1], dz, b[2], b[3]);
                }
                frag[frag_at(0, tile, kc, ntiles, kt4) + lane] = dyt(dz);
            }
        }
        // ---- hidden layers 3, 2, 1: ReLU masks, store dY^T, propagate
        uint32_t dy[4][4];
        relu_back(dh, h3, dy);
#pragma unroll
        for (int mt = 0; mt < 4; mt++) frag[frag_at(2, tile, mt, ntiles, kt4) + lane] = dyt(dy[mt]);
        dgrad<4, 8>(dy, W3s, kLdh, dh, lane);
        relu_back(dh, h2, dy);
#pragma unroll
        for (int mt = 0; mt < 4; mt++) frag[frag_at(4, tile, mt, ntiles, kt4) + lane] = dyt(dy[mt]);
        dgrad<4, 8>(dy, W2s, kLdh, dh, lane);
#pragma unroll
        for (int kt = 0; kt < 4; kt++) {
            const __nv_bfloat16* r0 = H1s + g * kLdh + kt * 16 + 2 * t;
            h1[kt][0] = *reinterpret_cast<const uint32_t*>(r0);
            h1[kt][1] = *reinterpret_cast<const uint32_t*>(r0 + 8 * kLdh);
            h1[kt][2] = *reinterpret_cast<const uint32_t*>(r0 + 8);
            h1[kt][3] = *reinterpret_cast<const uint32_t*>(r0 + 8 * kLdh + 8);
        }
        relu_back(dh, h1, dy);
#pragma unroll
        for (int mt = 0; mt < 4; mt++) frag[frag_at(6, tile, mt, ntiles, kt4) + lane] = dyt(dy[mt]);
        // ---- encoding gradient: dX[:, 0:16] = dH1 W1[:, 0:16], scattered into the tables
        float dx[2][4];
        dgrad<4, 2>(dy, W1s, kLd1, dx, lane);
#pragma unroll
        for (int nt = 0; nt < 2; nt++) {
            dxs[g * 16 + nt * 8 + 2 * t] = dx[nt][0];
            dxs[g * 16 + nt * 8 + 2 * t + 1] = dx[nt][1];
            dxs[(g + 8) * 16 + nt * 8 + 2 * t] = dx[nt][2];
            dxs[(g + 8) * 16 + nt * 8 + 2 * t + 1] = dx[nt][3];
        }
        __syncwarp();
        if (valid) {
            const float4 ga = *reinterpret_cast<const float4*>(dxs + r * 16 + half * 8);
            const float4 gbv = *reinterpret_cast<const float4*>(dxs + r * 16 + half * 8 + 4);
            const int R = half == 0 ? d.res0 : d.res1;
            const float sc = (float)R * (1.0f / 1024.0f);
            const float ux = fminf(fmaxf(pin.x * sc, 0.0f), (float)R), uy = fminf(fmaxf(pin.y * sc, 0.0f), (float)R),
                        uz = fminf(fmaxf(pin.z * sc, 0.0f), (float)R);
            const int ix = min((int)ux, R - 1), iy = min((int)uy, R - 1), iz = min((int)uz, R - 1);
            const float fx = ux - (float)ix, fy = uy - (float)iy, fz = uz - (float)iz;
#pragma unroll
            for (int qc = 0; qc < 8; qc++) {
                const int ox = qc & 1, oy = (qc >> 1) & 1, oz = qc >> 2;
                const uint32_t idx = (uint32_t)half * (mask + 1u) +
                                     grid_hash((uint32_t)(ix + ox), (uint32_t)(iy + oy), (uint32_t)(iz + oz), mask);
                const float w = (ox ? fx : 1.0f - fx) * (oy ? fy : 1.0f - fy) * (oz ? fz : 1.0f - fz);
                float4* dst = reinterpret_cast<float4*>(encGrad + (size_t)idx * kFeat);
                atomicAdd(dst, make_float4(w * ga.x, w * ga.y, w * ga.z, w * ga.w));
                atomicAdd(dst + 1, make_float4(w * gbv.x, w * gbv.y, w * gbv.z, w * gbv.w));
            }
        }
        __syncwarp();
    }
    // ---- this CTA's loss
#pragma unroll
    for (int o = 16; o; o >>= 1) lossAcc += __shfl_xor_sync(0xffffffffu, lossAcc, o);
    if (lane == 0) s_loss[warp] = lossAcc;
    __syncthreads();
    if (threadIdx.x == 0) {
        float s = 0.0f;
        for (int w = 0; w < kTW; w++) s += s_loss[w];
        a.lossPart[blockIdx.x] = s;
    }
}

// Weight and bias gradients of one layer's 16 output rows (blockIdx.y: job) over one chunk
// of 16-sample tiles (blockIdx.x), from train_kernel's fragments. Jobs: dW4 row tiles
// 0..K/16-1, then 4 row tiles each of dW3, dW2, dW1. Bias gradients are the row sums of
// dY^T: an extra mma against a B fragment of ones.
__global__ void __launch_bounds__(256) wgrad_kernel(WgradArgs a) {
    __shared__ float red[kTW][32][37];
    const int kt4 = a.K / 16;
    const int job = blockIdx.y, chunk = blockIdx.x;
    const int layer = job < kt4 ? 4 : 3 - (job - kt4) / 4;
    const int mt = job < kt4 ? job : (job - kt4) % 4;
    const int ra = 2 * (4 - layer), rb = ra + 1;          // fragment regions of dY^T and X^T
    const int np = layer == 1 ? 2 : 4;                    // pairs of 8-column n-tiles
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t ones = pack_bf16(1.0f, 1.0f);
    float c[8][4], cb[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int i = 0; i < 8; i++) c[i][0] = c[i][1] = c[i][2] = c[i][3] = 0.0f;
    const uint32_t k0 = (uint32_t)chunk * a.chunkTiles;
    const uint32_t k1 = min(k0 + a.chunkTiles, a.ntiles);
    // two tiles per iteration: both tiles' loads are in flight before the first mma
    for (uint32_t kt = k0 + warp; kt < k1; kt += 2 * kTW) {
        const uint32_t kt2 = kt + kTW;
        const bool two = kt2 < k1;
        uint4 av[2], bv[2][4];
        av[0] = __ldcs(a.frag + frag_at(ra, kt, mt, a.ntiles, kt4) + lane);
        av[1] = two ? __ldcs(a.frag + frag_at(ra, kt2, mt, a.ntiles, kt4) + lane) : make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
        for (int p = 0; p < 4; p++) {
            if (p >= np) break;
            bv[0][p] = __ldg(a.frag + frag_at(rb, kt, p, a.ntiles, kt4) + lane);
            bv[1][p] = two ? __ldg(a.frag + frag_at(rb, kt2, p, a.ntiles, kt4) + lane) : make_uint4(0u, 0u, 0u, 0u);
        }
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const uint32_t af[4] = {av[u].x, av[u].y, av[u].z, av[u].w};
#pragma unroll
            for (int p = 0; p < 4; p++) {
                if (p >= np) break;
                mma16816(c[2 * p], af, bv[u][p].x, bv[u][p].y);
                mma16816(c[2 * p + 1], af, bv[u][p].z, bv[u][p].w);
            }
            mma16816(cb, af, ones, ones);
        }
    }
#pragma unroll
    for (int i = 0; i < 8; i++)
#pragma unroll
        for (int q = 0; q < 4; q++) red[warp][lane][i * 4 + q] = c[i][q];
    red[warp][lane][32] = cb[0];
    red[warp][lane][33] = cb[2];
    __syncthreads();
    // the warps' sums in a fixed order, into this chunk's row of the partial table
    const int ncol = np * 16, ncols = layer == 1 ? kIn : kTH;
    // parameter order from W1: W1 [64][32], b1, W2 [64][64], b2, W3 [64][64], b3, W4 [K][64], b4
    const int offW = layer == 1 ? 0 : kTH * kIn + kTH + (layer - 2) * (kTH * kTH + kTH);
    const int offB = offW + (layer == 4 ? a.K : kTH) * ncols;
    float* out = a.partials + (size_t)chunk * a.nmlp;
    for (int e = threadIdx.x; e < 16 * ncol + 16; e += blockDim.x) {
        int ln, idx, dst;
        if (e < 16 * ncol) {
            const int row = e / ncol, col = e % ncol;
            ln = (row & 7) * 4 + ((col & 7) >> 1);
            idx = (col >> 3) * 4 + (row >> 3) * 2 + (col & 1);
            dst = offW + (mt * 16 + row) * ncols + col;
        } else {
            const int row = e - 16 * ncol;
            ln = (row & 7) * 4;
            idx = 32 + (row >> 3);
            dst = offB + mt * 16 + row;
        }
        float sum = 0.0f;
#pragma unroll
        for (int w = 0; w < kTW; w++) sum += red[w][ln][idx];
        out[dst] = sum;
    }
}

// 256 threads per block: 64 parameters, each summed over the partial rows by 4 groups of
// 64 threads (group q takes rows q, q + 4, ...; coalesced along the parameters), the
// groups' sums added in a fixed order
__global__ void __launch_bounds__(256) train_reduce_kernel(ReduceArgs r) {
    __shared__ float part[4][64];
    const int H = kTH, K = r.K;
    const int sb1 = H * kIn, sW2 = sb1 + H, sb2 = sW2 + H * H, sW3 = sb2 + H, sb3 = sW3 + H * H, sW4 = sb3 + H,
              sb4 = sW4 + K * H;
    const int q = threadIdx.x >> 6, col = threadIdx.x & 63;
    for (int base = blockIdx.x * 64; base < r.nmlp; base += gridDim.x * 64) {
        const int ic = base + col;
        float gq = 0.0f;
        if (ic < r.nmlp)
            for (int c = q; c < r.nparts; c += 4) gq += r.partials[(size_t)c * r.nmlp + ic];
        part[q][col] = gq;
        __syncthreads();
        const int i = ic;
        const bool mine = q == 0 && i < r.nmlp;
        const float g = (part[0][col] + part[1][col]) + (part[2][col] + part[3][col]);
        __syncthreads();
        if (!mine) continue;
        r.grads[i] = g;
        if (!r.apply) continue;
        const float mi = r.b1 * r.m[i] + (1.0f - r.b1) * g;
        const float vi = r.b2 * r.v[i] + (1.0f - r.b2) * g * g;
        r.m[i] = mi;
        r.v[i] = vi;
        const float p = r.params[i] - r.lr * (mi * r.c1) / (sqrtf(vi * r.c2) + r.eps);
        r.params[i] = p;
        int o = -1;
        if (i < sb1) o = i;
        else if (i >= sW2 && i < sb2) o = H * kIn + (i - sW2);
        else if (i >= sW3 && i < sb3) o = H * kIn + H * H + (i - sW3);
        else if (i >= sW4 && i < sb4) o = H * kIn + 2 * H * H + (i - sW4);
        if (o >= 0) r.wbf[o] = __float2bfloat16_rn(p);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        float l = 0.0f, w = 0.0f;
        for (int c = 0; c < r.nloss; c++) l += r.lossPart[c];
        for (uint32_t c = 0; c < r.nwpart; c++) w += r.wpart[c];
        r.scal[0] = l;
        r.scal[1] = w;
    }
}

// Adam on the hash tables (n a multiple of 4); the gradient is cleared for the next step
__global__ void adam_enc_kernel(float4* __restrict__ p, float4* __restrict__ gr, float4* __restrict__ m,
                                float4* __restrict__ v, size_t n4, float lr, float b1, float b2, float eps, float c1,
                                float c2) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x) {
        const float4 g = gr[i];
        gr[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        float4 mi = m[i], vi = v[i], pi = p[i];
        auto upd = [&](float gg, float& mm, float& vv, float& pp) {
            mm = b1 * mm + (1.0f - b1) * gg;
            vv = b2 * vv + (1.0f - b2) * gg * gg;
            pp -= lr * (mm * c1) / (sqrtf(vv * c2) + eps);
        };
        upd(g.x, mi.x, vi.x, pi.x);
        upd(g.y, mi.y, vi.y, pi.y);
        upd(g.z, mi.z, vi.z, pi.z);
        upd(g.w, mi.w, vi.w, pi.w);
        m[i] = mi;
        v[i] = vi;
        p[i] = pi;
    }
}

int device_sms() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

}  // namespace

bool train_supported(const Dims& d) { return d.H == kTH && d.K >= 16 && d.K <= 256 && d.K % 16 == 0; }

int train_mlp_count(const Dims& d) { return (int)(layout(d).total - layout(d).W1); }

size_t train_smem_bytes(const Dims& d) {
    return (size_t)(kTH * kLd1 + 2 * kTH * kLdh + d.K * kLdh) * 2 + (size_t)(3 * kTH + d.K) * 4 +
           (size_t)kTW * kTrainWarpBytes;
}

size_t train_frag_bytes(const Dims& d, uint32_t B) {
    return (size_t)((B + 15) / 16) * frag_prefix(8, d.K / 16) * 512;
}

uint32_t train_chunks(uint32_t B) { return std::max(1u, ((B + 15) / 16 + kChunkTiles - 1) / kChunkTiles); }

int train_max_ctas() { return kTrainCtasPerSm * device_sms(); }
uint32_t train_wsum_blocks() { return kWsumBlocks; }

void launch_wsum(const float* w, uint32_t B, float* part, cudaStream_t s) {
    wsum_kernel<<<kWsumBlocks, 256, 0, s>>>(w, B, part);
}

cudaError_t launch_train(const TrainArgs& a, cudaStream_t s, int* nparts, int* nloss) {
    const size_t sm = train_smem_bytes(a.dims);
    cudaError_t e = cudaFuncSetAttribute(train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    const uint32_t tiles = (a.B + 15) / 16;
    const int ctas = (int)std::max<uint32_t>(1, std::min<uint32_t>((tiles + kTW - 1) / kTW, (uint32_t)train_max_ctas()));
    train_kernel<<<ctas, kTW * 32, sm, s>>>(a);
    *nloss = ctas;
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    WgradArgs w{};
    w.frag = a.frag;
    w.ntiles = tiles;
    w.chunkTiles = kChunkTiles;
    w.K = a.dims.K;
    w.nmlp = train_mlp_count(a.dims);
    w.partials = a.partials;
    const uint32_t chunks = train_chunks(a.B);
    wgrad_kernel<<<dim3(chunks, a.dims.K / 16 + 12), 256, 0, s>>>(w);
    *nparts = (int)chunks;
    return cudaGetLastError();
}

void launch_train_reduce(const ReduceArgs& r, cudaStream_t s) {
    const int blocks = std::max(1, std::min((r.nmlp + 63) / 64, 2048));
    train_reduce_kernel<<<blocks, 256, 0, s>>>(r);
}

void launch_adam_enc(float* p, float* g, float* m, float* v, size_t n, float lr, int step, cudaStream_t s) {
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f / (1.0f - powf(b1, (float)step)), c2 = 1.0f / (1.0f - powf(b2, (float)step));
    const size_t n4 = n / 4;
    adam_enc_kernel<<<(unsigned)std::min<size_t>((n4 + 255) / 256, 4096), 256, 0, s>>>(
        reinterpret_cast<float4*>(p), reinterpret_cast<float4*>(g), reinterpret_cast<float4*>(m),
        reinterpret_cast<float4*>(v), n4, lr, b1, b2, 1e-8f, c1, c2);
}

}  // namespace prop
}  // namespace vxr
