// proposal.cu - kernels of the learned candidate proposal (see proposal.cuh).
//
// Inference (one launch per frame, over the hit-pixel list): per warp of 32 pixels the
// hash-grid encoding is built in shared memory, the MLP runs on the tensor cores with
// BF16 mma.sync.m16n8k16 (FP32 accumulation, hidden layers kept in registers: the
// accumulator fragment of one layer is the A fragment of the next), the K logits land
// in shared memory as FP16, and every lane draws its pixel's candidates from
// p_src(e) = (1 - eps) softmax(c(e)) / |c(e)| + eps / N: with probability eps an emitter
// uniformly, else a cluster through a two-level (16 groups) inverse CDF and one of its
// emitters uniformly. Output: (emitter, p_src) per candidate, candidate-major so that
// both this kernel's stores and the candidate kernel's loads are coalesced.
//
// Training (FP32 CUDA cores): batch gather from the reservoirs, encoding, a tiled
// strided GEMM with fused epilogues for every forward / backward product, softmax
// cross-entropy, encoding scatter, Adam.
//
// This file builds with FMA contraction on: the learned path is checked against FP64
// with tolerances, not bit for bit.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cstdint>

#include "device.cuh"
#include "proposal.cuh"
#include "proposal.hpp"
#include "proposal_dev.cuh"

namespace vxr {
namespace prop {

// ---- inference --------------------------------------------------------------------------
// A warp handles 16 pixels (one m16 tile): two lanes per pixel (lane = half * 16 + row)
// split the encoding (one hash-grid level each), the softmax tables (8 groups each) and
// the candidates (every other one each). 16 pixels per warp keep the MLP within 128
// registers per thread, so 16 warps share one copy of the weights per SM.
// Shared memory: W1 [H][kIn+8], W2,W3 [H][H+8], W4 [K][H+8] (BF16, rows padded against
// bank conflicts), biases (FP32), cluster offsets [K+1], then per warp X [16][kIn+8]
// (BF16; later the rows' group prefix sums [16][16] FP32) and logits [16][K+8] (FP16, then
// the sampling tables; rows 16-byte aligned).
template <int H>
__global__ void __launch_bounds__(512, 1) infer_kernel(InferArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const Dims d = a.dims;
    const int K = d.K;
    const int ld1 = kIn + 8, ldh = H + 8, ldl = K + 8, ldx = kIn + 8;
    const int nwarps = blockDim.x >> 5;
    __nv_bfloat16* W1s = reinterpret_cast<__nv_bfloat16*>(smem);
    __nv_bfloat16* W2s = W1s + H * ld1;
    __nv_bfloat16* W3s = W2s + H * ldh;
    __nv_bfloat16* W4s = W3s + H * ldh;
    float* bs = reinterpret_cast<float*>(W4s + (size_t)K * ldh);           // b1 | b2 | b3 | b4
    uint32_t* offs = reinterpret_cast<uint32_t*>(bs + 3 * H + K);          // cluster offsets [K + 1]
    __nv_bfloat16* Xall = reinterpret_cast<__nv_bfloat16*>(offs + ((K + 1 + 3) & ~3));
    __half* Lall = reinterpret_cast<__half*>(Xall + (size_t)nwarps * 16 * ldx);
    {
        const __nv_bfloat16* wg = a.wbf;   // W1 [H][kIn] | W2 [H][H] | W3 [H][H] | W4 [K][H]
        for (int e = threadIdx.x; e < H * kIn; e += blockDim.x) W1s[(e / kIn) * ld1 + e % kIn] = wg[e];
        wg += H * kIn;
        for (int e = threadIdx.x; e < H * H; e += blockDim.x) W2s[(e / H) * ldh + e % H] = wg[e];
        wg += H * H;
        for (int e = threadIdx.x; e < H * H; e += blockDim.x) W3s[(e / H) * ldh + e % H] = wg[e];
        wg += H * H;
        for (int e = threadIdx.x; e < K * H; e += blockDim.x) W4s[(e / H) * ldh + e % H] = wg[e];
        const float* p = a.params;
        for (int e = threadIdx.x; e < H; e += blockDim.x) {
            bs[e] = p[a.L.b1 + e];
            bs[H + e] = p[a.L.b2 + e];
            bs[2 * H + e] = p[a.L.b3 + e];
        }
        for (int e = threadIdx.x; e < K; e += blockDim.x) bs[3 * H + e] = p[a.L.b4 + e];
        if (a.clOff)
            for (int e = threadIdx.x; e <= K; e += blockDim.x) offs[e] = a.clOff[e];
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int r = lane & 15, half = lane >> 4;
    __nv_bfloat16* Xs = Xall + (size_t)warp * 16 * ldx;
    __half* Ls = Lall + (size_t)warp * 16 * ldl;
    const float* enc = a.params + a.L.enc;
    const uint32_t n = a.count ? *a.count : a.n;
    const int gs = K / 16;
    for (uint32_t base = (blockIdx.x * nwarps + warp) * 16; base < n; base += gridDim.x * nwarps * 16) {
        const uint32_t j = base + r;
        const bool valid = j < n;
        float4 pin = make_float4(0.f, 0.f, 0.f, __uint_as_float(6u));
        uint32_t pix = 0;
        if (valid) {
            if (a.samples) {
                pin = a.samples[j];
            } else {
                pix = a.hits[j];
                const int x = (int)(pix % (uint32_t)a.k.W), y = (int)(pix / (uint32_t)a.k.W);
                const uint2 gv = a.vd[pix];
                const uint32_t side = gv.x >> 24;
                const float dist = __uint_as_float(gv.y);
                const float3 D = dev::camera_ray(a.k, x, y);
                const float ns = dev::side_sign(side, D);
                pin = make_float4(D.x * dist + a.k.E.x, D.y * dist + a.k.E.y, D.z * dist + a.k.E.z,
                                  __uint_as_float(side_code(side, ns)));
            }
        }
        // input row: this lane's hash-grid level; the first half also the one-hot side
        {
            float f[8];
            level_features(enc, d, pin.x, pin.y, pin.z, half, f);
            __nv_bfloat16* xr = Xs + r * ldx;
#pragma unroll
            for (int q = 0; q < 8; q += 2)
                *reinterpret_cast<uint32_t*>(xr + half * 8 + q) = valid ? pack_bf16(f[q], f[q + 1]) : 0u;
            if (half == 0) {
                const uint32_t code = __float_as_uint(pin.w);
#pragma unroll
                for (int q = 16; q < kIn; q += 2)
                    *reinterpret_cast<uint32_t*>(xr + q) =
                        valid ? pack_bf16(code == (uint32_t)(q - 16) ? 1.f : 0.f, code == (uint32_t)(q - 15) ? 1.f : 0.f) : 0u;
            }
        }
        __syncwarp();
        // layer 1 (kIn = 32 -> H) from shared memory
        uint32_t act[H / 16][4], act2[H / 16][4];
        {
            uint32_t xa[2][4];
#pragma unroll
            for (int kt = 0; kt < 2; kt++) {
                const __nv_bfloat16* r0 = Xs + g * ldx + kt * 16 + 2 * t;
                const __nv_bfloat16* r1 = r0 + 8 * ldx;
                xa[kt][0] = *reinterpret_cast<const uint32_t*>(r0);
                xa[kt][1] = *reinterpret_cast<const uint32_t*>(r1);
                xa[kt][2] = *reinterpret_cast<const uint32_t*>(r0 + 8);
                xa[kt][3] = *reinterpret_cast<const uint32_t*>(r1 + 8);
            }
            float c[H / 8][4];
#pragma unroll
            for (int nt = 0; nt < H / 8; nt++) {
                const float b0 = bs[nt * 8 + 2 * t], b1 = bs[nt * 8 + 2 * t + 1];
                c[nt][0] = b0; c[nt][1] = b1; c[nt][2] = b0; c[nt][3] = b1;
            }
#pragma unroll
            for (int kt = 0; kt < 2; kt++)
#pragma unroll
                for (int nt = 0; nt < H / 8; nt++) {
                    const __nv_bfloat16* row = W1s + (nt * 8 + g) * ld1 + kt * 16 + 2 * t;
                    mma16816(c[nt], xa[kt], *reinterpret_cast<const uint32_t*>(row),
                             *reinterpret_cast<const uint32_t*>(row + 8));
                }
#pragma unroll
            for (int kt = 0; kt < H / 16; kt++) {
                act[kt][0] = pack_bf16(fmaxf(c[2 * kt][0], 0.f), fmaxf(c[2 * kt][1], 0.f));
                act[kt][1] = pack_bf16(fmaxf(c[2 * kt][2], 0.f), fmaxf(c[2 * kt][3], 0.f));
                act[kt][2] = pack_bf16(fmaxf(c[2 * kt + 1][0], 0.f), fmaxf(c[2 * kt + 1][1], 0.f));
                act[kt][3] = pack_bf16(fmaxf(c[2 * kt + 1][2], 0.f), fmaxf(c[2 * kt + 1][3], 0.f));
            }
        }
        hidden_layer<H>(act, act2, W2s, ldh, bs + H, g, t);
        hidden_layer<H>(act2, act, W3s, ldh, bs + 2 * H, g, t);
        // output layer: K logits, 8 columns at a time, to shared memory as FP16
        for (int nt = 0; nt < K / 8; nt++) {
            const float b0 = bs[3 * H + nt * 8 + 2 * t], b1 = bs[3 * H + nt * 8 + 2 * t + 1];
            float c0[4] = {b0, b1, b0, b1};
#pragma unroll
            for (int kt = 0; kt < H / 16; kt++) {
                const __nv_bfloat16* row = W4s + (size_t)(nt * 8 + g) * ldh + kt * 16 + 2 * t;
                mma16816(c0, act[kt], *reinterpret_cast<const uint32_t*>(row), *reinterpret_cast<const uint32_t*>(row + 8));
            }
            const int col = nt * 8 + 2 * t;
            *reinterpret_cast<__half2*>(Ls + g * ldl + col) = __floats2half2_rn(c0[0], c0[1]);
            *reinterpret_cast<__half2*>(Ls + (g + 8) * ldl + col) = __floats2half2_rn(c0[2], c0[3]);
        }
        __syncwarp();
        // Softmax of each row, stored for sampling as 16-bit fixed-point prefix sums inside
        // each group of K/16 clusters (fraction of the group total, last = 65535),
        // overwriting the logits, and FP32 prefix sums Prow over the 16 group totals. Every
        // probability the sampler reports comes from these stored numbers: group q has
        // weight P[q] - P[q-1], cluster c inside it (fp[c] - fp[c-1]) / 65535 of that, so
        // the pdf returned with a sample is the pdf it was drawn with (up to FP32
        // rounding) and small clusters keep a resolution of 1/65535 of their group.
        float* Prow = reinterpret_cast<float*>(Xs);   // X is dead after layer 1
        if (K == 256) {
            // two rows at a time, a half-warp per row: lane l of the half holds group l
            // (16 columns, 32 bytes), so the group total and its in-group prefix sums stay in
            // the lane; row maxima and the scan over the 16 groups are half-warp shuffles
            const int lr = lane & 15;
            for (int rr = half; rr < 16; rr += 2) {
                uint4* rowv = reinterpret_cast<uint4*>(Ls + rr * ldl) + 2 * lr;
                const uint4 raw0 = rowv[0], raw1 = rowv[1];
                float z[16];
                {
                    const __half2* h0 = reinterpret_cast<const __half2*>(&raw0);
                    const __half2* h1 = reinterpret_cast<const __half2*>(&raw1);
#pragma unroll
                    for (int i = 0; i < 4; i++) {
                        const float2 f0 = __half22float2(h0[i]), f1 = __half22float2(h1[i]);
                        z[2 * i] = f0.x; z[2 * i + 1] = f0.y;
                        z[8 + 2 * i] = f1.x; z[8 + 2 * i + 1] = f1.y;
                    }
                }
                float m = z[0];
#pragma unroll
                for (int i = 1; i < 16; i++) m = fmaxf(m, z[i]);
#pragma unroll
                for (int o = 8; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
                // in-group prefix sums as two chains of 8, joined
                float pa[8], pb[8];
                float ea = 0.0f, eb = 0.0f;
#pragma unroll
                for (int i = 0; i < 8; i++) {
                    ea += __expf(z[i] - m);
                    eb += __expf(z[8 + i] - m);
                    pa[i] = ea;
                    pb[i] = eb;
                }
                const float T = ea + eb;
                const float sc = T > 0.0f ? 65535.0f / T : 0.0f;
                uint32_t pk[8];
#pragma unroll
                for (int i = 0; i < 8; i += 2) {
                    pk[i / 2] = min((uint32_t)(pa[i] * sc), 65535u) | (min((uint32_t)(pa[i + 1] * sc), 65535u) << 16);
                    const uint32_t hi = i == 6 ? 65535u : min((uint32_t)((ea + pb[i + 1]) * sc), 65535u);
                    pk[4 + i / 2] = min((uint32_t)((ea + pb[i]) * sc), 65535u) | (hi << 16);
                }
                rowv[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                rowv[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
                // inclusive scan of the group totals over the half-warp
                float v = T;
#pragma unroll
                for (int o = 1; o < 16; o <<= 1) {
                    const float u = __shfl_up_sync(0xffffffffu, v, o, 16);
                    if (lr >= o) v += u;
                }
                Prow[rr * 16 + lr] = v;
            }
        } else {
            // generic K: the two lanes of a row take 8 groups each
            __half* row = Ls + r * ldl;
            uint16_t* fpw = reinterpret_cast<uint16_t*>(row);
            float mx = -INFINITY;
            for (int c = half * (K / 2); c < (half + 1) * (K / 2); c++) mx = fmaxf(mx, __half2float(row[c]));
            mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 16));
            float Pl[8];
            float Zl = 0.0f;
#pragma unroll
            for (int q8 = 0; q8 < 8; q8++) {
                const int q = half * 8 + q8;
                float T = 0.0f;
                for (int c = q * gs; c < (q + 1) * gs; c++) {
                    const __half h = __float2half_rn(__expf(__half2float(row[c]) - mx));
                    row[c] = h;
                    T += __half2float(h);
                }
                const float sc = T > 0.0f ? 65535.0f / T : 0.0f;
                float acc = 0.0f;
                for (int c = q * gs; c < (q + 1) * gs; c++) {
                    acc += __half2float(row[c]);
                    fpw[c] = c == (q + 1) * gs - 1 ? (uint16_t)65535u : (uint16_t)min((uint32_t)(acc * sc), 65535u);
                }
                Zl += T;
                Pl[q8] = Zl;
            }
            const float lowZ = __shfl_xor_sync(0xffffffffu, Pl[7], 16);
#pragma unroll
            for (int i = 0; i < 8; i++) Prow[r * 16 + half * 8 + i] = half ? Pl[i] + lowZ : Pl[i];
        }
        __syncwarp();
        const uint16_t* fp = reinterpret_cast<const uint16_t*>(Ls + r * ldl);
        float P[16];
#pragma unroll
        for (int i = 0; i < 16; i += 4) {
            const float4 p4 = *reinterpret_cast<const float4*>(Prow + r * 16 + i);
            P[i] = p4.x; P[i + 1] = p4.y; P[i + 2] = p4.z; P[i + 3] = p4.w;
        }
        const float Z = P[15], invZ = 1.0f / Z;
        // fraction of its group held by cluster c
        auto frac = [&](int c) {
            const uint32_t hi = fp[c], lo = (c % gs) ? fp[c - 1] : 0u;
            return (float)(hi - lo) * (1.0f / 65535.0f);
        };
        if (valid) {
            if (a.probs) {
#pragma unroll
                for (int q = 0; q < 16; q++) {
                    if ((q >> 3) != half) continue;
                    const float gw = q ? P[q] - P[q - 1] : P[0];
                    for (int c = q * gs; c < (q + 1) * gs; c++) a.probs[(size_t)j * K + c] = (gw * frac(c)) * invZ;
                }
            } else {
                uint32_t s = dev::wang_hash(pix * 2654435761u + a.k.R0 * 0x85EBCA6Bu + 0x9E3779B9u + (uint32_t)half * 0x68E31DA4u);
                const float eps = d.eps, invN = 1.0f / (float)a.nlights;
                uint2* out = a.cand + j;
                // unrolled so that the emitter loads of several candidates are in flight together
#pragma unroll 4
                for (uint32_t m = (uint32_t)half; m < a.ncand; m += 2) {
                    const float u = dev::rnd(s);
                    const float v = dev::rnd(s);
                    const float w = dev::rnd(s);
                    int c;
                    uint32_t e;
                    float gw;   // weight of the chosen cluster's group
                    if (u < eps) {
                        // defensive part: an emitter uniformly
                        e = min((uint32_t)(v * (float)a.nlights), a.nlights - 1u);
                        c = (int)__ldg(a.lightCluster + e);
                        const int q = c / gs;
                        float lo = 0.0f, hi = P[0];
#pragma unroll
                        for (int i = 1; i < 16; i++)
                            if (q == i) { lo = P[i - 1]; hi = P[i]; }
                        gw = hi - lo;
                    } else {
                        // group: count of prefix sums <= target (branch-free)
                        const float target = v * Z;
                        int q = 0;
                        float lo = 0.0f, hi = P[0];
#pragma unroll
                        for (int i = 0; i < 15; i++)
                            if (target >= P[i]) { q = i + 1; lo = P[i]; hi = P[i + 1]; }
                        // cluster inside the group: count of in-group prefix fractions <= the
                        // target's fraction of the group
                        gw = hi - lo;
                        const float x = gw > 0.0f ? (target - lo) * (65535.0f / gw) : 0.0f;
                        int in = 0;
                        if (gs == 16) {
                            const uint4 a0 = *reinterpret_cast<const uint4*>(fp + q * 16);
                            const uint4 a1 = *reinterpret_cast<const uint4*>(fp + q * 16 + 8);
                            const uint32_t wv[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
#pragma unroll
                            for (int i = 0; i < 15; i++)
                                in += x >= (float)((wv[i >> 1] >> ((i & 1) * 16)) & 0xFFFFu) ? 1 : 0;
                        } else {
                            for (int i = 0; i < gs - 1; i++) in += x >= (float)fp[q * gs + i] ? 1 : 0;
                        }
                        c = q * gs + in;
                        // an emitter of cluster c, uniformly
                        const uint32_t off = offs[c], sz = offs[c + 1] - off;
                        e = __ldg(a.clMembers + off + min((uint32_t)(w * (float)sz), sz - 1u));
                    }
                    // p_src(e) = (1 - eps) softmax(c(e)) / |c(e)| + eps / N
                    const float sz = (float)(offs[c + 1] - offs[c]);
                    const float pe = (1.0f - eps) * (((gw * frac(c)) * invZ) / sz) + eps * invN;
                    out[(size_t)m * a.candStride] = make_uint2(e, __float_as_uint(pe));
                }
            }
        }
        __syncwarp();
    }
}

// ---- inference on the 5th-generation tensor cores (tcgen05, TMEM) --------------------------
// The same network and sampler as infer_kernel for H = 64 and K = 256. A CTA of 256 threads
// runs two independent tiles of 128 hit pixels (threads 0-127 and 128-255, one pixel per
// thread = one TMEM lane). Per layer one thread issues tcgen05.mma (M = 128, N = 64 or 256,
// K = 16 per instruction; A = the tile's activations, B = the weights, both BF16 in shared
// memory in the K-major no-swizzle core-matrix layout), the accumulator stays in tensor
// memory (FP32), tcgen05.commit arrives on an mbarrier, and every thread reads its own
// row back with tcgen05.ld for the epilogue (bias, ReLU, BF16 into the next layer's A) or,
// after the output layer, for its pixel's softmax tables and candidates. All waits are
// bounded; on a timeout the kernel raises *a.err, skips its remaining tiles and still
// frees its tensor memory.
constexpr float kLog2e = 1.44269504088896340736f;   // log2(e)

namespace tc {
constexpr int kTile = 128;
constexpr uint32_t kCols = 512;          // TMEM columns: 256 per tile
constexpr int kRowBytes = 512 + 16;      // a pixel's sampling table (256 x u16), padded

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (r, k) in a K-major no-swizzle operand with `kdim` columns:
// 8-row x 16-byte core matrices, 128 bytes apart along K, kdim * 16 bytes apart along rows
__device__ __forceinline__ uint32_t core_off(int r, int k, int kdim) {
    return (uint32_t)((r >> 3) * (kdim * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}
// shared-memory matrix descriptor (no swizzle): start address, leading-dimension (K)
// byte offset, stride-dimension (M/N) byte offset, descriptor version 1
__device__ __forceinline__ uint64_t desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}
// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, M x N
__device__ __forceinline__ constexpr uint32_t idesc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(id), "r"(acc));
}
__device__ __forceinline__ void commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void bar_tile(int id) { asm volatile("bar.sync %0, 256;" ::"r"(id) : "memory"); }
// 2^x on the special-function unit (PTX ex2.approx.f32)
__device__ __forceinline__ float ex2(float x) {
    float y;
    asm("ex2.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
constexpr uint32_t kWaitLimit = 1u << 22;   // tries of a wait for an MMA in flight
// bounded wait for the mbarrier phase of parity `par`; false when `limit` tries ran out
__device__ __forceinline__ bool wait(uint32_t mbar, uint32_t par, uint32_t limit) {
    for (uint32_t i = 0; i < limit; i++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred P;\n\tmbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\n\tselp.b32 %0, 1, 0, P;\n\t}\n"
            : "=r"(done)
            : "r"(mbar), "r"(par)
            : "memory");
        if (done) return true;
    }
    return false;
}
// AND of `pred` over the 256 threads of tile barrier `id` (a barrier itself), so that a
// tile leaves its layer loop as one when a wait gives up in any of its threads
__device__ __forceinline__ bool tile_all(int id, bool pred) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.and.pred q, %2, 256, p;\n\tselp.u32 %0, 1, 0, q;\n\t}\n"
        : "=r"(r)
        : "r"((uint32_t)pred), "r"(id)
        : "memory");
    return r != 0;
}
// 32 consecutive TMEM columns of this thread's lane
__device__ __forceinline__ void ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    __syncwarp();
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}
// copy a BF16 [rows][kdim] row-major matrix into the core-matrix layout (16-byte chunks)
__device__ __forceinline__ void stage(const __nv_bfloat16* g, unsigned char* s, int rows, int kdim) {
    const int chunks = rows * (kdim / 8);
    for (int c = threadIdx.x; c < chunks; c += blockDim.x) {
        const int r = c / (kdim / 8), k = (c % (kdim / 8)) * 8;
        *reinterpret_cast<uint4*>(s + core_off(r, k, kdim)) = *reinterpret_cast<const uint4*>(g + (size_t)r * kdim + k);
    }
}
// columns [32 half, 32 half + 32) of one thread's row of 64 accumulators -> bias, ReLU,
// BF16, into the next A operand (K = 64)
__device__ __forceinline__ void epilogue32(uint32_t taddr, const float* bias, unsigned char* A, int row, int half) {
    float v[32];
    ld32(taddr + half * 32, v);
#pragma unroll
    for (int c = 0; c < 4; c++) {
        uint32_t w[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int k = half * 32 + c * 8 + 2 * q;
            w[q] = pack_bf16(fmaxf(v[c * 8 + 2 * q] + bias[k], 0.0f), fmaxf(v[c * 8 + 2 * q + 1] + bias[k + 1], 0.0f));
        }
        *reinterpret_cast<uint4*>(A + core_off(row, half * 32 + c * 8, 64)) = make_uint4(w[0], w[1], w[2], w[3]);
    }
}
}  // namespace tc

// Two tiles of 128 pixels per CTA, each owned by two warpgroups that split the work of a
// pixel by columns: warpgroup `half` encodes hash-grid level `half` (half 1 also the
// one-hot side), moves columns [32 half, 32 half + 32) of each hidden layer from TMEM to
// the next A operand, builds the sampling tables of cluster groups [8 half, 8 half + 8)
// and draws the candidates m with m % 2 == half (both advance the pixel's RNG alike).
// The two halves' group totals meet through shared memory. 16 warps per SM.
__global__ void __launch_bounds__(512, 1) infer_tc_kernel(InferArgs a) {
    extern __shared__ __align__(1024) unsigned char smem[];
    constexpr int H = 64, K = 256;
    unsigned char* W1c = smem;                     // [64][32]
    unsigned char* W2c = W1c + H * kIn * 2;        // [64][64]
    unsigned char* W3c = W2c + H * H * 2;
    unsigned char* W4c = W3c + H * H * 2;          // [256][64]
    float* bs = reinterpret_cast<float*>(W4c + K * H * 2);   // b1 | b2 | b3 | b4
    uint32_t* offs = reinterpret_cast<uint32_t*>(bs + 3 * H + K);
    unsigned char* Abuf = reinterpret_cast<unsigned char*>(offs + 260);            // 2 x [128][64]
    unsigned char* Tbuf = Abuf + 2 * tc::kTile * H * 2;                             // 2 x 128 table rows
    uint64_t* mbars = reinterpret_cast<uint64_t*>(Tbuf + 2 * tc::kTile * tc::kRowBytes);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(mbars + 2);
    const int warp = threadIdx.x >> 5;
    {
        const __nv_bfloat16* wg = a.wbf;
        tc::stage(wg, W1c, H, kIn);
        tc::stage(wg + H * kIn, W2c, H, H);
        tc::stage(wg + H * kIn + H * H, W3c, H, H);
        tc::stage(wg + H * kIn + 2 * H * H, W4c, K, H);
        const float* p = a.params;
        for (int e = threadIdx.x; e < H; e += blockDim.x) {
            bs[e] = p[a.L.b1 + e];
            bs[H + e] = p[a.L.b2 + e];
            bs[2 * H + e] = p[a.L.b3 + e];
        }
        // output bias in log2 units: the softmax works with 2^(log2(e) z)
        for (int e = threadIdx.x; e < K; e += blockDim.x) bs[3 * H + e] = p[a.L.b4 + e] * kLog2e;
        if (a.clOff)
            for (int e = threadIdx.x; e <= K; e += blockDim.x) offs[e] = a.clOff[e];
        if (threadIdx.x == 0) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc::smem_u32(&mbars[0])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc::smem_u32(&mbars[1])));
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        if (warp == 0) {
            __syncwarp();
            asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc::smem_u32(tslot)),
                         "r"(tc::kCols));
            asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
        }
        tc::fence_async_smem();
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *tslot;
    const int h = threadIdx.x >> 8, t = threadIdx.x & 255, half = t >> 7, tid = t & 127, wq = warp & 3, bar = 1 + h;
    unsigned char* A = Abuf + h * tc::kTile * H * 2;
    unsigned char* T = Tbuf + h * tc::kTile * tc::kRowBytes;
    uint16_t* fp = reinterpret_cast<uint16_t*>(T + tid * tc::kRowBytes);
    // after the last layer A is free until the next tile's input: the halves' maxima and
    // group totals, [half][9][128] floats
    float* X = reinterpret_cast<float*>(A);
    const uint32_t mbar = tc::smem_u32(&mbars[h]);
    const uint32_t dcol = tmem + (uint32_t)(h * 256);                 // this tile's accumulator columns
    const uint32_t trow = dcol + ((uint32_t)(wq * 32) << 16);         // this warp's lanes
    const uint32_t aaddr = tc::smem_u32(A);
    const float* enc = a.params + a.L.enc;
    const Dims d = a.dims;
    const uint32_t n = a.count ? *a.count : a.n;
    const int gs = K / 16;
    uint32_t phase = 0;
    bool ok = true;
    bool pending = false;   // an MMA was committed whose completion no wait has seen
    const uint32_t limit = a.waitLimit ? a.waitLimit : tc::kWaitLimit;
    const bool issue = !a.skipMma;
    // render mode with sharing: a table row may serve up to eight consecutive hit pixels
    // (the network runs on the first one's shading point; each draws its own candidates
    // from the row's tables)
    const bool useRows = a.rows && !a.samples && !a.probs;
    const uint32_t rows = useRows ? *a.rowCount : n;
    uint32_t tile = blockIdx.x * 2 + h;
    for (; ok && (size_t)tile * tc::kTile < rows; tile += gridDim.x * 2) {
        const uint32_t row = tile * tc::kTile + tid;
        const bool valid = row < rows;
        uint32_t j = row, span = 1u;
        if (useRows && valid) {
            const uint32_t e = a.rows[row];
            j = e & 0x1FFFFFFFu;
            span = (e >> 29) + 1u;
        }
        float4 pin = make_float4(0.f, 0.f, 0.f, __uint_as_float(6u));
        uint32_t pix = 0;
        if (valid) {
            if (a.samples) {
                pin = a.samples[j];
            } else {
                pix = a.hits[j];
                const int x = (int)(pix % (uint32_t)a.k.W), y = (int)(pix / (uint32_t)a.k.W);
                const uint2 gv = a.vd[pix];
                const uint32_t side = gv.x >> 24;
                const float dist = __uint_as_float(gv.y);
                const float3 D = dev::camera_ray(a.k, x, y);
                const float ns = dev::side_sign(side, D);
                pin = make_float4(D.x * dist + a.k.E.x, D.y * dist + a.k.E.y, D.z * dist + a.k.E.z,
                                  __uint_as_float(side_code(side, ns)));
            }
        }
        // input row (K = 32): hash-grid level `half` in columns [8 half, 8 half + 8); half 1
        // also the one-hot side (columns 16-21) and the zero columns 22-31
        {
            float f[8];
            level_features(enc, d, pin.x, pin.y, pin.z, half, f);
            uint32_t w[4];
#pragma unroll
            for (int q = 0; q < 4; q++) w[q] = valid ? pack_bf16(f[2 * q], f[2 * q + 1]) : 0u;
            *reinterpret_cast<uint4*>(A + tc::core_off(tid, half * 8, kIn)) = make_uint4(w[0], w[1], w[2], w[3]);
            if (half) {
                const uint32_t code = __float_as_uint(pin.w);
#pragma unroll
                for (int c = 2; c < kIn / 8; c++) {
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        const uint32_t k = (uint32_t)(c * 8 + 2 * q - 16);
                        w[q] = valid ? pack_bf16(code == k ? 1.0f : 0.0f, code == k + 1u ? 1.0f : 0.0f) : 0u;
                    }
                    *reinterpret_cast<uint4*>(A + tc::core_off(tid, c * 8, kIn)) = make_uint4(w[0], w[1], w[2], w[3]);
                }
            }
        }
        // four layers; between them every thread moves its row from TMEM to A
#pragma unroll 1
        for (int layer = 0; layer < 4; layer++) {
            tc::fence_async_smem();
            tc::fence_before();
            tc::bar_tile(bar);
            if (t == 0 && issue) {
                tc::fence_after();
                const int kdim = layer == 0 ? kIn : H;
                const unsigned char* W = layer == 0 ? W1c : (layer == 1 ? W2c : (layer == 2 ? W3c : W4c));
                const int N = layer == 3 ? K : H;
                const uint32_t id = layer == 3 ? tc::idesc(128, 256) : tc::idesc(128, 64);
                for (int kk = 0; kk < kdim / 16; kk++)
                    tc::mma(dcol, tc::desc(aaddr + kk * 256, 128, kdim * 16),
                            tc::desc(tc::smem_u32(W) + kk * 256, 128, kdim * 16), id, kk > 0 ? 1u : 0u);
                (void)N;
                tc::commit(mbar);
            }
            if (!tc::tile_all(bar, tc::wait(mbar, phase, limit))) {
                ok = false;
                pending = issue;
                if (t == 0 && a.err) atomicOr(a.err, 16u);
                break;
            }
            phase ^= 1u;
            tc::fence_after();
            if (layer < 3) tc::epilogue32(trow, bs + layer * H, A, tid, half);
        }
        if (!ok) break;
        // softmax tables of this pixel's cluster groups [8 half, 8 half + 8) from its logits
        // in TMEM, one pass: each 32-column chunk (two groups) uses its own maximum; the
        // in-group fractions do not depend on it, and the group totals are rescaled to the
        // half's maximum, then (after the exchange) to the row maximum
        float Tg[8], Mc[4];
#pragma unroll
        for (int ch = 0; ch < 4; ch++) {
            const int gc = half * 4 + ch;   // chunk of the row
            float v[32];
            tc::ld32(trow + gc * 32, v);
            float m = -INFINITY;
#pragma unroll
            for (int i = 0; i < 32; i++) {
                v[i] = v[i] * kLog2e + bs[3 * H + gc * 32 + i];   // log2(e) * logit
                m = fmaxf(m, v[i]);
            }
            Mc[ch] = m;
#pragma unroll
            for (int g2 = 0; g2 < 2; g2++) {
                float pre[16];
                float acc = 0.0f;
#pragma unroll
                for (int i = 0; i < 16; i++) {
                    acc += tc::ex2(v[g2 * 16 + i] - m);
                    pre[i] = acc;
                }
                const float sc = acc > 0.0f ? 65535.0f / acc : 0.0f;
                uint32_t pk[8];
#pragma unroll
                for (int i = 0; i < 16; i += 2) {
                    const uint32_t lo = min((uint32_t)(pre[i] * sc), 65535u);
                    const uint32_t hi = i == 14 ? 65535u : min((uint32_t)(pre[i + 1] * sc), 65535u);
                    pk[i / 2] = lo | (hi << 16);
                }
                uint4* dst = reinterpret_cast<uint4*>(fp + (gc * 2 + g2) * 16);
                dst[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                dst[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
                Tg[ch * 2 + g2] = acc;
            }
        }
        tc::fence_before();   // this thread's TMEM reads are complete before the next tile's MMAs
        {
            const float mh = fmaxf(fmaxf(Mc[0], Mc[1]), fmaxf(Mc[2], Mc[3]));
            X[(half * 9) * tc::kTile + tid] = mh;
#pragma unroll
            for (int q = 0; q < 8; q++) X[(half * 9 + 1 + q) * tc::kTile + tid] = Tg[q] * tc::ex2(Mc[q >> 1] - mh);
        }
        tc::bar_tile(bar);    // both halves' tables and totals are written
        float P[16];
        float Z = 0.0f;
        {
            const float m0 = X[tid], m1 = X[9 * tc::kTile + tid];
            const float mx = fmaxf(m0, m1), s0 = tc::ex2(m0 - mx), s1 = tc::ex2(m1 - mx);
#pragma unroll
            for (int q = 0; q < 16; q++) {
                Z += X[((q >> 3) * 9 + 1 + (q & 7)) * tc::kTile + tid] * (q < 8 ? s0 : s1);
                P[q] = Z;
            }
        }
        tc::bar_tile(bar);    // every thread has read X before the next tile writes its input
        const float invZ = 1.0f / Z;
        auto frac = [&](int c) {
            const uint32_t hi = fp[c], lo = (c % gs) ? fp[c - 1] : 0u;
            return (float)(hi - lo) * (1.0f / 65535.0f);
        };
        if (!valid) continue;
        if (a.probs) {
#pragma unroll
            for (int q = half * 8; q < half * 8 + 8; q++) {
                const float gw = q ? P[q] - P[q - 1] : P[0];
                for (int c = q * gs; c < (q + 1) * gs; c++) a.probs[(size_t)j * K + c] = (gw * frac(c)) * invZ;
            }
            continue;
        }
        // the hit pixels this thread draws for: in a shared row the row's entries j + half,
        // j + half + 2, ... (all their candidates), else the row's pixel (every other candidate,
        // the other warpgroup taking the rest; both advance the pixel's RNG alike)
        const float eps = d.eps, invN = 1.0f / (float)a.nlights;
        for (uint32_t jm = j + (span > 1u ? (uint32_t)half : 0u); jm < j + span; jm += 2u) {
            const uint32_t pm = span > 1u ? a.hits[jm] : pix;
            uint32_t s = dev::wang_hash(pm * 2654435761u + a.k.R0 * 0x85EBCA6Bu + 0x9E3779B9u);
            uint2* out = a.cand + jm;
#pragma unroll 4
            for (uint32_t m = 0; m < a.ncand; m++) {
                const float u = dev::rnd(s);
                const float v = dev::rnd(s);
                const float w = dev::rnd(s);
                if (span == 1u && (int)(m & 1u) != half) continue;   // the other warpgroup's candidate
                int c;
                uint32_t e;
                float gw;
                if (u < eps) {
                    e = min((uint32_t)(v * (float)a.nlights), a.nlights - 1u);
                    c = (int)__ldg(a.lightCluster + e);
                    const int q = c / gs;
                    float lo = 0.0f, hi = P[0];
#pragma unroll
                    for (int i = 1; i < 16; i++)
                        if (q == i) { lo = P[i - 1]; hi = P[i]; }
                    gw = hi - lo;
                } else {
                    const float target = v * Z;
                    int q = 0;
                    float lo = 0.0f, hi = P[0];
#pragma unroll
                    for (int i = 0; i < 15; i++)
                        if (target >= P[i]) { q = i + 1; lo = P[i]; hi = P[i + 1]; }
                    gw = hi - lo;
                    const float x = gw > 0.0f ? (target - lo) * (65535.0f / gw) : 0.0f;
                    const uint4 a0 = *reinterpret_cast<const uint4*>(fp + q * 16);
                    const uint4 a1 = *reinterpret_cast<const uint4*>(fp + q * 16 + 8);
                    const uint32_t wv[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
                    int in = 0;
#pragma unroll
                    for (int i = 0; i < 15; i++) in += x >= (float)((wv[i >> 1] >> ((i & 1) * 16)) & 0xFFFFu) ? 1 : 0;
                    c = q * gs + in;
                    const uint32_t off = offs[c], sz = offs[c + 1] - off;
                    e = __ldg(a.clMembers + off + min((uint32_t)(w * (float)sz), sz - 1u));
                }
                const float sz = (float)(offs[c + 1] - offs[c]);
                const float pe = (1.0f - eps) * (((gw * frac(c)) * invZ) / sz) + eps * invN;
                out[(size_t)m * a.candStride] = make_uint2(e, __float_as_uint(pe));
            }
        }
    }
    // a wait gave up: the candidate entries of this half's remaining rows, from the tile it
    // stopped in, are marked as not drawn (light index ~0), which the candidate kernel
    // replaces by uniform candidates - so no entry of an earlier frame, or of memory never
    // written, is read as a draw of this one
    if (!ok && a.cand && !a.samples && !a.probs && half == 0) {
        for (; (size_t)tile * tc::kTile < rows; tile += gridDim.x * 2) {
            const uint32_t row = tile * tc::kTile + tid;
            if (row >= rows) continue;
            uint32_t j = row, span = 1u;
            if (useRows) {
                const uint32_t e = a.rows[row];
                j = e & 0x1FFFFFFFu;
                span = (e >> 29) + 1u;
            }
            for (uint32_t jm = j; jm < j + span && jm < n; jm++)
                for (uint32_t m = 0; m < a.ncand; m++) a.cand[(size_t)m * a.candStride + jm] = make_uint2(0xFFFFFFFFu, 0u);
        }
    }
    // every MMA of this CTA has completed (each was waited for) unless a wait gave up
    // with one in flight: then wait for it once more, with the full limit, before the
    // tensor memory is freed
    if (!ok && pending) tc::wait(mbar, phase, tc::kWaitLimit);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (warp == 0) {
        __syncwarp();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tc::kCols));
    }
}

// ---- training ------------------------------------------------------------------------------
// training batch from the view's final reservoirs: sample b takes the hit pixel at
// stratum b of the hit list; target = cluster of the selected emitter, weight = W * pHat
__global__ void gather_kernel(GatherArgs a) {
    const uint32_t nh = *a.count;
    for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < a.B; b += gridDim.x * blockDim.x) {
        float4 pin = make_float4(0.f, 0.f, 0.f, __uint_as_float(6u));
        uint32_t tgt = 0;
        float w = 0.0f;
        if (nh > 0) {
            const uint32_t j = (uint32_t)(((uint64_t)b * nh + a.offset) / a.B) % nh;
            const uint32_t pix = a.hits[j];
            const uint4 qa = a.hA[pix];
            const uint32_t M = qa.y & 0x1FFFFFFFu;
            const float pH = __uint_as_float(qa.w);
            const float W = __uint_as_float(qa.z) / fmaxf(1e-5f, pH * (float)M);
            if (M > 0u && W > 0.0f && qa.x < a.nlights) {
                w = W * pH;
                tgt = a.lightCluster[qa.x];
            }
            const int x = (int)(pix % (uint32_t)a.k.W), y = (int)(pix / (uint32_t)a.k.W);
            const uint2 gv = a.vd[pix];
            const uint32_t side = gv.x >> 24;
            const float dist = __uint_as_float(gv.y);
            const float3 D = dev::camera_ray(a.k, x, y);
            const float ns = dev::side_sign(side, D);
            pin = make_float4(D.x * dist + a.k.E.x, D.y * dist + a.k.E.y, D.z * dist + a.k.E.z,
                              __uint_as_float(side_code(side, ns)));
        }
        a.samples[b] = pin;
        a.target[b] = tgt;
        a.weight[b] = w;
    }
}

__global__ void encode_kernel(const float* __restrict__ params, Layout L, Dims d, const float4* __restrict__ samples,
                              uint32_t B, float* __restrict__ X) {
    for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x) {
        float xr[kIn];
        input_row(params + L.enc, d, samples[b], xr);
#pragma unroll
        for (int f = 0; f < kIn; f++) X[(size_t)b * kIn + f] = xr[f];
    }
}

// C(m, n) = sum_k A(m, k) B(k, n) with arbitrary strides; 64x64 tiles, 4x4 per thread.
// mode: 0 store, 1 +bias & relu, 2 +bias, 3 store * (mask(m, n) > 0), 4 atomic add (split-K)
__global__ void __launch_bounds__(256) gemm_kernel(GemmArgs g) {
    __shared__ float As[16][68];
    __shared__ float Bs[16][68];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
    const long kbeg = (long)blockIdx.z * g.kchunk;
    const long kend = min((long)g.K, kbeg + g.kchunk);
    float acc[4][4] = {};
    for (long k0 = kbeg; k0 < kend; k0 += 16) {
        for (int e = threadIdx.x; e < 1024; e += 256) {
            int mm, kk;
            if (g.sak == 1) { mm = e >> 4; kk = e & 15; } else { kk = e >> 6; mm = e & 63; }
            const long m = m0 + mm, k = k0 + kk;
            As[kk][mm] = (m < g.M && k < kend) ? g.A[m * g.sam + k * g.sak] : 0.0f;
        }
        for (int e = threadIdx.x; e < 1024; e += 256) {
            int kk, nn;
            if (g.sbn == 1) { kk = e >> 6; nn = e & 63; } else { nn = e >> 4; kk = e & 15; }
            const long k = k0 + kk, nI = n0 + nn;
            Bs[kk][nn] = (k < kend && nI < g.N) ? g.B[k * g.sbk + nI * g.sbn] : 0.0f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; kk++) {
            float av[4], bv[4];
#pragma unroll
            for (int i = 0; i < 4; i++) { av[i] = As[kk][ty * 4 + i]; bv[i] = Bs[kk][tx * 4 + i]; }
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] += av[i] * bv[j];
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const long m = m0 + ty * 4 + i, nI = n0 + tx * 4 + j;
            if (m >= g.M || nI >= g.N) continue;
            float v = acc[i][j];
            float* dst = g.C + m * g.scm + nI * g.scn;
            if (g.mode == 4) { atomicAdd(dst, v); continue; }
            if (g.mode == 1 || g.mode == 2) v += g.bias[nI];
            if (g.mode == 1) v = fmaxf(v, 0.0f);
            if (g.mode == 3 && !(g.mask[m * g.smm + nI] > 0.0f)) v = 0.0f;
            *dst = v;
        }
}

// weighted softmax cross-entropy per row; dZ = w/sum(w) * (softmax - onehot); one warp per row
__global__ void softmax_ce_kernel(float* __restrict__ Z, const uint32_t* __restrict__ target,
                                  const float* __restrict__ weight, uint32_t B, int K, const float* __restrict__ wsum,
                                  float* loss) {
    const int lane = threadIdx.x & 31;
    const float inv = *wsum > 0.0f ? 1.0f / *wsum : 0.0f;
    for (uint32_t b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; b < B; b += (gridDim.x * blockDim.x) >> 5) {
        float* z = Z + (size_t)b * K;
        float mx = -INFINITY;
        for (int c = lane; c < K; c += 32) mx = fmaxf(mx, z[c]);
        for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        float s = 0.0f;
        for (int c = lane; c < K; c += 32) s += expf(z[c] - mx);
        for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        const float w = weight[b] * inv;
        const uint32_t t = target[b];
        float lt = 0.0f;
        for (int c = lane; c < K; c += 32) {
            const float p = expf(z[c] - mx) / s;
            if ((uint32_t)c == t) lt = -(z[c] - mx - logf(s));
            z[c] = w * (p - ((uint32_t)c == t ? 1.0f : 0.0f));
        }
        for (int o = 16; o; o >>= 1) lt += __shfl_xor_sync(0xffffffffu, lt, o);
        if (lane == 0 && w > 0.0f) atomicAdd(loss, w * lt);
    }
}

__global__ void sum_kernel(const float* __restrict__ v, uint32_t n, float* out) {
    float s = 0.0f;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) s += v[i];
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, s);
}

// column sums of a row-major [B][N] matrix into out[N] (bias gradients)
__global__ void colsum_kernel(const float* __restrict__ X, uint32_t B, int N, float* out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    float s = 0.0f;
    for (uint32_t b = blockIdx.y; b < B; b += gridDim.y) s += X[(size_t)b * N + c];
    atomicAdd(&out[c], s);
}

// encoding gradients: scatter dX[:, 0:16] into the hash tables with the trilinear weights
__global__ void encode_backward_kernel(Dims d, Layout L, const float4* __restrict__ samples, const float* __restrict__ dX,
                                       uint32_t B, float* grad) {
    for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x) {
        Corner c;
        const float4 p = samples[b];
        corners(d, p.x, p.y, p.z, c);
#pragma unroll
        for (int l = 0; l < kLevels; l++)
#pragma unroll
            for (int q = 0; q < 8; q++) {
                float* dst = grad + L.enc + (size_t)c.idx[l][q] * kFeat;
                const float w = c.w[l][q];
#pragma unroll
                for (int f = 0; f < kFeat; f++) {
                    const float gv = w * dX[(size_t)b * kIn + l * 8 + f];
                    if (gv != 0.0f) atomicAdd(dst + f, gv);
                }
            }
    }
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ gr, float* __restrict__ m,
                            float* __restrict__ v, size_t n, float lr, float b1, float b2, float eps, float c1, float c2) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float g = gr[i];
        const float mi = b1 * m[i] + (1.0f - b1) * g;
        const float vi = b2 * v[i] + (1.0f - b2) * g * g;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    }
}

__global__ void to_bf16_kernel(const float* __restrict__ src, __nv_bfloat16* __restrict__ dst, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = __float2bfloat16_rn(src[i]);
}

// seeded initialisation: encoding U(-1e-4, 1e-4), weights U(-a, a) with a = sqrt(6 / fan_in), biases 0
__global__ void init_kernel(float* p, Layout L, Dims d, uint32_t seed) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < L.total; i += (size_t)gridDim.x * blockDim.x) {
        uint32_t s = dev::wang_hash((uint32_t)i * 2654435761u ^ dev::wang_hash(seed + (uint32_t)(i >> 32)));
        const float u = dev::rnd(s) * 2.0f - 1.0f;
        float v = 0.0f;
        if (i < L.W1) v = 1e-4f * u;
        else if (i < L.b1) v = u * sqrtf(6.0f / (float)kIn);
        else if (i >= L.W2 && i < L.b2) v = u * sqrtf(6.0f / (float)d.H);
        else if (i >= L.W3 && i < L.b3) v = u * sqrtf(6.0f / (float)d.H);
        else if (i >= L.W4 && i < L.b4) v = u * sqrtf(6.0f / (float)d.H);
        p[i] = v;
    }
}

}  // namespace prop

// ---- host launchers ---------------------------------------------------------------------
namespace prop {

static int sms() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

static size_t infer_fixed_bytes(const Dims& d) {
    const int H = d.H, K = d.K;
    return (size_t)H * (kIn + 8) * 2 + 2 * (size_t)H * (H + 8) * 2 + (size_t)K * (H + 8) * 2 + (3 * H + K) * 4 +
           (size_t)((K + 1 + 3) & ~3) * 4;
}
static size_t infer_warp_bytes(const Dims& d) { return 16 * (kIn + 8) * 2 + 16 * (size_t)(d.K + 8) * 2; }
// warps per block: as many as the shared memory holds, at most 16
static int infer_warps(const Dims& d) {
    const size_t fixed = infer_fixed_bytes(d), per = infer_warp_bytes(d), cap = 227 * 1024;
    if (fixed + per > cap) return 0;
    return (int)std::min<size_t>(16, (cap - fixed) / per);
}

size_t infer_smem_bytes(const Dims& d) { return infer_fixed_bytes(d) + (size_t)std::max(infer_warps(d), 1) * infer_warp_bytes(d); }

bool infer_supported(const Dims& d) {
    return d.H == 64 && d.K >= 16 && d.K % 16 == 0 && d.K <= 1024 && infer_warps(d) >= 1;
}

bool infer_tc_supported(const Dims& d) { return d.H == 64 && d.K == 256; }

static size_t infer_tc_smem_bytes() {
    return (size_t)64 * kIn * 2 + 2 * 64 * 64 * 2 + 256 * 64 * 2 + (3 * 64 + 256) * 4 + 260 * 4 + 2 * 128 * 64 * 2 +
           2 * 128 * (512 + 16) + 2 * 8 + 16;
}

// Table rows for shared network evaluations. The hit list is cut into aligned groups of
// `group` entries (2, 4 or 8); inside a group, a run of consecutive entries whose shading
// points lie on the same voxel side (axis and facing) as the run's first entry, within
// maxDist of it in every coordinate, becomes one row (first entry | (length - 1) << 29);
// an entry that fails the test starts the next run. Rows are appended per warp (one
// atomic each), so their order is not the hit list's.
__global__ void pair_rows_kernel(dev::Frame k, const uint2* __restrict__ vd, const uint32_t* __restrict__ hits,
                                 const uint32_t* __restrict__ count, uint32_t group, float maxDist, uint32_t* rows,
                                 uint32_t* rowCount) {
    const uint32_t n = *count, ng = (n + group - 1u) / group;
    const int lane = threadIdx.x & 31;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < ng; base += stride) {
        const uint32_t i = base + (uint32_t)lane;
        uint32_t emit = 0, r[8];
#pragma unroll
        for (int q = 0; q < 8; q++) r[q] = 0;
        if (i < ng) {
            const uint32_t j0 = i * group, m = min(group, n - j0);
            float3 f = make_float3(0.0f, 0.0f, 0.0f);   // the current run's first shading point
            uint32_t fcode = 0, start = 0;
#pragma unroll
            for (uint32_t q = 0; q < 8; q++) {
                if (q >= m) break;
                const uint32_t pix = hits[j0 + q];
                const int x = (int)(pix % (uint32_t)k.W), y = (int)(pix / (uint32_t)k.W);
                const uint2 gv = vd[pix];
                const uint32_t side = gv.x >> 24;
                const float dist = __uint_as_float(gv.y);
                const float3 D = dev::camera_ray(k, x, y);
                const uint32_t code = side_code(side, dev::side_sign(side, D));
                const float3 sp = make_float3(D.x * dist + k.E.x, D.y * dist + k.E.y, D.z * dist + k.E.z);
                const bool join = q > 0 && code == fcode && fabsf(sp.x - f.x) <= maxDist &&
                                  fabsf(sp.y - f.y) <= maxDist && fabsf(sp.z - f.z) <= maxDist;
                if (q > 0 && !join) {
                    const uint32_t row = (j0 + start) | ((q - start - 1u) << 29);
#pragma unroll
                    for (uint32_t t = 0; t < 8; t++) r[t] = emit == t ? row : r[t];
                    emit++;
                    start = q;
                }
                if (!join) {
                    f = sp;
                    fcode = code;
                }
            }
            const uint32_t row = (j0 + start) | ((m - start - 1u) << 29);
#pragma unroll
            for (uint32_t t = 0; t < 8; t++) r[t] = emit == t ? row : r[t];
            emit++;
        }
        // warp-aggregated append
        uint32_t pre = emit;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, pre, o);
            if (lane >= o) pre += u;
        }
        const uint32_t total = __shfl_sync(0xffffffffu, pre, 31);
        uint32_t at = 0;
        if (lane == 31 && total) at = atomicAdd(rowCount, total);
        at = __shfl_sync(0xffffffffu, at, 31);
        const uint32_t slot = at + pre - emit;
#pragma unroll
        for (uint32_t t = 0; t < 8; t++)
            if (t < emit) rows[slot + t] = r[t];
    }
}

void launch_pair_rows(const dev::Frame& k, const uint2* vd, const uint32_t* hits, const uint32_t* count, uint32_t n,
                      uint32_t group, float maxDist, uint32_t* rows, uint32_t* rowCount, cudaStream_t s) {
    const uint32_t ng = (n + group - 1u) / group;
    const unsigned blocks = (unsigned)std::max<uint32_t>(1, std::min<uint32_t>((ng + 255) / 256, (uint32_t)sms() * 8u));
    pair_rows_kernel<<<blocks, 256, 0, s>>>(k, vd, hits, count, group, maxDist, rows, rowCount);
}

cudaError_t launch_infer(const InferArgs& a, uint32_t max_items, cudaStream_t s) {
    const bool use_tc = a.dims.kernel == 2 || (a.dims.kernel == 0 && infer_tc_supported(a.dims));
    if (use_tc) {
        const size_t sm = infer_tc_smem_bytes();
        cudaError_t e = cudaFuncSetAttribute(infer_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        const unsigned blocks = (unsigned)std::max<uint32_t>(1, std::min<uint32_t>((max_items + 255) / 256, (uint32_t)sms()));
        infer_tc_kernel<<<blocks, 512, sm, s>>>(a);
        return cudaGetLastError();
    }
    const int nw = infer_warps(a.dims);
    const size_t sm = infer_fixed_bytes(a.dims) + (size_t)nw * infer_warp_bytes(a.dims);
    cudaError_t e = cudaFuncSetAttribute(infer_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    const uint32_t per = (uint32_t)nw * 16;
    const unsigned blocks = (unsigned)std::max<uint32_t>(1, std::min<uint32_t>((max_items + per - 1) / per, (uint32_t)sms()));
    infer_kernel<64><<<blocks, nw * 32, sm, s>>>(a);
    return cudaGetLastError();
}

void launch_gather(const GatherArgs& a, cudaStream_t s) { gather_kernel<<<(a.B + 255) / 256, 256, 0, s>>>(a); }

void launch_encode(const float* params, const Layout& L, const Dims& d, const float4* samples, uint32_t B, float* X,
                   cudaStream_t s) {
    encode_kernel<<<(B + 255) / 256, 256, 0, s>>>(params, L, d, samples, B, X);
}

void launch_gemm(const GemmArgs& g0, cudaStream_t s) {
    GemmArgs g = g0;
    if (g.kchunk <= 0) g.kchunk = g.K;
    const unsigned gz = (unsigned)((g.K + g.kchunk - 1) / g.kchunk);
    gemm_kernel<<<dim3((g.N + 63) / 64, (g.M + 63) / 64, gz), 256, 0, s>>>(g);
}

void launch_softmax_ce(float* Z, const uint32_t* target, const float* weight, uint32_t B, int K, const float* wsum,
                       float* loss, cudaStream_t s) {
    softmax_ce_kernel<<<std::max<uint32_t>(1, std::min<uint32_t>((B + 7) / 8, 4096)), 256, 0, s>>>(Z, target, weight, B, K,
                                                                                                   wsum, loss);
}

void launch_sum(const float* v, uint32_t n, float* out, cudaStream_t s) {
    sum_kernel<<<std::max<uint32_t>(1, std::min<uint32_t>((n + 255) / 256, 1024)), 256, 0, s>>>(v, n, out);
}

void launch_colsum(const float* X, uint32_t B, int N, float* out, cudaStream_t s) {
    // enough row groups that every thread sums only ~16 rows (latency, not bandwidth, bound)
    colsum_kernel<<<dim3((N + 127) / 128, std::min<uint32_t>(std::max<uint32_t>(B / 16, 1), 8192)), 128, 0, s>>>(X, B, N, out);
}

void launch_encode_backward(const Dims& d, const Layout& L, const float4* samples, const float* dX, uint32_t B, float* grad,
                            cudaStream_t s) {
    encode_backward_kernel<<<(B + 255) / 256, 256, 0, s>>>(d, L, samples, dX, B, grad);
}

void launch_adam(float* p, const float* g, float* m, float* v, size_t n, float lr, int step, cudaStream_t s) {
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f / (1.0f - powf(b1, (float)step)), c2 = 1.0f / (1.0f - powf(b2, (float)step));
    adam_kernel<<<(unsigned)std::min<size_t>((n + 255) / 256, 4096), 256, 0, s>>>(p, g, m, v, n, lr, b1, b2, 1e-8f, c1, c2);
}

void launch_to_bf16(const float* src, __nv_bfloat16* dst, size_t n, cudaStream_t s) {
    to_bf16_kernel<<<(unsigned)std::min<size_t>((n + 255) / 256, 4096), 256, 0, s>>>(src, dst, n);
}

void launch_init(float* p, const Layout& L, const Dims& d, uint32_t seed, cudaStream_t s) {
    init_kernel<<<(unsigned)std::min<size_t>((L.total + 255) / 256, 8192), 256, 0, s>>>(p, L, d, seed);
}

}  // namespace prop
}  // namespace vxr
