// proposal.hpp - launch interface of the learned-proposal kernels (proposal.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "device.cuh"
#include "proposal.cuh"

namespace vxr {
namespace prop {

struct InferArgs {
    Dims dims;
    Layout L;
    const float* params;              // FP32 parameter vector (encoding tables, biases)
    const __nv_bfloat16* wbf;         // BF16 W1 | W2 | W3 | W4
    // render mode: hit pixels of the current frame
    dev::Frame k;
    const uint2* vd;
    const uint32_t* hits;
    const uint32_t* count;            // device hit count (render mode)
    uint32_t ncand;                   // candidates per pixel (<= kMaxCand)
    const uint32_t* clOff;            // cluster c = emitters clMembers[clOff[c] .. clOff[c+1])
    const uint32_t* clMembers;
    const uint32_t* lightCluster;     // cluster of every emitter
    uint32_t nlights;
    uint32_t candStride;              // hits per candidate row of `cand`
    uint2* cand;                      // out: [candidate][candStride] (emitter, bits(p_src))
    uint32_t* err;                    // device error flags (16: a tensor-core wait gave up)
    // sample mode (tests): explicit inputs (x, y, z, bits(side code)) and softmax output
    const float4* samples;
    uint32_t n;
    float* probs;                     // [n][K] when not null (sample mode)
};

struct GatherArgs {
    dev::Frame k;
    const uint2* vd;
    const uint32_t* hits;
    const uint32_t* count;
    const uint4* hA;
    const uint32_t* lightCluster;
    uint32_t nlights;
    uint32_t B;
    uint32_t offset;
    float4* samples;
    uint32_t* target;
    float* weight;
};

struct GemmArgs {
    const float* A;
    long sam, sak;
    const float* B;
    long sbk, sbn;
    float* C;
    long scm, scn;
    int M, N, K;
    const float* bias;
    const float* mask;
    long smm;
    int mode;     // 0 store, 1 +bias relu, 2 +bias, 3 masked by mask > 0, 4 atomic add
    long kchunk;  // split-K chunk (mode 4); 0 = whole K
};

size_t infer_smem_bytes(const Dims& d);
bool infer_supported(const Dims& d);
bool infer_tc_supported(const Dims& d);   // the tcgen05 kernel (H = 64, K = 256)
cudaError_t launch_infer(const InferArgs& a, uint32_t max_items, cudaStream_t s);
void launch_gather(const GatherArgs& a, cudaStream_t s);
void launch_encode(const float* params, const Layout& L, const Dims& d, const float4* samples, uint32_t B, float* X,
                   cudaStream_t s);
void launch_gemm(const GemmArgs& g, cudaStream_t s);
void launch_softmax_ce(float* Z, const uint32_t* target, const float* weight, uint32_t B, int K, const float* wsum,
                       float* loss, cudaStream_t s);
void launch_sum(const float* v, uint32_t n, float* out, cudaStream_t s);
void launch_colsum(const float* X, uint32_t B, int N, float* out, cudaStream_t s);
void launch_encode_backward(const Dims& d, const Layout& L, const float4* samples, const float* dX, uint32_t B,
                            float* grad, cudaStream_t s);
void launch_adam(float* p, const float* g, float* m, float* v, size_t n, float lr, int step, cudaStream_t s);
void launch_to_bf16(const float* src, __nv_bfloat16* dst, size_t n, cudaStream_t s);
void launch_init(float* p, const Layout& L, const Dims& d, uint32_t seed, cudaStream_t s);

}  // namespace prop
}  // namespace vxr
