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
    uint32_t waitLimit;               // tries of each in-loop tensor-core wait (0: the full limit)
    uint32_t skipMma;                 // test only: issue no MMA, so every wait runs out with nothing in flight
    // tcgen05 render mode with sharing: the table rows (pair_rows_kernel): row r serves hit
    // entries (rows[r] & 0x1FFFFFFF) + [0, (rows[r] >> 29) + 1); null: one row per hit entry
    const uint32_t* rows;
    const uint32_t* rowCount;
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

// fused training step on the tensor cores (train.cu), hidden 64 and 16 <= K <= 256
constexpr int kTrainWarpBytes = 16 * (kIn + 8) * 2 + 16 * (64 + 8) * 2 + 16 * 16 * 4;   // X, H1, dX per warp

struct TrainArgs {
    Dims dims;
    Layout L;
    const float* params;              // FP32 master (hash tables, biases)
    const __nv_bfloat16* wbf;         // BF16 W1 | W2 | W3 | W4
    const float4* samples;            // batch: (x, y, z, bits(side code))
    const uint32_t* target;           // cluster of the selected emitter
    const float* weight;              // W * pHat (0: no contribution)
    const float* wpart;               // weight sums per wsum block
    uint32_t nwpart;
    uint32_t B;
    float* grads;                     // full gradient vector; the hash-table part must be zero
    uint4* frag;                      // weight-gradient operands as mma fragments (train_frag_bytes)
    float* partials;                  // [chunk][MLP parameters] gradient sums
    float* lossPart;                  // [CTA] loss sums
};

struct WgradArgs {
    const uint4* frag;
    uint32_t ntiles, chunkTiles;
    int K, nmlp;
    float* partials;
};

struct ReduceArgs {
    const float* partials;
    int nparts, nmlp, K;              // rows of the partial-gradient table
    const float* lossPart;
    int nloss;                        // entries of lossPart
    const float* wpart;
    uint32_t nwpart;
    float* grads;                     // grads + L.W1
    float* params;                    // params + L.W1
    float* m;
    float* v;
    __nv_bfloat16* wbf;
    int apply;                        // 0: gradients only (no update)
    float lr, b1, b2, eps, c1, c2;
    float* scal;                      // out: [loss, weight sum]
};

bool train_supported(const Dims& d);
int train_mlp_count(const Dims& d);
size_t train_smem_bytes(const Dims& d);
size_t train_frag_bytes(const Dims& d, uint32_t B);
uint32_t train_chunks(uint32_t B);   // rows of the partial-gradient table for a batch of B
int train_max_ctas();
uint32_t train_wsum_blocks();
void launch_wsum(const float* w, uint32_t B, float* part, cudaStream_t s);
cudaError_t launch_train(const TrainArgs& a, cudaStream_t s, int* nparts, int* nloss);
void launch_train_reduce(const ReduceArgs& r, cudaStream_t s);
void launch_adam_enc(float* p, float* g, float* m, float* v, size_t n, float lr, int step, cudaStream_t s);

size_t infer_smem_bytes(const Dims& d);
bool infer_supported(const Dims& d);
bool infer_tc_supported(const Dims& d);   // the tcgen05 kernel (H = 64, K = 256)
cudaError_t launch_infer(const InferArgs& a, uint32_t max_items, cudaStream_t s);
// rows of the tcgen05 inference that shares one network evaluation between up to `group`
// (2, 4 or 8) consecutive hit entries whose shading points lie on the same voxel side as the
// first one's within maxDist voxels (each coordinate); other entries start rows of their
// own. rowCount must be zero before.
void launch_pair_rows(const dev::Frame& k, const uint2* vd, const uint32_t* hits, const uint32_t* count, uint32_t n,
                      uint32_t group, float maxDist, uint32_t* rows, uint32_t* rowCount, cudaStream_t s);
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
