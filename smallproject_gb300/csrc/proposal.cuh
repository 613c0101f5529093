// proposal.cuh - learned candidate proposal: shared definitions (no reference counterpart).
//
// A small network replaces the uniform source pdf of RIS (GenerateLightCandidate,
// tools.cl:593-598, p = 1/N): given the shading point and its voxel side it predicts a
// distribution over K spatial emitter clusters. Sampling: with probability eps an emitter
// uniformly (the defensive part), else cluster c ~ softmax(z) and an emitter uniformly
// inside c, so
//   p_src(e) = (1 - eps) * softmax(z)_c(e) / |c(e)| + eps / N,
// every emitter keeps p_src >= eps / N (RIS weights at most 1/eps times the uniform
// method's) and the RIS weight p_hat / p_src stays consistent.
//
// Network: input 32 = hash-grid encoding (2 levels x 8 features, trilinear, 2^16-entry
// tables, spatial hash of Teschner et al. as used by Instant-NGP) + one-hot voxel side
// (6) + zero padding; 3 hidden layers of width H (ReLU); K logits.
// Parameters live in one FP32 vector (master copy for training with Adam); inference
// uses BF16 copies of the four weight matrices and FP32 accumulation.
#pragma once
#include <cstddef>
#include <cstdint>

namespace vxr {
namespace prop {

constexpr int kIn = 32;          // network input width
constexpr int kFeat = 8;         // features per hash-grid level
constexpr int kLevels = 2;
constexpr int kMaxCand = 32;     // candidates drawn per pixel

struct Dims {
    int H = 64;                  // hidden width
    int K = 256;                 // clusters
    int tableLog2 = 16;          // 2^16 entries per level
    int res0 = 32, res1 = 128;   // grid resolution of the two levels over the 1024^3 map
    float eps = 0.1f;            // defensive mixture weight
    int kernel = 0;              // inference: 0 auto (tcgen05 when supported), 1 mma.sync, 2 tcgen05
};

// Offsets (in floats) of each tensor inside the parameter vector.
struct Layout {
    size_t enc, W1, b1, W2, b2, W3, b3, W4, b4, total;
    size_t tableSize;
};
inline Layout layout(const Dims& d) {
    Layout L;
    L.tableSize = (size_t)1 << d.tableLog2;
    size_t o = 0;
    L.enc = o; o += (size_t)kLevels * L.tableSize * kFeat;
    L.W1 = o; o += (size_t)d.H * kIn;
    L.b1 = o; o += d.H;
    L.W2 = o; o += (size_t)d.H * d.H;
    L.b2 = o; o += d.H;
    L.W3 = o; o += (size_t)d.H * d.H;
    L.b3 = o; o += d.H;
    L.W4 = o; o += (size_t)d.K * d.H;
    L.b4 = o; o += d.K;
    L.total = o;
    return L;
}

}  // namespace prop
}  // namespace vxr
