// kernels.hpp - host-side launchers of the render-path kernels (defined in kernels.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "device.cuh"
#include "proposal.hpp"

namespace vxr {

// Per-view device buffers (layouts described in kernels.cu).
struct ViewBuffers {
    uint2* vd[2] = {nullptr, nullptr};   // current / previous G-buffer plane
    uint32_t* seed = nullptr;
    uint4* cA = nullptr;                  // candidate reservoirs
    float4* cB = nullptr;
    uint4* hA = nullptr;                  // spatial reservoirs = temporal history
    float4* hB = nullptr;
    float4* frame = nullptr;
    float4* accum = nullptr;
    uint32_t* err = nullptr;              // device error flags (bit set per fault kind)
    uint32_t* hits = nullptr;             // hit-pixel list (one entry per pixel at most)
    float4* qA = nullptr;                 // shadow-ray requests: (origin, bits(pixel))
    float4* qB = nullptr;                 //                      (direction, bits(light))
    uint32_t* counters = nullptr;         // [0] hits, [1] requests / [2] fetch of the candidate
                                          // queue, [3] requests / [4] fetch of the shading queue
};

struct LaunchShape {
    int bx = 16, by = 8;                  // threads per block (tile)
};

void launch_build_light_table(const uint4* raw, uint32_t n, float4* geom, float4* emit, cudaStream_t s);
void launch_build_uber(const uint32_t* grid, uint8_t* uber, cudaStream_t s);

// cur: index (0/1) of the current G-buffer plane
void launch_albedo(const dev::World& w, const dev::Frame& k, const ViewBuffers& b, int cur, LaunchShape sh, cudaStream_t s);
// learned proposal inputs of the candidate stage (nullptr = uniform source pdf)
struct LearnedHook {
    prop::InferArgs infer;      // dims, layout, params, BF16 weights
    uint2* cand;                // [pixels][kMaxCand] scratch for drawn clusters
    const uint32_t* clOff;      // cluster CSR on the device
    const uint32_t* clMembers;
};
void launch_candidates(bool point, const dev::World& w, const dev::Frame& k, const ViewBuffers& b, int cur, LaunchShape sh,
                       cudaStream_t s, const LearnedHook* learned = nullptr);
void launch_spatial(bool point, const dev::World& w, const dev::Frame& k, const ViewBuffers& b, int cur, LaunchShape sh,
                    cudaStream_t s);
void launch_shade(bool point, const dev::World& w, const dev::Frame& k, const ViewBuffers& b, int cur, bool fuse_accumulate,
                  LaunchShape sh, cudaStream_t s);
void launch_accumulate(const dev::Frame& k, const ViewBuffers& b, LaunchShape sh, cudaStream_t s);
// converged reference (FP64 running sum of shaded frames) and the MSE / MAE metric
void launch_sum64_add(const float4* frame, double* sum, uint32_t n, cudaStream_t s);
void launch_error(const float4* img, const double* sum, double inv_count, uint32_t n, double* out, cudaStream_t s);

}  // namespace vxr
