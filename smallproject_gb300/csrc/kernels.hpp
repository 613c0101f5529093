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
    uint32_t* hits = nullptr;             // work lists of a single-view batch (BatchDev)
    float4* qA = nullptr;
    float4* qB = nullptr;
    uint32_t* counters = nullptr;         // kCounters words
    // the previous frame's work lists (swapped with the four above as a frame begins):
    // a frame's candidate passes fill their own lists while the previous frame's shading
    // still reads its hit list and shadow-ray queue
    uint32_t* hitsAlt = nullptr;
    float4* qAAlt = nullptr;
    float4* qBAlt = nullptr;
    uint32_t* countersAlt = nullptr;
};

// Work-list counters of a batch: list lengths and work-queue cursors.
enum : int {
    kCtrHits = 0,       // hit-list length
    kCtrQ1 = 1,         // candidate shadow queue: [1] requests, [2] fetch cursor
    kCtrQ2 = 3,         // shading shadow queue:   [3] requests, [4] fetch cursor
    kCtrFinish = 5,     // tile cursors of the persistent pixel stages
    kCtrAlbedo = 6,
    kCtrSpatial = 7,
    kCtrAccum = 8,
    kCounters = 16
};

// learned-proposal candidates read by the candidate loop (null = uniform source pdf)
struct LearnedLists {
    const uint2* cand = nullptr;          // [candidate][stride] (emitter, bits(p_src)), hit j at column j
    uint32_t stride = 0;
};

// Everything a kernel needs about one view of a batch.
struct ViewDev {
    dev::World w;
    dev::Frame k;
    ViewBuffers b;
    int cur = 0;                          // current G-buffer plane
    int point = 0;                        // point-light model
    LearnedLists ll;
    uint32_t tileBase = 0;                // first tile of this view in the batch's tile space
    uint32_t tilesX = 0;
};

// Optional per-kernel CUDA-event timing: the launchers bracket every kernel they launch
// with mark(id, false, s) / mark(id, true, s) when a timer is attached (runtime.cu).
enum KernelId : int {
    K_ALBEDO = 0, K_COMPACT, K_INFER, K_RIS, K_SHADOW_CAND, K_TEMPORAL, K_SPATIAL, K_SHADE_REQ, K_SHADOW_SHADE,
    K_SHADE_FINISH, K_ACCUM, K_TRAIN, K_COUNT
};
struct KernelTimer {
    virtual void mark(int id, bool end, cudaStream_t s) = 0;
    virtual ~KernelTimer() = default;
};

// One launch's work: a single view (read from the kernel parameter `one`) or a table of
// views in device memory. Hit-list entries are (view << 27 | pixel), at most 16 views
// of at most 2^27 pixels each.
constexpr uint32_t kMaxBatchViews = 16;
constexpr int kMaxTileThreads = 256;      // threads of a pixel-stage block (tile_x * tile_y)
struct BatchDev {
    ViewDev one;
    const ViewDev* views = nullptr;       // device table when nviews > 1
    uint32_t nviews = 1;
    uint32_t totalPixels = 0;
    uint32_t totalTiles = 0;
    int tx = 16, ty = 8;                  // tile = block shape of the pixel stages
    int persistent = 0;                   // pixel stages: resident blocks pull tiles from a queue
    int refill = 8;                       // shadow tracer: idle lanes of a warp that trigger a refill
    int burst = 4;                        // shadow tracer: cell visits per lane between refill checks
    int listPerSm = 16;                   // blocks per SM of the hit-list kernels
    int occupancy = 0;                    // 1: register-capped shadow / RIS kernels (more warps per SM)
    int schedule = 0;                     // shadow tracer: 1 = one DDA level per round (the majority's)
    int earlyOut = 0;                     // shadow tracer: stop a walk once its budget cannot reach the emitter
    // shadow tracer's brick cache (single views): the table (global; each CTA copies it
    // into shared memory) when bcLog2 > 0, and per-brick walk counts (calibration) or null
    const uint32_t* bcKeys = nullptr;
    const uint32_t* bcMask = nullptr;
    uint32_t* bcCount = nullptr;
    int bcLog2 = 0;
    int fuse = 0;                         // shading also accumulates
    int sky = 0;                          // some view has a sky dome (shading runs its variant)
    uint32_t* hits = nullptr;             // hit list over all views
    float4* qA = nullptr;                 // shadow-ray requests: (origin, bits(entry))
    float4* qB = nullptr;                 //                      (direction, bits(light))
    uint32_t* counters = nullptr;         // kCounters words
    KernelTimer* timer = nullptr;         // host object (never dereferenced on the device)
};

// Launch parameters that change speed but never results (autotuned per configuration).
struct Tuning {
    int bx = 16, by = 8;                  // threads per block (tile) of the pixel stages
    int persistent = 0;
    int refill = 8;
    int burst = 4;
    int listPerSm = 16;
    int occupancy = 0;
    int schedule = 0;
    int earlyOut = 0;
    int brickCache = 0;
};

size_t brick_cache_smem(int log2);   // shared memory of the shadow tracer's brick-cache variant
void launch_build_light_table(const uint4* raw, uint32_t n, float4* geom, float4* emit, cudaStream_t s);
void launch_build_uber(const uint32_t* grid, uint8_t* uber, cudaStream_t s);
void launch_build_brick_boxes(const uint32_t* bricks, const uint32_t* list, uint32_t n, uint32_t* bbox, uint32_t* bbox0,
                              cudaStream_t s);
void launch_commit_bricks(const uint32_t* list, const uint32_t* voxels, uint32_t n, uint32_t* bricks, cudaStream_t s);
void launch_build_uber_boxes(const uint32_t* grid, const uint32_t* bbox0, uint32_t* ubox0, cudaStream_t s);

// learned proposal inputs of the candidate stage
struct LearnedHook {
    prop::InferArgs infer;      // dims, layout, params, BF16 weights
    uint2* cand;                // [kMaxCand][pixels] scratch for the drawn candidates
    uint32_t* rows;             // shared evaluations: table rows [pixels] and their count (null: one per pixel)
    uint32_t* rowCount;
    uint32_t group;             // hit entries a shared evaluation may serve (2, 4 or 8)
    float pairDist;             // largest per-coordinate distance within a shared row (voxels)
    const uint32_t* clOff;      // cluster CSR on the device
    const uint32_t* clMembers;
    const uint32_t* lightCluster;
};

// A batch of one view over its own list buffers.
BatchDev single_batch(const dev::World& w, const dev::Frame& k, const ViewBuffers& b, int cur, bool point, const Tuning& tu);
void apply_tuning(BatchDev& bd, const Tuning& tu);

// Stage launchers over a batch. variant: 0 single view / area lights, 1 single view /
// point lights, 2 view table (light model per view). A learned proposal needs variant 0/1.
void launch_batch_albedo(const BatchDev& bd, int variant, cudaStream_t s);
void launch_path_trace(const BatchDev& bd, cudaStream_t s);
// tail, ev (optional): the temporal pass runs on stream tail after an event ev that s
// records behind the candidate visibility pass
void launch_batch_candidates(const BatchDev& bd, int variant, const LearnedHook* learned, cudaStream_t s,
                             cudaStream_t tail = nullptr, cudaEvent_t ev = nullptr);
void launch_batch_spatial(const BatchDev& bd, int variant, cudaStream_t s);
void launch_batch_shade(const BatchDev& bd, int variant, cudaStream_t s);
void launch_batch_accumulate(const BatchDev& bd, int variant, cudaStream_t s);

// converged reference (FP64 running sum of shaded frames) and the MSE / MAE metric
void launch_sum64_add(const float4* frame, double* sum, uint32_t n, cudaStream_t s);
void launch_error(const float4* img, const double* sum, double inv_count, uint32_t n, double* out, cudaStream_t s);

}  // namespace vxr
