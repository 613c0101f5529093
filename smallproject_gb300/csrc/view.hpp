// view.hpp - the view object behind the C ABI (shared by runtime.cu and proposal_api.cu).
#pragma once
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "camera.hpp"
#include "kernels.hpp"
#include "world.hpp"

namespace vxr {
// GPU copy of a World (runtime.cu)
struct DeviceWorld {
    uint32_t* grid = nullptr;
    uint8_t* uber = nullptr;
    uint32_t* bricks = nullptr;
    uint32_t cap = 0;                // bricks the pool (and the box tables) can hold
    uint32_t high = 0;               // bricks [0, high) are on the device
    uint32_t* bbox = nullptr;        // boxes of the opaque voxels per brick (brick skipping),
    uint32_t* bbox0 = nullptr;       // then those of the non-zero voxels (bbox + cap)
    uint32_t* ubox0 = nullptr;       // box of the non-zero voxels per uber cell (32^3)
    // incremental commits: changed bricks (index list, then their voxels) staged in
    // page-locked memory and copied to `stageDev` (capacity `stageCap` bricks)
    uint32_t* stageHost = nullptr;
    uint32_t* stageDev = nullptr;
    uint32_t stageCap = 0;
    uint32_t lastSent = 0;           // bricks sent by the last commit
    bool lastFull = false;           // the last commit sent everything
    uint4* lraw = nullptr;
    float4* lgeom = nullptr;
    float4* lemit = nullptr;
    uint32_t nl = 0;
    size_t lcap = 0;
    uint64_t version = 0, lightVersion = 0, lightMoveVersion = 0;
    int device = -1;
};
struct Proposal;   // learned candidate proposal state (proposal_api.cu)
// Per-kernel CUDA-event timing of one view: event pairs from a ring, harvested after a
// wait into per-kernel sums (runtime.cu).
struct ViewKernelTimer : KernelTimer {
    static constexpr int kPairs = 4096;
    std::vector<cudaEvent_t> ev;          // 2 * kPairs
    std::vector<int> id;                  // kernel of each pair
    uint64_t next = 0, harvested = 0;
    int open[K_COUNT];                    // pair index of an open mark per kernel
    double sum[K_COUNT] = {};
    uint32_t count[K_COUNT] = {};
    void mark(int k, bool end, cudaStream_t s) override;
    void harvest();
    ~ViewKernelTimer() override;
};
void destroy_proposal(Proposal* p);

// The shadow tracer's brick cache of a view (tuning brick_cache = N > 0): the N bricks its
// shadow rays walked most in a calibration frame, as an open-addressed table of 2N keys
// and their opacity masks (built on the host, copied into shared memory by every CTA).
struct BrickCacheState {
    uint32_t* keys = nullptr;       // device: 2N keys (brick << 11 | slot)
    uint32_t* mask = nullptr;       // device: N x 16 words
    uint32_t* count = nullptr;      // device: brick walks per brick (calibration)
    uint32_t countCap = 0;
    int log2 = 0;                   // log2(2N) of the built table, 0 = none
    int slots = 0;                  // N of the built table
    uint64_t worldVersion = 0;      // world the table was built for
    bool calibrating = false;       // this frame counts brick walks
};
}  // namespace vxr

struct vxr_view {
    vxr_world* world = nullptr;
    vxr_view_desc desc{};
    vxr::CameraState cam;
    vxr::ViewBuffers buf;
    vxr::Tuning tuning;                               // launch parameters (vxr_view_set_tuning)
    int cur = 0;
    cudaStream_t stream = nullptr;
    // vxr_view_render: a frame's front half (primary rays to candidate visibility) runs
    // on stream2 as soon as the previous frame's spatial pass is done (evSpatial), beside
    // that frame's shading; the temporal pass on the view's stream waits for it
    // (evFront). spatialEvOk: evSpatial marks the last frame's spatial pass and nothing
    // has touched the buffers since.
    cudaStream_t stream2 = nullptr;
    cudaEvent_t evSpatial = nullptr, evFront = nullptr, evNow = nullptr;
    bool spatialEvOk = false;
    cudaEvent_t evs[6] = {}, eve[6] = {};            // [0]: vxr_view_timer_*, [1..5]: last frame's stages
    bool ran[6] = {};
    // per-stage event ring over the last kRing frames, harvested by vxr_view_wait
    static constexpr int kRing = 256;
    std::vector<cudaEvent_t> ringS, ringE;             // kRing * 6
    std::vector<uint8_t> ringUsed;                     // kRing * 6
    uint64_t frameSerial = 0, harvested = 0;
    double statSum[6] = {};
    uint32_t statCount[6] = {};
    // vxr_view_render_to_host_async: one event per outstanding image, ticket % kImages
    static constexpr int kImages = 4;
    cudaEvent_t imgEv[kImages] = {};
    uint64_t imgSerial = 0;
    double* sum64 = nullptr;                          // FP64 running sum of shaded frames (rgb)
    uint32_t sum64Count = 0;
    double* errOut = nullptr;                         // [mse sum, mae sum]
    vxr::Proposal* prop = nullptr;                    // learned proposal (optional)
    vxr::BrickCacheState bc;                          // shadow tracer's brick cache (tuning)
    vxr::ViewKernelTimer* ktimer = nullptr;           // per-kernel timing (vxr_view_kernel_timing)
    vxr::dev::Sky* skyDev = nullptr;                  // sky dome (vxr_view_set_sky), null = off
    float4* skyTex = nullptr;
    uint32_t* skyBlueNoise = nullptr;
    bool ktimerOn = false;
    bool useProposal = false;
    bool frameOpen = false;
    vxr_frame_consts k{};
    uint64_t seenLightVersion = 0, seenLightMoveVersion = 0;
    float times[5] = {};
    size_t npx = 0;
};


namespace vxr {
int check_view(vxr_view* v, const char* fn);
dev::World dev_world(vxr_view* v);
dev::Frame dev_frame(const vxr_frame_consts& c);
int ensure_world(vxr_view* v);
void free_view(vxr_view* v);
void harvest(vxr_view* v);
Tuning shape(const vxr_view* v);
int check_tuning(const vxr_tuning* t, const char* fn);
Tuning to_tuning(const vxr_tuning& t);
}  // namespace vxr
