// noalloc.cu - a render entry point that allocates no memory.
//
// Some callers cannot call cudaMalloc: a host application that already owns all GPU
// memory through its own pool or arena, a plugin loaded into a process whose allocator
// must not be bypassed, or code running while a CUDA graph is being recorded elsewhere.
// vxr_render_frame_noalloc renders one frame for them from device buffers they already
// own (the world grid, its bricks and the light list) into an image buffer they own.
// Everything else the frame needs - G-buffer, seeds, both reservoir planes, the hit
// list, the shadow-ray queue, the 32^3 uber grid, the per-light table, the counters and
// the device error word - lives in one file-scope
// __device__ array of fixed size, which every GPU that loads this library holds until
// the process exits (VXR_NOALLOC_SCRATCH_BYTES = 10,518,784 bytes, 10.0 MiB).
//
// The stage kernels are the ones the view path launches; only the buffers differ.
#include <cstring>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "internal.hpp"
#include "kernels.hpp"
#include "view.hpp"

namespace {

constexpr size_t kMaxPx = VXR_NOALLOC_MAX_PIXELS;
constexpr size_t kMaxLights = VXR_NOALLOC_MAX_LIGHTS;
// layout (byte offsets, every region 256-byte aligned)
constexpr size_t kOffVd = 0;                                   // uint2 [kMaxPx]
constexpr size_t kOffSeed = kOffVd + 8 * kMaxPx;               // uint32 [kMaxPx]
constexpr size_t kOffCA = kOffSeed + 4 * kMaxPx;               // uint4 [kMaxPx]
constexpr size_t kOffCB = kOffCA + 16 * kMaxPx;                // float4 [kMaxPx]
constexpr size_t kOffHA = kOffCB + 16 * kMaxPx;                // uint4 [kMaxPx]
constexpr size_t kOffHB = kOffHA + 16 * kMaxPx;                // float4 [kMaxPx]
constexpr size_t kOffUber = kOffHB + 16 * kMaxPx;              // uint8 [32^3]
constexpr size_t kOffGeom = kOffUber + 32 * 32 * 32;           // float4 [kMaxLights]
constexpr size_t kOffEmit = kOffGeom + 16 * kMaxLights;        // float4 [kMaxLights]
constexpr size_t kOffRaw = kOffEmit + 16 * kMaxLights;         // uint4 [kMaxLights]
constexpr size_t kOffHits = kOffRaw + 16 * kMaxLights;         // uint32 [kMaxPx] hit list
constexpr size_t kOffQA = kOffHits + 4 * kMaxPx;               // float4 [kMaxPx] shadow requests
constexpr size_t kOffQB = kOffQA + 16 * kMaxPx;                // float4 [kMaxPx]
constexpr size_t kOffErr = kOffQB + 16 * kMaxPx;               // uint32 error word, then the work-list counters
constexpr size_t kScratchBytes = kOffErr + 256;
static_assert(kScratchBytes == VXR_NOALLOC_SCRATCH_BYTES, "scratch size must match the header");
static_assert(kOffSeed % 256 == 0 && kOffCA % 256 == 0 && kOffUber % 256 == 0 && kOffGeom % 256 == 0 &&
                  kOffHits % 256 == 0 && kOffQA % 256 == 0 && kOffErr % 256 == 0,
              "scratch regions must stay 256-byte aligned");

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Host-side address of g_noalloc_scratch per device. The symbol's name in host code is
// only a host stand-in, so the device address is looked up once per device with
// cudaGetSymbolAddress while that device is current.
constexpr int kMaxDevices = 64;
unsigned char* g_scratch_ptr[kMaxDevices] = {};
std::mutex g_scratch_mutex;

int scratch_for_current_device(unsigned char** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return vxr::set_error(VXR_E_NODEVICE, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return vxr::set_error(VXR_E_INVALID, "vxr_render_frame_noalloc: device index >= 64");
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return vxr::set_error(VXR_E_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        g_scratch_ptr[dev] = (unsigned char*)p;
    }
    *out = g_scratch_ptr[dev];
    return VXR_OK;
}

// vxr_light (12 bytes) -> the 16-byte records the light-table kernel reads
__global__ void widen_lights_kernel(const vxr_light* __restrict__ in, uint32_t n, uint4* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = make_uint4(in[i].position, in[i].voxel, in[i].size, 0u);
}

// every brick cell of the grid must index inside the caller's brick array
__global__ void check_grid_kernel(const uint32_t* __restrict__ grid, uint32_t nbricks, uint32_t* err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 128u * 128u * 128u) return;
    const uint32_t c = grid[i];
    if ((c & 1u) && (c >> 1) >= nbricks) atomicOr(err, 16u);
}

}  // namespace

#define CUN(call, what)                                                                                     \
    do {                                                                                                    \
        cudaError_t e_ = (call);                                                                            \
        if (e_ != cudaSuccess) return vxr::set_error(VXR_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e_)); \
    } while (0)

extern "C" int vxr_render_frame_noalloc(const uint32_t* grid, const uint32_t* bricks, uint32_t nbricks,
                                        const vxr_light* lights, uint32_t nlights, uint32_t light_model,
                                        const vxr_frame_consts* k, float* out_rgba, void* stream) {
    VXR_CHECK_ARG(grid && bricks && k && out_rgba && (lights || nlights == 0), "vxr_render_frame_noalloc: null argument");
    VXR_CHECK_ARG(light_model == VXR_LIGHTS_AREA || light_model == VXR_LIGHTS_POINT,
                  "vxr_render_frame_noalloc: unknown light model");
    VXR_CHECK_ARG(k->width >= 1 && k->height >= 1, "vxr_render_frame_noalloc: empty frame");
    if ((size_t)k->width * k->height > kMaxPx)
        return vxr::set_error(VXR_E_INVALID, "vxr_render_frame_noalloc: " + std::to_string(k->width) + "x" +
                                                 std::to_string(k->height) + " exceeds the fixed scratch of " +
                                                 std::to_string(kMaxPx) + " pixels");
    if (nlights > kMaxLights)
        return vxr::set_error(VXR_E_INVALID, "vxr_render_frame_noalloc: " + std::to_string(nlights) +
                                                 " lights exceed the fixed scratch of " + std::to_string(kMaxLights));
    VXR_CHECK_ARG(k->numberOfLights == nlights, "vxr_render_frame_noalloc: numberOfLights differs from nlights");
    VXR_CHECK_ARG(k->spatialRadius >= 1, "vxr_render_frame_noalloc: spatialRadius must be >= 1");
    VXR_CHECK_ARG(nbricks >= 1, "vxr_render_frame_noalloc: nbricks must be >= 1");

    unsigned char* s = nullptr;
    if (int r = scratch_for_current_device(&s)) return r;
    cudaStream_t st = (cudaStream_t)stream;
    uint32_t* err = (uint32_t*)(s + kOffErr);
    CUN(cudaMemsetAsync(err, 0, sizeof(uint32_t), st), "clear error word");

    // validate the grid before any traversal reads the bricks through it
    check_grid_kernel<<<(128 * 128 * 128 + 255) / 256, 256, 0, st>>>(grid, nbricks, err);
    CUN(cudaGetLastError(), "grid check");
    uint32_t herr = 0;
    CUN(cudaMemcpyAsync(&herr, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st), "read error word");
    CUN(cudaStreamSynchronize(st), "grid check");
    if (herr & 16u) return vxr::set_error(VXR_E_INVALID, "vxr_render_frame_noalloc: grid references a brick >= nbricks");

    // derive the uber grid and the light table in scratch
    uint4* raw = (uint4*)(s + kOffRaw);
    float4* geom = (float4*)(s + kOffGeom);
    float4* emit = (float4*)(s + kOffEmit);
    if (nlights) {
        widen_lights_kernel<<<(nlights + 255) / 256, 256, 0, st>>>(lights, nlights, raw);
        vxr::launch_build_light_table(raw, nlights, geom, emit, st);
    }
    vxr::launch_build_uber(grid, s + kOffUber, st);
    CUN(cudaGetLastError(), "world kernels");

    vxr::dev::World w;
    w.grid = grid;
    w.uber = s + kOffUber;
    w.bricks = bricks;
    w.bbox = nullptr;   // no room for brick boxes: rays walk every brick they meet
    w.bbox0 = nullptr;
    w.ubox0 = nullptr;
    w.lgeom = geom;
    w.lemit = emit;
    w.nlights = nlights;

    // a single frame: no temporal history is read (the scratch keeps the previous
    // call's contents, which may belong to another world or camera)
    vxr::dev::Frame f = vxr::dev_frame(*k);
    f.restirtemporalframe = 0;
    f.temporal = 0;
    f.accumulate = 0;
    f.sky = nullptr;

    vxr::ViewBuffers b;
    b.vd[0] = (uint2*)(s + kOffVd);
    b.vd[1] = (uint2*)(s + kOffVd);          // previous G-buffer: never read without temporal reuse
    b.seed = (uint32_t*)(s + kOffSeed);
    b.cA = (uint4*)(s + kOffCA);
    b.cB = (float4*)(s + kOffCB);
    b.hA = (uint4*)(s + kOffHA);
    b.hB = (float4*)(s + kOffHB);
    b.frame = (float4*)out_rgba;
    b.accum = (float4*)out_rgba;             // unused: shading runs without the accumulate fusion
    b.err = err;
    b.hits = (uint32_t*)(s + kOffHits);
    b.qA = (float4*)(s + kOffQA);
    b.qB = (float4*)(s + kOffQB);
    b.counters = (uint32_t*)(s + kOffErr + 64);
    const bool point = light_model == VXR_LIGHTS_POINT;
    const vxr::Tuning sh;
    const vxr::BatchDev bd = vxr::single_batch(w, f, b, 0, point, sh);
    const int variant = point ? 1 : 0;
    vxr::launch_batch_albedo(bd, variant, st);
    vxr::launch_batch_candidates(bd, variant, nullptr, st);
    vxr::launch_batch_spatial(bd, variant, st);
    vxr::launch_batch_shade(bd, variant, st);
    CUN(cudaGetLastError(), "stage kernels");
    CUN(cudaMemcpyAsync(&herr, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st), "read error word");
    CUN(cudaStreamSynchronize(st), "vxr_render_frame_noalloc");
    if (herr) return vxr::set_error(VXR_E_DEVICE, "vxr_render_frame_noalloc: " + vxr::device_flags_message(herr));
    return VXR_OK;
}
