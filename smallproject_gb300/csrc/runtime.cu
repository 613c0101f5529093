// runtime.cu - device world copies, views (one camera on one world) and the render
// orchestration behind the C ABI: the GB300 counterpart of World::Render/Commit
// (template/world.cpp:2127-2483) on one CUDA stream per view.
#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "camera.hpp"
#include "internal.hpp"
#include "kernels.hpp"
#include "world.hpp"
#include "view.hpp"

namespace vxr {



static int cuda_fail(cudaError_t e, const char* what) {
    return set_error(VXR_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define CU(call, what)                                  \
    do {                                                \
        cudaError_t e_ = (call);                        \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

void release_device_world(World& w) {
    DeviceWorld* d = w.dev;
    if (!d) return;
    cudaFree(d->grid);
    cudaFree(d->uber);
    cudaFree(d->bricks);
    cudaFree(d->bbox);
    cudaFree(d->ubox0);
    cudaFree(d->stageDev);
    cudaFreeHost(d->stageHost);
    cudaFree(d->lraw);
    cudaFree(d->lgeom);
    cudaFree(d->lemit);
    delete d;
    w.dev = nullptr;
}

// World::Commit (world.cpp:2357-2420) with the commit kernel (kernels.cl:448-477): bring
// the device copy up to date. Waits for all device work first (frames in flight read the
// buffers this writes). Sends everything when there is no copy yet, after clear() or a
// scene build, or when the brick pool outgrew the device pool (which is then reallocated
// with headroom); otherwise only the bricks marked dirty (their voxels, then a scatter
// kernel), the grid when it changed, and the lights when they changed, and rebuilds the
// derived tables of what changed.
static int upload(World& w) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return set_error(VXR_E_NODEVICE, "no CUDA device visible");
    int dev = 0;
    CU(cudaGetDevice(&dev), "cudaGetDevice");
    const bool full = w.fullDirty || !w.dev || !w.dev->grid || w.dev->device != dev || w.brickHigh > w.dev->cap;
    // every brick cell must point into the pool (edits through World::set / optimize keep
    // this, so incremental commits skip the scan)
    if (full)
        for (uint32_t i = 0; i < kGridSize; i++)
            if ((w.grid[i] & 1u) && (w.grid[i] >> 1) >= w.brickHigh)
                return set_error(VXR_E_STATE, "vxr_world_upload: grid cell references a brick outside the pool");
    CU(cudaDeviceSynchronize(), "upload: wait for device work");
    if (!w.dev) w.dev = new DeviceWorld();
    DeviceWorld& d = *w.dev;
    d.device = dev;
    if (!d.grid) CU(cudaMalloc(&d.grid, kGridSize * sizeof(uint32_t)), "cudaMalloc(grid)");
    if (!d.uber) CU(cudaMalloc(&d.uber, 32 * 32 * 32), "cudaMalloc(uber)");
    if (!d.ubox0) CU(cudaMalloc(&d.ubox0, 32 * 32 * 32 * sizeof(uint32_t)), "cudaMalloc(uber boxes)");
    uint32_t sent = 0;
    if (full) {
        if (w.brickHigh > d.cap || !d.bricks) {
            // headroom for bricks split by later edits without a full upload
            const uint32_t cap = std::max<uint32_t>(w.brickHigh + w.brickHigh / 8u + 256u, 1u);
            cudaFree(d.bricks);
            cudaFree(d.bbox);
            d.bricks = nullptr;
            d.bbox = nullptr;
            d.cap = 0;
            CU(cudaMalloc(&d.bricks, (size_t)cap * kBrick * sizeof(uint32_t)), "cudaMalloc(bricks)");
            CU(cudaMalloc(&d.bbox, (size_t)cap * 2u * sizeof(uint32_t)), "cudaMalloc(brick boxes)");
            d.cap = cap;
        }
        d.bbox0 = d.bbox + d.cap;
        CU(cudaMemcpy(d.grid, w.grid.data(), kGridSize * sizeof(uint32_t), cudaMemcpyHostToDevice), "upload grid");
        if (w.brickHigh)
            CU(cudaMemcpy(d.bricks, w.bricks.data(), (size_t)w.brickHigh * kBrick * sizeof(uint32_t), cudaMemcpyHostToDevice),
               "upload bricks");
        launch_build_brick_boxes(d.bricks, nullptr, w.brickHigh, d.bbox, d.bbox0, 0);
        sent = w.brickHigh;
    } else if (w.dirtyCount) {
        if (w.dirtyCount > d.stageCap) {
            cudaFreeHost(d.stageHost);
            cudaFree(d.stageDev);
            d.stageHost = nullptr;
            d.stageDev = nullptr;
            d.stageCap = 0;
            const uint32_t cap = std::max<uint32_t>(w.dirtyCount + w.dirtyCount / 2u, 64u);
            const size_t bytes = (size_t)cap * (kBrick + 1u) * sizeof(uint32_t);
            CU(cudaMallocHost(&d.stageHost, bytes), "cudaMallocHost(commit staging)");
            CU(cudaMalloc(&d.stageDev, bytes), "cudaMalloc(commit staging)");
            d.stageCap = cap;
        }
        // staging: the brick indices, then (at a 16-byte aligned offset) their voxels
        const uint32_t n = w.dirtyCount;
        const size_t voxOff = ((size_t)n + 3u) & ~(size_t)3u;
        uint32_t* list = d.stageHost;
        uint32_t* vox = d.stageHost + voxOff;
        uint32_t k = 0;
        for (size_t wd = 0; wd < w.dirty.size() && k < n; wd++) {
            for (uint32_t m = w.dirty[wd]; m; m &= m - 1u) {
                const uint32_t b = (uint32_t)(wd * 32u) + (uint32_t)__builtin_ctz(m);
                if (b >= w.brickHigh) continue;
                list[k] = b;
                std::memcpy(vox + (size_t)k * kBrick, &w.bricks[(size_t)b * kBrick], kBrick * sizeof(uint32_t));
                k++;
            }
        }
        sent = k;
        if (k) {
            const size_t bytes = (voxOff + (size_t)k * kBrick) * sizeof(uint32_t);
            CU(cudaMemcpy(d.stageDev, d.stageHost, bytes, cudaMemcpyHostToDevice), "commit bricks");
            launch_commit_bricks(d.stageDev, d.stageDev + voxOff, k, d.bricks, 0);
            launch_build_brick_boxes(d.bricks, d.stageDev, k, d.bbox, d.bbox0, 0);
        }
    }
    if (full || w.gridDirty) {
        if (!full) {
            // the changed y-layers of the grid (128^2 cells each), runs copied together
            const size_t layer = (size_t)kGrid * kGrid;
            for (uint32_t y = 0; y < kGrid;) {
                if (!(w.gridRows[y >> 5] >> (y & 31) & 1u)) { y++; continue; }
                uint32_t e = y + 1;
                while (e < kGrid && (w.gridRows[e >> 5] >> (e & 31) & 1u)) e++;
                CU(cudaMemcpy(d.grid + y * layer, w.grid.data() + y * layer, (e - y) * layer * sizeof(uint32_t),
                              cudaMemcpyHostToDevice),
                   "upload grid layers");
                y = e;
            }
        }
        launch_build_uber(d.grid, d.uber, 0);
    }
    if (full || w.gridDirty || sent) launch_build_uber_boxes(d.grid, d.bbox0, d.ubox0, 0);
    if (full || d.lightVersion != w.lightVersion || d.lightMoveVersion != w.lightMoveVersion) {
        const uint32_t nl = (uint32_t)w.lights.size();
        const size_t need = std::max<uint32_t>(nl, 1u);
        if (need > d.lcap) {
            cudaFree(d.lraw);
            cudaFree(d.lgeom);
            cudaFree(d.lemit);
            d.lraw = nullptr; d.lgeom = nullptr; d.lemit = nullptr;
            CU(cudaMalloc(&d.lraw, need * sizeof(uint4)), "cudaMalloc(lights)");
            CU(cudaMalloc(&d.lgeom, need * sizeof(float4)), "cudaMalloc(light geom)");
            CU(cudaMalloc(&d.lemit, need * sizeof(float4)), "cudaMalloc(light emit)");
            d.lcap = need;
        }
        std::vector<uint4> raw(need, make_uint4(0, 0, 1, 0));
        for (uint32_t i = 0; i < nl; i++) raw[i] = make_uint4(w.lights[i].position, w.lights[i].voxel, w.lights[i].size, 0);
        CU(cudaMemcpy(d.lraw, raw.data(), need * sizeof(uint4), cudaMemcpyHostToDevice), "upload lights");
        launch_build_light_table(d.lraw, (uint32_t)need, d.lgeom, d.lemit, 0);
        d.nl = nl;
    }
    CU(cudaGetLastError(), "world kernels launch");
    CU(cudaDeviceSynchronize(), "world kernels");
    d.high = w.brickHigh;
    d.version = w.version;
    d.lightVersion = w.lightVersion;
    d.lightMoveVersion = w.lightMoveVersion;
    d.lastSent = sent;
    d.lastFull = full;
    std::fill(w.dirty.begin(), w.dirty.end(), 0u);
    w.dirtyCount = 0;
    w.gridDirty = false;
    std::fill(std::begin(w.gridRows), std::end(w.gridRows), 0u);
    w.fullDirty = false;
    return VXR_OK;
}

}  // namespace vxr


namespace vxr {
bool learned_hook(vxr_view* v, LearnedHook* h, cudaStream_t s);
int proposal_frame_train(vxr_view* v);
void proposal_join(vxr_view* v);   // the view stream waits for the frame's training step
}

using vxr::set_error;

namespace vxr {

int check_view(vxr_view* v, const char* fn) {
    if (!v) return set_error(VXR_E_INVALID, std::string(fn) + ": null view");
    return VXR_OK;
}

vxr::dev::World dev_world(vxr_view* v) {
    const vxr::DeviceWorld& d = *v->world->w.dev;
    vxr::dev::World w;
    w.grid = d.grid;
    w.uber = d.uber;
    w.bricks = d.bricks;
    w.bbox = d.bbox;
    w.bbox0 = d.bbox0;
    w.ubox0 = d.ubox0;
    w.lgeom = d.lgeom;
    w.lemit = d.lemit;
    w.nlights = d.nl;
    return w;
}

vxr::dev::Frame dev_frame(const vxr_frame_consts& c) {
    vxr::dev::Frame k;
    k.E = make_float3(c.E[0], c.E[1], c.E[2]);
    k.p0 = make_float3(c.p0[0], c.p0[1], c.p0[2]);
    k.dx = make_float3(c.p1[0] - c.p0[0], c.p1[1] - c.p0[1], c.p1[2] - c.p0[2]);
    k.dy = make_float3(c.p2[0] - c.p0[0], c.p2[1] - c.p0[1], c.p2[2] - c.p0[2]);
    k.frame = c.frame;
    k.oorx = c.oneOverRes[0];
    k.oory = c.oneOverRes[1];
    k.Nl = make_float4(c.Nleft[0], c.Nleft[1], c.Nleft[2], c.Nleft[3]);
    k.Nr = make_float4(c.Nright[0], c.Nright[1], c.Nright[2], c.Nright[3]);
    k.Nt = make_float4(c.Ntop[0], c.Ntop[1], c.Ntop[2], c.Ntop[3]);
    k.Nb = make_float4(c.Nbottom[0], c.Nbottom[1], c.Nbottom[2], c.Nbottom[3]);
    k.R0 = c.R0;
    k.framecount = c.framecount;
    k.restirtemporalframe = c.restirtemporalframe;
    k.spatial = c.spatial;
    k.temporal = c.temporal;
    k.accumulate = c.accumulate;
    k.nlights = c.numberOfLights;
    k.ncand = c.numberOfLights < c.numberOfCandidates ? c.numberOfLights : c.numberOfCandidates;
    k.maxTemporal = c.numberOfMaxTemporalImportance;
    k.radius = c.spatialRadius;
    k.taps = c.spatialTaps;
    k.W = (int32_t)c.width;
    k.H = (int32_t)c.height;
    k.sky = nullptr;
    return k;
}

int ensure_world(vxr_view* v) {
    vxr::World& w = v->world->w;
    if (!w.dev || w.dev->version != w.version) {
        const int r = vxr::upload(w);
        if (r != VXR_OK) return r;
    }
    return VXR_OK;
}

void free_view(vxr_view* v) {
    vxr::ViewBuffers& b = v->buf;
    cudaFree(b.vd[0]); cudaFree(b.vd[1]); cudaFree(b.seed);
    cudaFree(b.cA); cudaFree(b.cB); cudaFree(b.hA); cudaFree(b.hB);
    cudaFree(b.frame); cudaFree(b.accum); cudaFree(b.err);
    cudaFree(b.hits); cudaFree(b.qA); cudaFree(b.qB); cudaFree(b.counters);
    cudaFree(b.hitsAlt); cudaFree(b.qAAlt); cudaFree(b.qBAlt); cudaFree(b.countersAlt);
    cudaFree(v->sum64); cudaFree(v->errOut);
    cudaFree(v->skyDev); cudaFree(v->skyTex); cudaFree(v->skyBlueNoise);
    cudaFree(v->bc.keys); cudaFree(v->bc.mask); cudaFree(v->bc.count);
    if (v->prop) vxr::destroy_proposal(v->prop);
    v->prop = nullptr;
    delete v->ktimer;
    v->ktimer = nullptr;
    for (int i = 0; i < 6; i++) {
        if (v->evs[i]) cudaEventDestroy(v->evs[i]);
        if (v->eve[i]) cudaEventDestroy(v->eve[i]);
    }
    for (cudaEvent_t e : v->ringS) cudaEventDestroy(e);
    for (cudaEvent_t e : v->ringE) cudaEventDestroy(e);
    for (cudaEvent_t e : v->imgEv)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : {v->evSpatial, v->evFront, v->evNow})
        if (e) cudaEventDestroy(e);
    if (v->stream2) cudaStreamDestroy(v->stream2);
    if (v->stream) cudaStreamDestroy(v->stream);
}

// Accumulate the stage durations of every finished frame still in the ring.
void harvest(vxr_view* v) {
    const uint64_t from = v->frameSerial > (uint64_t)vxr_view::kRing ? std::max(v->harvested, v->frameSerial - vxr_view::kRing)
                                                                       : v->harvested;
    for (uint64_t f = from; f < v->frameSerial; f++) {
        const int slot = (int)(f % vxr_view::kRing);
        for (int s = 1; s <= 5; s++) {
            const int i = slot * 6 + s;
            if (!v->ringUsed[i]) continue;
            float ms = 0.0f;
            if (cudaEventElapsedTime(&ms, v->ringS[i], v->ringE[i]) == cudaSuccess) {
                v->statSum[s] += ms;
                v->statCount[s]++;
            }
            v->ringUsed[i] = 0;
        }
    }
    v->harvested = v->frameSerial;
}

void ViewKernelTimer::mark(int k, bool end, cudaStream_t s) {
    if (!end) {
        const int slot = (int)(next % kPairs);
        open[k] = slot;
        id[slot] = k;
        next++;
        cudaEventRecord(ev[2 * slot], s);
    } else {
        cudaEventRecord(ev[2 * open[k] + 1], s);
    }
}

void ViewKernelTimer::harvest() {
    const uint64_t from = next > (uint64_t)kPairs ? std::max(harvested, next - kPairs) : harvested;
    for (uint64_t i = from; i < next; i++) {
        const int slot = (int)(i % kPairs);
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, ev[2 * slot], ev[2 * slot + 1]) == cudaSuccess) {
            sum[id[slot]] += ms;
            count[id[slot]]++;
        }
    }
    harvested = next;
}

ViewKernelTimer::~ViewKernelTimer() {
    for (cudaEvent_t e : ev)
        if (e) cudaEventDestroy(e);
}

vxr::Tuning shape(const vxr_view* v) {
    vxr::Tuning s = v->tuning;
    if (v->desc.tile_x) s.bx = (int)v->desc.tile_x;
    if (v->desc.tile_y) s.by = (int)v->desc.tile_y;
    return s;
}

}  // namespace vxr

using vxr::check_view;
using vxr::dev_world;
using vxr::dev_frame;
using vxr::ensure_world;
using vxr::free_view;
using vxr::harvest;
using vxr::shape;

#define CUV(call, what)                                                                   \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) return set_error(VXR_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e_)); \
    } while (0)

namespace vxr {
// Brick cache: a frame that finds no table for the tuning's size and the world's version
// calibrates (its shadow passes count brick walks); at its end the N most walked bricks
// become the table. Both run only when the tuning asks for a cache.
int brick_cache_begin(vxr_view* v) {
    BrickCacheState& c = v->bc;
    const int want = v->tuning.brickCache;
    const uint64_t ver = v->world->w.version;
    if (want <= 0 || (c.log2 > 0 && c.slots == want && c.worldVersion == ver)) return VXR_OK;
    const uint32_t nb = std::max<uint32_t>(v->world->w.brickHigh, 1u);
    if (c.countCap < nb) {
        cudaFree(c.count);
        c.count = nullptr;
        c.countCap = 0;
        CUV(cudaMalloc(&c.count, nb * sizeof(uint32_t)), "cudaMalloc(brick walk counts)");
        c.countCap = nb;
    }
    CUV(cudaMemsetAsync(c.count, 0, nb * sizeof(uint32_t), v->stream), "clear brick walk counts");
    c.calibrating = true;
    return VXR_OK;
}

int brick_cache_end(vxr_view* v) {
    BrickCacheState& c = v->bc;
    if (!c.calibrating) return VXR_OK;
    c.calibrating = false;
    const World& w = v->world->w;
    const uint32_t nb = std::max<uint32_t>(w.brickHigh, 1u);
    std::vector<uint32_t> cnt(nb);
    CUV(cudaMemcpyAsync(cnt.data(), c.count, nb * sizeof(uint32_t), cudaMemcpyDeviceToHost, v->stream),
        "read brick walk counts");
    CUV(cudaStreamSynchronize(v->stream), "brick cache calibration");
    const int N = v->tuning.brickCache;
    std::vector<uint32_t> order;
    for (uint32_t b = 0; b < nb; b++)
        if (cnt[b] > 0) order.push_back(b);
    const size_t top = std::min<size_t>((size_t)N, order.size());
    std::partial_sort(order.begin(), order.begin() + top, order.end(),
                      [&](uint32_t a, uint32_t b) { return cnt[a] != cnt[b] ? cnt[a] > cnt[b] : a < b; });
    int log2 = 1;
    while ((1 << log2) < 2 * N) log2++;
    const uint32_t nk = 1u << log2;
    std::vector<uint32_t> keys(nk, dev::kNoKey), mask((size_t)(nk / 2) * 16u, 0u);
    uint32_t slot = 0;
    for (size_t i = 0; i < top; i++) {
        const uint32_t b = order[i];
        if (b >= (1u << 21)) continue;
        const uint32_t h = (b * 2654435761u) >> (32 - log2);
        for (uint32_t p = 0; p < 4; p++) {
            uint32_t& key = keys[(h + p) & (nk - 1u)];
            if (key != dev::kNoKey) continue;
            key = (b << 11) | slot;
            for (uint32_t vi = 0; vi < 512; vi++)
                if (((w.bricks[(size_t)b * 512 + vi] >> 12) & 15u) == 15u) mask[(size_t)slot * 16 + (vi >> 5)] |= 1u << (vi & 31u);
            slot++;
            break;
        }
    }
    if (c.log2 != log2) {
        cudaFree(c.keys);
        cudaFree(c.mask);
        c.keys = nullptr;
        c.mask = nullptr;
        c.log2 = 0;
        CUV(cudaMalloc(&c.keys, nk * sizeof(uint32_t)), "cudaMalloc(brick cache)");
        CUV(cudaMalloc(&c.mask, mask.size() * sizeof(uint32_t)), "cudaMalloc(brick cache)");
    }
    CUV(cudaMemcpy(c.keys, keys.data(), nk * sizeof(uint32_t), cudaMemcpyHostToDevice), "upload brick cache");
    CUV(cudaMemcpy(c.mask, mask.data(), mask.size() * sizeof(uint32_t), cudaMemcpyHostToDevice), "upload brick cache");
    c.log2 = log2;
    c.slots = N;
    c.worldVersion = w.version;
    return VXR_OK;
}

}  // namespace vxr

extern "C" {

int vxr_world_upload(vxr_world* w) {
    VXR_CHECK_ARG(w, "vxr_world_upload: null world");
    w->w.mark_all();
    return vxr::upload(w->w);
}

int vxr_world_commit(vxr_world* w, uint32_t* bricks_sent, int* full) {
    VXR_CHECK_ARG(w, "vxr_world_commit: null world");
    const int r = vxr::upload(w->w);
    if (r != VXR_OK) return r;
    if (bricks_sent) *bricks_sent = w->w.dev->lastSent;
    if (full) *full = w->w.dev->lastFull ? 1 : 0;
    return VXR_OK;
}

int vxr_world_pending(const vxr_world* w, uint32_t* dirty_bricks, int* grid_changed, int* full) {
    VXR_CHECK_ARG(w, "vxr_world_pending: null world");
    const vxr::World& W = w->w;
    const bool everything = W.fullDirty || !W.dev || W.brickHigh > W.dev->cap;
    if (dirty_bricks) *dirty_bricks = everything ? W.brickHigh : W.dirtyCount;
    if (grid_changed) *grid_changed = (everything || W.gridDirty) ? 1 : 0;
    if (full) *full = everything ? 1 : 0;
    return VXR_OK;
}

int vxr_world_device_bytes(const vxr_world* w, uint64_t* bytes) {
    VXR_CHECK_ARG(w && bytes, "vxr_world_device_bytes: null argument");
    const vxr::DeviceWorld* d = w->w.dev;
    // grid, uber grid and its boxes, bricks and their boxes, light tables
    *bytes = d ? (uint64_t)(vxr::kGridSize * 4 + 32768 + 32768 * 4 + (uint64_t)d->cap * (vxr::kBrick * 4 + 8) +
                            (uint64_t)d->stageCap * (vxr::kBrick + 1) * 4 + d->lcap * 48)
               : 0;
    return VXR_OK;
}

int vxr_view_default_desc(vxr_view_desc* d) {
    VXR_CHECK_ARG(d, "vxr_view_default_desc: null desc");
    std::memset(d, 0, sizeof(*d));
    d->width = 1600;   // common.h:2-3
    d->height = 1024;
    d->light_model = VXR_LIGHTS_AREA;
    d->num_candidates = 32;
    d->spatial_taps = 5;
    d->spatial_radius = 30;
    d->temporal_max_importance = 20;
    d->spatial = 1;
    d->temporal = 1;
    d->accumulate = 0;
    d->rng_seed = 0x12345678u;
    return VXR_OK;
}

int vxr_view_create(vxr_world* w, const vxr_view_desc* d, vxr_view** out) {
    VXR_CHECK_ARG(w && d && out, "vxr_view_create: null argument");
    VXR_CHECK_ARG(d->width >= 1 && d->height >= 1 && d->width <= 16384 && d->height <= 16384,
                  "vxr_view_create: resolution out of range [1, 16384]");
    VXR_CHECK_ARG(d->light_model == VXR_LIGHTS_AREA || d->light_model == VXR_LIGHTS_POINT,
                  "vxr_view_create: unknown light model");
    VXR_CHECK_ARG(d->spatial_radius >= 1, "vxr_view_create: spatial_radius must be >= 1");
    VXR_CHECK_ARG(d->tile_x <= 256 && d->tile_y <= 256 && d->tile_x * d->tile_y <= 256, "vxr_view_create: tile larger than 256 threads");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return set_error(VXR_E_NODEVICE, "no CUDA device visible");
    vxr_view* v = new (std::nothrow) vxr_view();
    if (!v) return set_error(VXR_E_NOMEM, "vxr_view_create: out of host memory");
    v->world = w;
    v->desc = *d;
    v->cam.rng = d->rng_seed;
    v->npx = (size_t)d->width * d->height;
    const size_t n = v->npx;
    vxr::ViewBuffers& b = v->buf;
    cudaError_t e = cudaSuccess;
    auto alloc = [&](void** p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, bytes);
        if (e == cudaSuccess) e = cudaMemset(*p, 0, bytes);
    };
    alloc((void**)&b.vd[0], n * sizeof(uint2));
    alloc((void**)&b.vd[1], n * sizeof(uint2));
    alloc((void**)&b.seed, n * sizeof(uint32_t));
    alloc((void**)&b.cA, n * sizeof(uint4));
    alloc((void**)&b.cB, n * sizeof(float4));
    alloc((void**)&b.hA, n * sizeof(uint4));
    alloc((void**)&b.hB, n * sizeof(float4));
    alloc((void**)&b.frame, n * sizeof(float4));
    alloc((void**)&b.accum, n * sizeof(float4));
    alloc((void**)&b.err, sizeof(uint32_t));
    alloc((void**)&b.hits, n * sizeof(uint32_t));
    alloc((void**)&b.qA, n * sizeof(float4));
    alloc((void**)&b.qB, n * sizeof(float4));
    alloc((void**)&b.counters, vxr::kCounters * sizeof(uint32_t));
    alloc((void**)&b.hitsAlt, n * sizeof(uint32_t));
    alloc((void**)&b.qAAlt, n * sizeof(float4));
    alloc((void**)&b.qBAlt, n * sizeof(float4));
    alloc((void**)&b.countersAlt, vxr::kCounters * sizeof(uint32_t));
    // the highest stream priority: a learned view's training steps (a side stream of the
    // lowest priority with training_lag = 1) fill only the SM slots its frames leave free
    int leastPrio = 0, greatestPrio = 0;
    if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&leastPrio, &greatestPrio);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&v->stream, cudaStreamNonBlocking, greatestPrio);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&v->stream2, cudaStreamNonBlocking, greatestPrio);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&v->evSpatial, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&v->evFront, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&v->evNow, cudaEventDisableTiming);
    v->ringS.assign(vxr_view::kRing * 6, nullptr);
    v->ringE.assign(vxr_view::kRing * 6, nullptr);
    v->ringUsed.assign(vxr_view::kRing * 6, 0);
    for (int i = 0; i < vxr_view::kRing * 6 && e == cudaSuccess; i++) {
        e = cudaEventCreate(&v->ringS[i]);
        if (e == cudaSuccess) e = cudaEventCreate(&v->ringE[i]);
    }
    for (int i = 0; i < 6 && e == cudaSuccess; i++) {
        e = cudaEventCreate(&v->evs[i]);
        if (e == cudaSuccess) e = cudaEventCreate(&v->eve[i]);
    }
    if (e != cudaSuccess) {
        free_view(v);
        delete v;
        return set_error(e == cudaErrorMemoryAllocation ? VXR_E_NOMEM : VXR_E_CUDA,
                         std::string("vxr_view_create: ") + cudaGetErrorString(e));
    }
    const int r = ensure_world(v);
    if (r != VXR_OK) {
        free_view(v);
        delete v;
        return r;
    }
    v->seenLightVersion = w->w.lightVersion;
    v->seenLightMoveVersion = w->w.lightMoveVersion;
    *out = v;
    return VXR_OK;
}

int vxr_view_destroy(vxr_view* v) {
    if (!v) return VXR_OK;
    if (v->stream2) cudaStreamSynchronize(v->stream2);
    cudaStreamSynchronize(v->stream);
    free_view(v);
    delete v;
    return VXR_OK;
}

int vxr_view_lookat(vxr_view* v, const float pos[3], const float target[3]) {
    if (int r = check_view(v, "vxr_view_lookat")) return r;
    VXR_CHECK_ARG(pos && target, "vxr_view_lookat: null argument");
    v->cam.M = vxr::look_at(pos, target);
    return VXR_OK;
}

int vxr_view_set_camera_matrix(vxr_view* v, const float m[16]) {
    if (int r = check_view(v, "vxr_view_set_camera_matrix")) return r;
    VXR_CHECK_ARG(m, "vxr_view_set_camera_matrix: null matrix");
    std::memcpy(v->cam.M.cell, m, sizeof(float) * 16);
    return VXR_OK;
}

int vxr_view_set_params(vxr_view* v, const vxr_view_desc* d) {
    if (int r = check_view(v, "vxr_view_set_params")) return r;
    v->spatialEvOk = false;
    VXR_CHECK_ARG(d, "vxr_view_set_params: null desc");
    VXR_CHECK_ARG(d->width == v->desc.width && d->height == v->desc.height && d->light_model == v->desc.light_model,
                  "vxr_view_set_params: resolution and light model are fixed at creation");
    VXR_CHECK_ARG(d->spatial_radius >= 1, "vxr_view_set_params: spatial_radius must be >= 1");
    VXR_CHECK_ARG(d->tile_x <= 256 && d->tile_y <= 256 && d->tile_x * d->tile_y <= 256, "vxr_view_set_params: tile larger than 256 threads");
    const uint32_t seed = v->desc.rng_seed;
    v->desc = *d;
    v->desc.rng_seed = seed;
    return VXR_OK;
}

int vxr_view_set_sky(vxr_view* v, const float* rgba, uint32_t w, uint32_t h, const float sky_light[24],
                     float light_scale, const uint32_t* blue_noise) {
    if (int r = check_view(v, "vxr_view_set_sky")) return r;
    v->spatialEvOk = false;
    if (!rgba) {
        CUV(cudaStreamSynchronize(v->stream), "vxr_view_set_sky: wait");
        cudaFree(v->skyDev); cudaFree(v->skyTex); cudaFree(v->skyBlueNoise);
        v->skyDev = nullptr;
        v->skyTex = nullptr;
        v->skyBlueNoise = nullptr;
        return VXR_OK;
    }
    VXR_CHECK_ARG(sky_light && blue_noise, "vxr_view_set_sky: null sky_light or blue_noise");
    VXR_CHECK_ARG(w >= 1 && h >= 1 && w <= 65536 && h <= 65536 && (uint64_t)w * h < (1ull << 31),
                  "vxr_view_set_sky: size out of [1, 65536] or more than 2^31 - 1 texels");
    const size_t texels = (size_t)w * h;
    // the frames in flight may read the old sky
    CUV(cudaStreamSynchronize(v->stream), "vxr_view_set_sky: wait");
    if (!v->skyDev) CUV(cudaMalloc(&v->skyDev, sizeof(vxr::dev::Sky)), "cudaMalloc(sky)");
    if (!v->skyBlueNoise) CUV(cudaMalloc(&v->skyBlueNoise, VXR_BLUE_NOISE_WORDS * sizeof(uint32_t)), "cudaMalloc(blue noise)");
    cudaFree(v->skyTex);
    v->skyTex = nullptr;
    CUV(cudaMalloc(&v->skyTex, texels * sizeof(float4)), "cudaMalloc(sky texture)");
    CUV(cudaMemcpy(v->skyTex, rgba, texels * sizeof(float4), cudaMemcpyHostToDevice), "copy sky texture");
    CUV(cudaMemcpy(v->skyBlueNoise, blue_noise, VXR_BLUE_NOISE_WORDS * sizeof(uint32_t), cudaMemcpyHostToDevice),
        "copy blue noise");
    vxr::dev::Sky s;
    s.tex = v->skyTex;
    s.blueNoise = v->skyBlueNoise;
    s.w = w;
    s.h = h;
    s.lightScale = light_scale;
    for (int i = 0; i < 6; i++)
        s.light[i] = make_float4(sky_light[4 * i], sky_light[4 * i + 1], sky_light[4 * i + 2], sky_light[4 * i + 3]);
    CUV(cudaMemcpy(v->skyDev, &s, sizeof(s), cudaMemcpyHostToDevice), "copy sky constants");
    return VXR_OK;
}

int vxr_view_begin_frame(vxr_view* v, vxr_frame_consts* out) {
    if (int r = check_view(v, "vxr_view_begin_frame")) return r;
    v->spatialEvOk = false;
    if (int r = ensure_world(v)) return r;
    vxr::World& w = v->world->w;
    if (w.lightVersion != v->seenLightVersion) {
        v->cam.restirtemporalframe = 0;   // any light change resets temporal reuse (world.cpp:245)
        v->seenLightVersion = w.lightVersion;
    }
    if (w.lightMoveVersion != v->seenLightMoveVersion) {
        // moved lights reset temporal reuse only without spatial reuse (world.cpp:300-301)
        if (!v->desc.spatial) v->cam.restirtemporalframe = 0;
        v->seenLightMoveVersion = w.lightMoveVersion;
    }
    vxr_frame_consts& k = v->k;
    std::memset(&k, 0, sizeof(k));
    vxr::begin_frame(v->cam, v->desc.width, v->desc.height, &k);
    k.accumulate = v->desc.accumulate;
    k.spatial = v->desc.spatial;
    k.temporal = v->desc.temporal;
    k.numberOfLights = w.dev->nl;
    k.numberOfCandidates = v->desc.num_candidates;
    k.numberOfMaxTemporalImportance = v->desc.temporal_max_importance;
    k.spatialRadius = v->desc.spatial_radius;
    k.spatialTaps = v->desc.spatial_taps;
    v->cur ^= 1;   // G-buffer swap (world.cpp:2221-2223)
    std::swap(v->buf.hits, v->buf.hitsAlt);   // this frame's work lists
    std::swap(v->buf.qA, v->buf.qAAlt);
    std::swap(v->buf.qB, v->buf.qBAlt);
    std::swap(v->buf.counters, v->buf.countersAlt);
    if (int r = vxr::brick_cache_begin(v)) return r;
    v->frameOpen = true;
    for (int i = 0; i < 6; i++) v->ran[i] = false;
    if (out) *out = k;
    return VXR_OK;
}

int vxr_view_set_frame_consts(vxr_view* v, const vxr_frame_consts* k) {
    if (int r = check_view(v, "vxr_view_set_frame_consts")) return r;
    VXR_CHECK_ARG(k, "vxr_view_set_frame_consts: null consts");
    VXR_CHECK_ARG(v->frameOpen, "vxr_view_set_frame_consts: no frame in progress");
    VXR_CHECK_ARG(k->width == v->desc.width && k->height == v->desc.height, "vxr_view_set_frame_consts: resolution mismatch");
    VXR_CHECK_ARG(k->numberOfLights == v->world->w.dev->nl, "vxr_view_set_frame_consts: light count differs from the uploaded list");
    VXR_CHECK_ARG(k->spatialRadius >= 1, "vxr_view_set_frame_consts: spatialRadius must be >= 1");
    v->k = *k;
    return VXR_OK;
}

// s: the stream of the stage's launches; tail (candidate stage): the stream of its
// temporal pass, handed on by an event (null: s)
static int run_stage(vxr_view* v, int stage, bool fuse, cudaStream_t s, cudaStream_t tail = nullptr) {
    if (!tail) tail = s;
    if (!v->frameOpen) return set_error(VXR_E_STATE, "vxr_view_stage: call vxr_view_begin_frame first");
    if (int r = ensure_world(v)) return r;
    const vxr::dev::World w = dev_world(v);
    vxr::dev::Frame k = dev_frame(v->k);
    k.sky = v->skyDev;
    const bool point = v->desc.light_model == VXR_LIGHTS_POINT;
    const vxr::Tuning sh = shape(v);
    if (stage == VXR_STAGE_PATH_TRACE) {   // ground-truth mode: no stage timing
        vxr::BatchDev bd = vxr::single_batch(w, k, v->buf, v->cur, point, sh);
        vxr::launch_path_trace(bd, s);
        CUV(cudaGetLastError(), "kernel launch");
        return VXR_OK;
    }
    const int ri = (int)(v->frameSerial % vxr_view::kRing) * 6 + stage;
    CUV(cudaEventRecord(v->evs[stage], s), "cudaEventRecord");
    CUV(cudaEventRecord(v->ringS[ri], s), "cudaEventRecord");
    vxr::BatchDev bd = vxr::single_batch(w, k, v->buf, v->cur, point, sh);
    bd.fuse = fuse ? 1 : 0;
    bd.timer = v->ktimerOn ? v->ktimer : nullptr;
    if (sh.brickCache > 0) {
        if (v->bc.calibrating) {
            bd.bcCount = v->bc.count;
        } else if (v->bc.log2 > 0) {
            bd.bcKeys = v->bc.keys;
            bd.bcMask = v->bc.mask;
            bd.bcLog2 = v->bc.log2;
        }
    }
    const int variant = point ? 1 : 0;
    switch (stage) {
    case VXR_STAGE_ALBEDO: vxr::launch_batch_albedo(bd, variant, s); break;
    case VXR_STAGE_CANDIDATES: {
        vxr::LearnedHook hook;
        const bool learned = vxr::learned_hook(v, &hook, s);
        vxr::launch_batch_candidates(bd, variant, learned ? &hook : nullptr, s, tail, v->evFront);
        break;
    }
    case VXR_STAGE_SPATIAL: vxr::launch_batch_spatial(bd, variant, s); break;
    case VXR_STAGE_SHADE: vxr::launch_batch_shade(bd, variant, s); break;
    case VXR_STAGE_ACCUMULATE: vxr::launch_batch_accumulate(bd, variant, s); break;
    default: return set_error(VXR_E_INVALID, "vxr_view_stage: unknown stage");
    }
    CUV(cudaGetLastError(), "kernel launch");
    CUV(cudaEventRecord(v->eve[stage], tail), "cudaEventRecord");
    CUV(cudaEventRecord(v->ringE[ri], tail), "cudaEventRecord");
    v->ringUsed[ri] = 1;
    v->ran[stage] = true;
    return VXR_OK;
}

int vxr_view_stage(vxr_view* v, int stage) {
    if (int r = check_view(v, "vxr_view_stage")) return r;
    return run_stage(v, stage, false, v->stream);
}

int vxr_view_end_frame(vxr_view* v) {
    if (int r = check_view(v, "vxr_view_end_frame")) return r;
    if (!v->frameOpen) return set_error(VXR_E_STATE, "vxr_view_end_frame: no frame in progress");
    vxr::end_frame(v->cam);
    v->frameOpen = false;
    v->frameSerial++;
    return vxr::brick_cache_end(v);
}

// One frame. Its front half (primary rays, hit list, proposal, candidates and their
// visibility) writes the G-buffer plane, the seeds and the candidate reservoirs that the
// previous frame's candidate and spatial passes were the last to touch, and this frame's
// own work lists; the previous frame's shading reads only the other plane, the spatial
// reservoirs and its own lists. So when the previous frame was rendered here with
// nothing in between, the front half runs on the second stream from the end of that
// frame's spatial pass, beside its shading; the temporal pass (which reads the history
// that shading patches) and everything after it run on the view's stream.
int vxr_view_render(vxr_view* v) {
    if (int r = check_view(v, "vxr_view_render")) return r;
    const bool overlap = v->spatialEvOk && shape(v).brickCache <= 0;
    if (int r = vxr_view_begin_frame(v, nullptr)) return r;
    if (!overlap) CUV(cudaEventRecord(v->evNow, v->stream), "cudaEventRecord");
    CUV(cudaStreamWaitEvent(v->stream2, overlap ? v->evSpatial : v->evNow, 0), "cudaStreamWaitEvent");
    if (int r = run_stage(v, VXR_STAGE_ALBEDO, false, v->stream2)) return r;
    if (int r = run_stage(v, VXR_STAGE_CANDIDATES, false, v->stream2, v->stream)) return r;
    if (int r = run_stage(v, VXR_STAGE_SPATIAL, false, v->stream)) return r;
    CUV(cudaEventRecord(v->evSpatial, v->stream), "cudaEventRecord");
    if (int r = run_stage(v, VXR_STAGE_SHADE, true, v->stream)) return r;
    if (int r = vxr::proposal_frame_train(v)) return r;
    if (int r = vxr_view_end_frame(v)) return r;
    v->spatialEvOk = true;
    return VXR_OK;
}

// waits for the view's stream; join: also for the online training step still running on
// its side stream (render_to_host returns once the image is on the host, the step
// overlapping the caller's next frame)
static int view_wait(vxr_view* v, bool join) {
    if (join) vxr::proposal_join(v);
    CUV(cudaStreamSynchronize(v->stream), "vxr_view_wait");
    for (int s = 1; s <= 5; s++) {
        float ms = 0.0f;
        if (v->ran[s]) cudaEventElapsedTime(&ms, v->evs[s], v->eve[s]);
        v->times[s - 1] = ms;
    }
    harvest(v);
    // kernel times once every marked kernel has run (the training step's marks are on its
    // side stream)
    if (v->ktimer && join) v->ktimer->harvest();
    uint32_t err = 0;
    CUV(cudaMemcpy(&err, v->buf.err, sizeof(err), cudaMemcpyDeviceToHost), "read device error flags");
    if (err) {
        cudaMemset(v->buf.err, 0, sizeof(uint32_t));
        return set_error(VXR_E_DEVICE, vxr::device_flags_message(err));
    }
    return VXR_OK;
}

int vxr_view_wait(vxr_view* v) {
    if (int r = check_view(v, "vxr_view_wait")) return r;
    return view_wait(v, true);
}

int vxr_view_stage_times(vxr_view* v, float ms[5]) {
    if (int r = check_view(v, "vxr_view_stage_times")) return r;
    VXR_CHECK_ARG(ms, "vxr_view_stage_times: null output");
    for (int i = 0; i < 5; i++) ms[i] = v->times[i];
    return VXR_OK;
}

int vxr_view_read_gbuffer(vxr_view* v, int which, vxr_gbuffer_rec* out) {
    if (int r = check_view(v, "vxr_view_read_gbuffer")) return r;
    VXR_CHECK_ARG(out && (which == 0 || which == 1), "vxr_view_read_gbuffer: bad argument");
    const size_t n = v->npx;
    std::vector<uint2> vd(n);
    std::vector<uint32_t> seed(n);
    CUV(cudaStreamSynchronize(v->stream), "sync");
    CUV(cudaMemcpy(vd.data(), v->buf.vd[which == 0 ? v->cur : v->cur ^ 1], n * sizeof(uint2), cudaMemcpyDeviceToHost), "read G-buffer");
    CUV(cudaMemcpy(seed.data(), v->buf.seed, n * sizeof(uint32_t), cudaMemcpyDeviceToHost), "read seeds");
    for (size_t i = 0; i < n; i++) {
        out[i].voxel = vd[i].x & 0x00FFFFFFu;
        out[i].side = vd[i].x >> 24;
        std::memcpy(&out[i].dist, &vd[i].y, 4);
        out[i].seed = seed[i];
    }
    return VXR_OK;
}

int vxr_view_write_gbuffer(vxr_view* v, int which, const vxr_gbuffer_rec* in) {
    if (int r = check_view(v, "vxr_view_write_gbuffer")) return r;
    v->spatialEvOk = false;
    VXR_CHECK_ARG(in && (which == 0 || which == 1), "vxr_view_write_gbuffer: bad argument");
    const size_t n = v->npx;
    std::vector<uint2> vd(n);
    std::vector<uint32_t> seed(n);
    for (size_t i = 0; i < n; i++) {
        VXR_CHECK_ARG(in[i].side <= 2 && in[i].voxel <= 0x00FFFFFFu, "vxr_view_write_gbuffer: side > 2 or voxel above 24 bits");
        uint32_t d;
        std::memcpy(&d, &in[i].dist, 4);
        vd[i] = make_uint2(in[i].voxel | (in[i].side << 24), d);
        seed[i] = in[i].seed;
    }
    CUV(cudaStreamSynchronize(v->stream), "sync");
    CUV(cudaMemcpy(v->buf.vd[which == 0 ? v->cur : v->cur ^ 1], vd.data(), n * sizeof(uint2), cudaMemcpyHostToDevice), "write G-buffer");
    if (which == 0) CUV(cudaMemcpy(v->buf.seed, seed.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice), "write seeds");
    return VXR_OK;
}

static const float kNormals[6][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {-1, 0, 0}, {0, -1, 0}, {0, 0, -1}};

int vxr_view_read_reservoirs(vxr_view* v, int role, vxr_reservoir_rec* out) {
    if (int r = check_view(v, "vxr_view_read_reservoirs")) return r;
    VXR_CHECK_ARG(out && (role == 0 || role == 1), "vxr_view_read_reservoirs: bad argument");
    const size_t n = v->npx;
    std::vector<uint4> a(n);
    std::vector<float4> b(n);
    CUV(cudaStreamSynchronize(v->stream), "sync");
    CUV(cudaMemcpy(a.data(), role == 0 ? v->buf.cA : v->buf.hA, n * sizeof(uint4), cudaMemcpyDeviceToHost), "read reservoirs");
    CUV(cudaMemcpy(b.data(), role == 0 ? v->buf.cB : v->buf.hB, n * sizeof(float4), cudaMemcpyDeviceToHost), "read reservoirs");
    for (size_t i = 0; i < n; i++) {
        vxr_reservoir_rec& r = out[i];
        std::memcpy(&r.sumOfWeights, &a[i].z, 4);
        std::memcpy(&r.pHat, &a[i].w, 4);
        r.streamLength = a[i].y & 0x1FFFFFFFu;
        r.lightIndex = a[i].x;
        const float den = std::max(1e-5f, r.pHat * (float)r.streamLength);
        r.adjustedWeight = r.sumOfWeights / den;
        r.positionOnVoxel[0] = b[i].x;
        r.positionOnVoxel[1] = b[i].y;
        r.positionOnVoxel[2] = b[i].z;
        r.invPositionProbability = b[i].w;
        const uint32_t c = a[i].y >> 29;
        for (int j = 0; j < 3; j++) r.Nlight[j] = c < 6 ? kNormals[c][j] : 0.0f;
    }
    return VXR_OK;
}

int vxr_view_write_reservoirs(vxr_view* v, int role, const vxr_reservoir_rec* in) {
    if (int r = check_view(v, "vxr_view_write_reservoirs")) return r;
    v->spatialEvOk = false;
    VXR_CHECK_ARG(in && (role == 0 || role == 1), "vxr_view_write_reservoirs: bad argument");
    const size_t n = v->npx;
    std::vector<uint4> a(n);
    std::vector<float4> b(n);
    for (size_t i = 0; i < n; i++) {
        const vxr_reservoir_rec& r = in[i];
        uint32_t c = 6;
        for (uint32_t j = 0; j < 6; j++)
            if (r.Nlight[0] == kNormals[j][0] && r.Nlight[1] == kNormals[j][1] && r.Nlight[2] == kNormals[j][2]) c = j;
        VXR_CHECK_ARG(c < 6 || (r.Nlight[0] == 0.0f && r.Nlight[1] == 0.0f && r.Nlight[2] == 0.0f),
                      "vxr_view_write_reservoirs: Nlight must be a face normal or zero");
        VXR_CHECK_ARG(r.streamLength < (1u << 29), "vxr_view_write_reservoirs: streamLength >= 2^29");
        uint32_t sw, ph;
        std::memcpy(&sw, &r.sumOfWeights, 4);
        std::memcpy(&ph, &r.pHat, 4);
        a[i] = make_uint4(r.lightIndex, r.streamLength | (c << 29), sw, ph);
        b[i] = make_float4(r.positionOnVoxel[0], r.positionOnVoxel[1], r.positionOnVoxel[2], r.invPositionProbability);
    }
    CUV(cudaStreamSynchronize(v->stream), "sync");
    CUV(cudaMemcpy(role == 0 ? v->buf.cA : v->buf.hA, a.data(), n * sizeof(uint4), cudaMemcpyHostToDevice), "write reservoirs");
    CUV(cudaMemcpy(role == 0 ? v->buf.cB : v->buf.hB, b.data(), n * sizeof(float4), cudaMemcpyHostToDevice), "write reservoirs");
    return VXR_OK;
}

int vxr_view_read_frame(vxr_view* v, float* rgba) {
    if (int r = check_view(v, "vxr_view_read_frame")) return r;
    VXR_CHECK_ARG(rgba, "vxr_view_read_frame: null output");
    CUV(cudaStreamSynchronize(v->stream), "sync");
    CUV(cudaMemcpy(rgba, v->buf.frame, v->npx * sizeof(float4), cudaMemcpyDeviceToHost), "read frame");
    return VXR_OK;
}

int vxr_view_read_accum(vxr_view* v, float* rgba) {
    if (int r = check_view(v, "vxr_view_read_accum")) return r;
    VXR_CHECK_ARG(rgba, "vxr_view_read_accum: null output");
    CUV(cudaStreamSynchronize(v->stream), "sync");
    CUV(cudaMemcpy(rgba, v->buf.accum, v->npx * sizeof(float4), cudaMemcpyDeviceToHost), "read accumulator");
    return VXR_OK;
}

int vxr_view_render_to_host(vxr_view* v, const float pos[3], const float target[3], float* host_rgba) {
    if (int r = check_view(v, "vxr_view_render_to_host")) return r;
    VXR_CHECK_ARG(pos && target && host_rgba, "vxr_view_render_to_host: null argument");
    if (int r = vxr_view_lookat(v, pos, target)) return r;
    if (int r = vxr_view_render(v)) return r;
    CUV(cudaMemcpyAsync(host_rgba, v->buf.accum, v->npx * sizeof(float4), cudaMemcpyDeviceToHost, v->stream), "copy image");
    return view_wait(v, false);
}

int vxr_view_render_to_host_async(vxr_view* v, const float pos[3], const float target[3], float* host_rgba,
                                  uint64_t* ticket) {
    if (int r = check_view(v, "vxr_view_render_to_host_async")) return r;
    VXR_CHECK_ARG(pos && target && host_rgba && ticket, "vxr_view_render_to_host_async: null argument");
    const int slot = (int)(v->imgSerial % vxr_view::kImages);
    if (v->imgSerial >= (uint64_t)vxr_view::kImages)   // the slot's previous image must be done
        CUV(cudaEventSynchronize(v->imgEv[slot]), "vxr_view_render_to_host_async: wait for an earlier image");
    if (!v->imgEv[slot]) CUV(cudaEventCreateWithFlags(&v->imgEv[slot], cudaEventDisableTiming), "cudaEventCreate");
    if (int r = vxr_view_lookat(v, pos, target)) return r;
    if (int r = vxr_view_render(v)) return r;
    CUV(cudaMemcpyAsync(host_rgba, v->buf.accum, v->npx * sizeof(float4), cudaMemcpyDeviceToHost, v->stream), "copy image");
    CUV(cudaEventRecord(v->imgEv[slot], v->stream), "cudaEventRecord");
    *ticket = v->imgSerial++;
    return VXR_OK;
}

int vxr_view_image_wait(vxr_view* v, uint64_t ticket) {
    if (int r = check_view(v, "vxr_view_image_wait")) return r;
    VXR_CHECK_ARG(ticket < v->imgSerial && v->imgSerial - ticket <= (uint64_t)vxr_view::kImages,
                  "vxr_view_image_wait: unknown or expired ticket");
    CUV(cudaEventSynchronize(v->imgEv[ticket % vxr_view::kImages]), "vxr_view_image_wait");
    uint32_t err = 0;
    CUV(cudaMemcpy(&err, v->buf.err, sizeof(err), cudaMemcpyDeviceToHost), "read device error flags");
    if (err) {
        cudaMemset(v->buf.err, 0, sizeof(uint32_t));
        return set_error(VXR_E_DEVICE, vxr::device_flags_message(err));
    }
    return VXR_OK;
}

}  // extern "C"

// ---- host-only camera, timers, pinned memory ---------------------------------------------
struct vxr_camera {
    vxr::CameraState st;
};

extern "C" {

int vxr_camera_create(uint32_t rng_seed, vxr_camera** out) {
    VXR_CHECK_ARG(out, "vxr_camera_create: null out");
    vxr_camera* c = new (std::nothrow) vxr_camera();
    if (!c) return set_error(VXR_E_NOMEM, "vxr_camera_create: out of host memory");
    c->st.rng = rng_seed;
    *out = c;
    return VXR_OK;
}

int vxr_camera_destroy(vxr_camera* c) {
    delete c;
    return VXR_OK;
}

int vxr_camera_lookat(vxr_camera* c, const float pos[3], const float target[3]) {
    VXR_CHECK_ARG(c && pos && target, "vxr_camera_lookat: null argument");
    c->st.M = vxr::look_at(pos, target);
    return VXR_OK;
}

int vxr_camera_set_matrix(vxr_camera* c, const float m[16]) {
    VXR_CHECK_ARG(c && m, "vxr_camera_set_matrix: null argument");
    std::memcpy(c->st.M.cell, m, sizeof(float) * 16);
    return VXR_OK;
}

int vxr_camera_begin_frame(vxr_camera* c, uint32_t W, uint32_t H, vxr_frame_consts* k) {
    VXR_CHECK_ARG(c && k && W > 0 && H > 0, "vxr_camera_begin_frame: bad argument");
    vxr::begin_frame(c->st, W, H, k);
    return VXR_OK;
}

int vxr_camera_end_frame(vxr_camera* c) {
    VXR_CHECK_ARG(c, "vxr_camera_end_frame: null camera");
    vxr::end_frame(c->st);
    return VXR_OK;
}

int vxr_host_alloc(size_t bytes, void** p) {
    VXR_CHECK_ARG(p && bytes > 0, "vxr_host_alloc: bad argument");
    CUV(cudaHostAlloc(p, bytes, cudaHostAllocDefault), "cudaHostAlloc");
    return VXR_OK;
}

int vxr_host_free(void* p) {
    if (p) CUV(cudaFreeHost(p), "cudaFreeHost");
    return VXR_OK;
}

int vxr_view_timer_begin(vxr_view* v) {
    if (int r = check_view(v, "vxr_view_timer_begin")) return r;
    v->spatialEvOk = false;   // the next frame's primary rays start after this mark
    CUV(cudaEventRecord(v->evs[0], v->stream), "cudaEventRecord");
    return VXR_OK;
}

int vxr_view_timer_end(vxr_view* v, float* ms) {
    if (int r = check_view(v, "vxr_view_timer_end")) return r;
    VXR_CHECK_ARG(ms, "vxr_view_timer_end: null output");
    vxr::proposal_join(v);   // the timed region ends after the last frame's training step
    CUV(cudaEventRecord(v->eve[0], v->stream), "cudaEventRecord");
    CUV(cudaEventSynchronize(v->eve[0]), "cudaEventSynchronize");
    CUV(cudaEventElapsedTime(ms, v->evs[0], v->eve[0]), "cudaEventElapsedTime");
    return VXR_OK;
}

}  // extern "C"

namespace vxr {
int check_tuning(const vxr_tuning* t, const char* fn) {
    if (!t) return set_error(VXR_E_INVALID, std::string(fn) + ": null tuning");
    const uint32_t n = t->tile_x * t->tile_y;
    if (t->tile_x < 1 || t->tile_y < 1 || t->tile_x > 256 || t->tile_y > 256 || n > 256 || n % 32 != 0)
        return set_error(VXR_E_INVALID, std::string(fn) + ": tile must hold a multiple of 32 threads, at most 256");
    if (t->persistent > 1) return set_error(VXR_E_INVALID, std::string(fn) + ": persistent must be 0 or 1");
    if (t->shadow_refill < 1 || t->shadow_refill > 32)
        return set_error(VXR_E_INVALID, std::string(fn) + ": shadow_refill out of range [1, 32]");
    if (t->shadow_burst < 1 || t->shadow_burst > 64)
        return set_error(VXR_E_INVALID, std::string(fn) + ": shadow_burst out of range [1, 64]");
    if (t->list_blocks_per_sm < 1 || t->list_blocks_per_sm > 64)
        return set_error(VXR_E_INVALID, std::string(fn) + ": list_blocks_per_sm out of range [1, 64]");
    if (t->occupancy > 1) return set_error(VXR_E_INVALID, std::string(fn) + ": occupancy must be 0 or 1");
    if (t->shadow_schedule > 1) return set_error(VXR_E_INVALID, std::string(fn) + ": shadow_schedule must be 0 or 1");
    if (t->shadow_early_out > 1) return set_error(VXR_E_INVALID, std::string(fn) + ": shadow_early_out must be 0 or 1");
    if (t->brick_cache != 0 && (t->brick_cache < 128 || t->brick_cache > 2048 || (t->brick_cache & (t->brick_cache - 1))))
        return set_error(VXR_E_INVALID, std::string(fn) + ": brick_cache must be 0 or a power of two in [128, 2048]");
    return VXR_OK;
}
Tuning to_tuning(const vxr_tuning& t) {
    Tuning u;
    u.bx = (int)t.tile_x;
    u.by = (int)t.tile_y;
    u.persistent = (int)t.persistent;
    u.refill = (int)t.shadow_refill;
    u.burst = (int)t.shadow_burst;
    u.listPerSm = (int)t.list_blocks_per_sm;
    u.occupancy = (int)t.occupancy;
    u.schedule = (int)t.shadow_schedule;
    u.earlyOut = (int)t.shadow_early_out;
    u.brickCache = (int)t.brick_cache;
    return u;
}
}  // namespace vxr

extern "C" int vxr_default_tuning(vxr_tuning* t) {
    VXR_CHECK_ARG(t, "vxr_default_tuning: null tuning");
    const vxr::Tuning u;
    t->tile_x = (uint32_t)u.bx;
    t->tile_y = (uint32_t)u.by;
    t->persistent = (uint32_t)u.persistent;
    t->shadow_refill = (uint32_t)u.refill;
    t->shadow_burst = (uint32_t)u.burst;
    t->list_blocks_per_sm = (uint32_t)u.listPerSm;
    t->occupancy = (uint32_t)u.occupancy;
    t->shadow_schedule = (uint32_t)u.schedule;
    t->shadow_early_out = (uint32_t)u.earlyOut;
    t->brick_cache = (uint32_t)u.brickCache;
    return VXR_OK;
}

extern "C" int vxr_device_info(char* name, size_t n, int* sms, int* cc_major, int* cc_minor) {
    VXR_CHECK_ARG(name && n > 0 && sms && cc_major && cc_minor, "vxr_device_info: null argument");
    int dev = 0;
    cudaDeviceProp p;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&p, dev) != cudaSuccess)
        return set_error(VXR_E_NODEVICE, "vxr_device_info: no CUDA device visible");
    std::strncpy(name, p.name, n - 1);
    name[n - 1] = '\0';
    *sms = p.multiProcessorCount;
    *cc_major = p.major;
    *cc_minor = p.minor;
    return VXR_OK;
}

extern "C" int vxr_view_set_tuning(vxr_view* v, const vxr_tuning* t) {
    if (int r = check_view(v, "vxr_view_set_tuning")) return r;
    if (int r = vxr::check_tuning(t, "vxr_view_set_tuning")) return r;
    v->tuning = vxr::to_tuning(*t);
    v->desc.tile_x = t->tile_x;
    v->desc.tile_y = t->tile_y;
    return VXR_OK;
}

extern "C" int vxr_view_get_tuning(vxr_view* v, vxr_tuning* t) {
    if (int r = check_view(v, "vxr_view_get_tuning")) return r;
    VXR_CHECK_ARG(t, "vxr_view_get_tuning: null tuning");
    const vxr::Tuning u = shape(v);
    t->tile_x = (uint32_t)u.bx;
    t->tile_y = (uint32_t)u.by;
    t->persistent = (uint32_t)u.persistent;
    t->shadow_refill = (uint32_t)u.refill;
    t->shadow_burst = (uint32_t)u.burst;
    t->list_blocks_per_sm = (uint32_t)u.listPerSm;
    t->occupancy = (uint32_t)u.occupancy;
    t->shadow_schedule = (uint32_t)u.schedule;
    t->shadow_early_out = (uint32_t)u.earlyOut;
    t->brick_cache = (uint32_t)u.brickCache;
    return VXR_OK;
}

extern "C" int vxr_view_kernel_timing(vxr_view* v, int on) {
    if (int r = check_view(v, "vxr_view_kernel_timing")) return r;
    if (on && !v->ktimer) {
        vxr::ViewKernelTimer* t = new (std::nothrow) vxr::ViewKernelTimer();
        if (!t) return set_error(VXR_E_NOMEM, "vxr_view_kernel_timing: out of host memory");
        t->ev.assign(2 * vxr::ViewKernelTimer::kPairs, nullptr);
        t->id.assign(vxr::ViewKernelTimer::kPairs, 0);
        for (cudaEvent_t& e : t->ev) {
            const cudaError_t ce = cudaEventCreate(&e);
            if (ce != cudaSuccess) {
                delete t;
                return set_error(VXR_E_CUDA, std::string("vxr_view_kernel_timing: ") + cudaGetErrorString(ce));
            }
        }
        v->ktimer = t;
    }
    v->ktimerOn = on != 0;
    return VXR_OK;
}

extern "C" int vxr_view_kernel_stats(vxr_view* v, double sum_ms[VXR_KERNEL_COUNT], uint32_t count[VXR_KERNEL_COUNT],
                                     int reset) {
    if (int r = check_view(v, "vxr_view_kernel_stats")) return r;
    VXR_CHECK_ARG(sum_ms && count, "vxr_view_kernel_stats: null argument");
    CUV(cudaStreamSynchronize(v->stream), "vxr_view_kernel_stats");
    for (int i = 0; i < VXR_KERNEL_COUNT; i++) {
        sum_ms[i] = 0.0;
        count[i] = 0;
    }
    if (!v->ktimer) return VXR_OK;
    v->ktimer->harvest();
    for (int i = 0; i < VXR_KERNEL_COUNT; i++) {
        sum_ms[i] = v->ktimer->sum[i];
        count[i] = v->ktimer->count[i];
        if (reset) {
            v->ktimer->sum[i] = 0.0;
            v->ktimer->count[i] = 0;
        }
    }
    return VXR_OK;
}

extern "C" int vxr_view_work_counts(vxr_view* v, uint32_t counts[3]) {
    if (int r = check_view(v, "vxr_view_work_counts")) return r;
    VXR_CHECK_ARG(counts, "vxr_view_work_counts: null argument");
    uint32_t c[vxr::kCounters];
    CUV(cudaMemcpyAsync(c, v->buf.counters, sizeof(c), cudaMemcpyDeviceToHost, v->stream), "read counters");
    CUV(cudaStreamSynchronize(v->stream), "vxr_view_work_counts");
    counts[0] = c[vxr::kCtrHits];
    counts[1] = c[vxr::kCtrQ1];
    counts[2] = c[vxr::kCtrQ2];
    return VXR_OK;
}

extern "C" const char* vxr_kernel_name(int id) {
    static const char* names[VXR_KERNEL_COUNT] = {"albedo", "compact_hits", "proposal_infer", "ris_candidates",
                                                  "shadow_candidates", "temporal", "spatial", "shade_request",
                                                  "shadow_shading", "shade_finish", "accumulate", "proposal_train"};
    return id >= 0 && id < VXR_KERNEL_COUNT ? names[id] : "";
}

extern "C" int vxr_view_stage_stats(vxr_view* v, double sum_ms[5], uint32_t count[5], int reset) {
    if (int r = check_view(v, "vxr_view_stage_stats")) return r;
    VXR_CHECK_ARG(sum_ms && count, "vxr_view_stage_stats: null output");
    CUV(cudaStreamSynchronize(v->stream), "vxr_view_stage_stats");
    harvest(v);
    for (int s = 1; s <= 5; s++) {
        sum_ms[s - 1] = v->statSum[s];
        count[s - 1] = v->statCount[s];
        if (reset) {
            v->statSum[s] = 0.0;
            v->statCount[s] = 0;
        }
    }
    return VXR_OK;
}

// ---- converged reference and error metric ----------------------------------------------
extern "C" {

int vxr_view_sum64_reset(vxr_view* v) {
    if (int r = check_view(v, "vxr_view_sum64_reset")) return r;
    if (!v->sum64) CUV(cudaMalloc(&v->sum64, v->npx * 3 * sizeof(double)), "cudaMalloc(sum64)");
    CUV(cudaMemsetAsync(v->sum64, 0, v->npx * 3 * sizeof(double), v->stream), "clear sum64");
    v->sum64Count = 0;
    return VXR_OK;
}

int vxr_view_sum64_add(vxr_view* v) {
    if (int r = check_view(v, "vxr_view_sum64_add")) return r;
    if (!v->sum64) return set_error(VXR_E_STATE, "vxr_view_sum64_add: call vxr_view_sum64_reset first");
    vxr::launch_sum64_add(v->buf.frame, v->sum64, (uint32_t)v->npx, v->stream);
    CUV(cudaGetLastError(), "sum64 kernel");
    v->sum64Count++;
    return VXR_OK;
}

int vxr_view_sum64_mean(vxr_view* v, uint32_t* count, double* mean) {
    if (int r = check_view(v, "vxr_view_sum64_mean")) return r;
    VXR_CHECK_ARG(count, "vxr_view_sum64_mean: null count");
    *count = v->sum64Count;
    if (mean) {
        if (!v->sum64 || !v->sum64Count) return set_error(VXR_E_STATE, "vxr_view_sum64_mean: no frames summed");
        CUV(cudaStreamSynchronize(v->stream), "sync");
        CUV(cudaMemcpy(mean, v->sum64, v->npx * 3 * sizeof(double), cudaMemcpyDeviceToHost), "read sum64");
        const double inv = 1.0 / (double)v->sum64Count;
        for (size_t i = 0; i < v->npx * 3; i++) mean[i] *= inv;
    }
    return VXR_OK;
}

int vxr_view_error(vxr_view* img, int which, vxr_view* ref, double* mse, double* mae) {
    if (int r = check_view(img, "vxr_view_error")) return r;
    if (int r = check_view(ref, "vxr_view_error")) return r;
    VXR_CHECK_ARG(mse && mae && (which == 0 || which == 1), "vxr_view_error: bad argument");
    VXR_CHECK_ARG(img->npx == ref->npx && img->desc.width == ref->desc.width, "vxr_view_error: resolution mismatch");
    if (!ref->sum64 || !ref->sum64Count) return set_error(VXR_E_STATE, "vxr_view_error: reference has no summed frames");
    if (!img->errOut) CUV(cudaMalloc(&img->errOut, 2 * sizeof(double)), "cudaMalloc(error)");
    CUV(cudaStreamSynchronize(ref->stream), "sync reference");
    CUV(cudaMemsetAsync(img->errOut, 0, 2 * sizeof(double), img->stream), "clear error");
    vxr::launch_error(which == 0 ? img->buf.frame : img->buf.accum, ref->sum64, 1.0 / (double)ref->sum64Count,
                      (uint32_t)img->npx, img->errOut, img->stream);
    CUV(cudaGetLastError(), "error kernel");
    double h[2];
    CUV(cudaMemcpyAsync(h, img->errOut, sizeof(h), cudaMemcpyDeviceToHost, img->stream), "read error");
    CUV(cudaStreamSynchronize(img->stream), "sync");
    *mse = h[0] / ((double)img->npx * 3.0);
    *mae = h[1] / ((double)img->npx * 3.0);
    return VXR_OK;
}

}  // extern "C"
