// batch.cu - several views rendered as one frame (no reference counterpart: World::Render
// draws one camera per call, template/world.cpp:2127-2340).
//
// A batch owns the work lists of all its views (hit list, shadow-ray queue, counters:
// sized for the sum of their pixels) and a device table of ViewDev records that every
// stage kernel reads. Each frame the host fills the table in page-locked memory, copies
// it to the device on the batch stream and launches the four stages once for all views
// (kernels.cu, VARIANT 2). With VXR_BATCH_GRAPH the table copy and the stage launches are
// recorded once per staging slot as a CUDA graph and a frame is one cudaGraphLaunch.
//
// Staging: two page-locked table slots used alternately; before the host rewrites a
// slot it waits for the frame that last read it (an event recorded after that frame).
// Graph validity: the captured launches depend only on the view count, the views'
// resolutions and the tile shape, all fixed at creation; everything that changes per
// frame (frame constants, camera, world buffers after a re-upload, G-buffer plane) is in
// the table.
//
// Chains (VXR_BATCH_CHAINS(c)): the views are split into c groups of about equal pixel
// count, each with its own work lists and its slice of the table, and each group's four
// stages run on a branch stream of its own, forked from and joined back to the batch
// stream (in the graph: c parallel branches). One launch per stage then covers a group,
// and different groups can be in different stages at once, as views on their own streams
// are, while the frame stays one graph launch.
#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "internal.hpp"
#include "kernels.hpp"
#include "view.hpp"

// one group of views: its launch parameters, table slice and work lists
struct BatchChain {
    vxr::BatchDev bd;                       // table slice, totals, list buffers
    uint32_t first = 0, count = 0;          // slice of the table
    cudaStream_t stream = nullptr;          // branch stream (chains > 1)
    cudaEvent_t join = nullptr;
};

struct vxr_batch {
    std::vector<vxr_view*> views;
    std::vector<uint32_t> order;            // table slot -> index into views
    std::vector<BatchChain> chains;
    cudaEvent_t fork = nullptr;
    int sky = 0;                            // some view has a sky dome (graphs record its shading variant)
    int tx = 16, ty = 8;                    // tile shape
    vxr::ViewDev* table = nullptr;          // device table [n]
    vxr::ViewDev* staging[2] = {nullptr, nullptr};   // page-locked host slots
    cudaEvent_t slotDone[2] = {nullptr, nullptr};
    bool slotUsed[2] = {false, false};
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    bool useGraph = false;
    int device = -1;
    cudaStream_t stream = nullptr;
    std::vector<cudaEvent_t> viewReady;     // per view: its stream's work before the frame
    cudaEvent_t frameDone = nullptr;
    cudaEvent_t t0 = nullptr, t1 = nullptr; // GPU time of the last frame
    bool timed = false;
    uint64_t frames = 0;
};

namespace {

void free_batch(vxr_batch* b) {
    for (int i = 0; i < 2; i++) {
        if (b->graph[i]) cudaGraphExecDestroy(b->graph[i]);
        if (b->staging[i]) cudaFreeHost(b->staging[i]);
        if (b->slotDone[i]) cudaEventDestroy(b->slotDone[i]);
    }
    cudaFree(b->table);
    for (BatchChain& c : b->chains) {
        cudaFree(c.bd.hits);
        cudaFree(c.bd.qA);
        cudaFree(c.bd.qB);
        cudaFree(c.bd.counters);
        if (c.stream) cudaStreamDestroy(c.stream);
        if (c.join) cudaEventDestroy(c.join);
    }
    if (b->fork) cudaEventDestroy(b->fork);
    for (cudaEvent_t e : b->viewReady)
        if (e) cudaEventDestroy(e);
    if (b->frameDone) cudaEventDestroy(b->frameDone);
    if (b->t0) cudaEventDestroy(b->t0);
    if (b->t1) cudaEventDestroy(b->t1);
    if (b->stream) cudaStreamDestroy(b->stream);
}

void enqueue_stages(const vxr::BatchDev& bd, cudaStream_t s) {
    vxr::launch_batch_albedo(bd, 2, s);
    vxr::launch_batch_candidates(bd, 2, nullptr, s);
    vxr::launch_batch_spatial(bd, 2, s);
    vxr::launch_batch_shade(bd, 2, s);
}

// The frame's device work on the batch stream: table upload from slot `slot`, stages 1-4
// of every chain (on the chains' branch streams when there are several).
void enqueue_frame(vxr_batch* b, int slot) {
    const size_t n = b->views.size();
    cudaMemcpyAsync(b->table, b->staging[slot], n * sizeof(vxr::ViewDev), cudaMemcpyHostToDevice, b->stream);
    if (b->chains.size() == 1) {
        enqueue_stages(b->chains[0].bd, b->stream);
        return;
    }
    cudaEventRecord(b->fork, b->stream);
    for (BatchChain& c : b->chains) {
        cudaStreamWaitEvent(c.stream, b->fork, 0);
        enqueue_stages(c.bd, c.stream);
        cudaEventRecord(c.join, c.stream);
        cudaStreamWaitEvent(b->stream, c.join, 0);
    }
}

int cuda_error(cudaError_t e, const char* what) {
    return vxr::set_error(e == cudaErrorMemoryAllocation ? VXR_E_NOMEM : VXR_E_CUDA,
                          std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace

extern "C" {

int vxr_batch_create(vxr_view* const* views, uint32_t n, uint32_t tile_x, uint32_t tile_y, uint32_t flags, vxr_batch** out) {
    VXR_CHECK_ARG(views && out, "vxr_batch_create: null argument");
    VXR_CHECK_ARG(n >= 1 && n <= VXR_BATCH_MAX_VIEWS, "vxr_batch_create: view count out of range [1, VXR_BATCH_MAX_VIEWS]");
    VXR_CHECK_ARG((flags & ~(VXR_BATCH_GRAPH | VXR_BATCH_CHAINS(15u))) == 0, "vxr_batch_create: unknown flags");
    const uint32_t nchains = std::max<uint32_t>((flags >> 8) & 15u, 1u);
    VXR_CHECK_ARG(nchains <= n, "vxr_batch_create: more chains than views");
    const uint32_t tx = tile_x ? tile_x : 16, ty = tile_y ? tile_y : 8;
    VXR_CHECK_ARG(tx <= 256 && ty <= 256 && tx * ty >= 32 && tx * ty <= 256 && (tx * ty) % 32 == 0,
                  "vxr_batch_create: tile must hold a multiple of 32 threads, at most 256");
    uint64_t total = 0, tiles = 0;
    for (uint32_t i = 0; i < n; i++) {
        VXR_CHECK_ARG(views[i], "vxr_batch_create: null view");
        for (uint32_t j = 0; j < i; j++) VXR_CHECK_ARG(views[j] != views[i], "vxr_batch_create: a view appears twice");
        VXR_CHECK_ARG(views[i]->npx < (1ull << 27), "vxr_batch_create: a batched view holds at most 2^27 - 1 pixels");
        VXR_CHECK_ARG(!views[i]->world->w.dev || views[i]->world->w.dev->device == views[0]->world->w.dev->device,
                      "vxr_batch_create: views on different devices");
        total += views[i]->npx;
        tiles += (uint64_t)((views[i]->desc.width + tx - 1) / tx) * ((views[i]->desc.height + ty - 1) / ty);
    }
    VXR_CHECK_ARG(total < (1ull << 32) && tiles < (1ull << 32), "vxr_batch_create: batch too large");
    vxr_batch* b = new (std::nothrow) vxr_batch();
    if (!b) return vxr::set_error(VXR_E_NOMEM, "vxr_batch_create: out of host memory");
    b->views.assign(views, views + n);
    b->useGraph = (flags & VXR_BATCH_GRAPH) != 0;
    b->tx = (int)tx;
    b->ty = (int)ty;
    cudaGetDevice(&b->device);
    // chains of about equal pixel count: the largest views first, each to the lightest chain
    std::vector<uint32_t> byPixels(n);
    for (uint32_t i = 0; i < n; i++) byPixels[i] = i;
    std::stable_sort(byPixels.begin(), byPixels.end(),
                     [&](uint32_t a, uint32_t c) { return views[a]->npx > views[c]->npx; });
    std::vector<std::vector<uint32_t>> members(nchains);
    std::vector<uint64_t> load(nchains, 0);
    for (uint32_t i : byPixels) {
        const size_t c = (size_t)(std::min_element(load.begin(), load.end()) - load.begin());
        members[c].push_back(i);
        load[c] += views[i]->npx;
    }
    b->chains.resize(nchains);
    vxr::Tuning tu;
    tu.bx = (int)tx;
    tu.by = (int)ty;
    cudaError_t e = cudaSuccess;
    auto dalloc = [&](void** p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, bytes);
        if (e == cudaSuccess) e = cudaMemset(*p, 0, bytes);
    };
    dalloc((void**)&b->table, n * sizeof(vxr::ViewDev));
    for (uint32_t c = 0; c < nchains; c++) {
        std::sort(members[c].begin(), members[c].end());
        BatchChain& ch = b->chains[c];
        ch.first = (uint32_t)b->order.size();
        ch.count = (uint32_t)members[c].size();
        uint64_t px = 0, tl = 0;
        for (uint32_t i : members[c]) {
            b->order.push_back(i);
            px += views[i]->npx;
            tl += (uint64_t)((views[i]->desc.width + tx - 1) / tx) * ((views[i]->desc.height + ty - 1) / ty);
        }
        vxr::BatchDev& bd = ch.bd;
        bd.nviews = ch.count;
        bd.totalPixels = (uint32_t)px;
        bd.totalTiles = (uint32_t)tl;
        vxr::apply_tuning(bd, tu);
        bd.fuse = 1;
        dalloc((void**)&bd.hits, px * sizeof(uint32_t));
        dalloc((void**)&bd.qA, px * sizeof(float4));
        dalloc((void**)&bd.qB, px * sizeof(float4));
        dalloc((void**)&bd.counters, vxr::kCounters * sizeof(uint32_t));
        bd.views = b->table + ch.first;
        if (nchains > 1) {
            if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ch.stream, cudaStreamNonBlocking);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ch.join, cudaEventDisableTiming);
        }
    }
    if (nchains > 1 && e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    for (int i = 0; i < 2 && e == cudaSuccess; i++) {
        e = cudaHostAlloc((void**)&b->staging[i], n * sizeof(vxr::ViewDev), cudaHostAllocDefault);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->slotDone[i], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    b->viewReady.assign(n, nullptr);
    for (uint32_t i = 0; i < n && e == cudaSuccess; i++) e = cudaEventCreateWithFlags(&b->viewReady[i], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->frameDone, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreate(&b->t0);
    if (e == cudaSuccess) e = cudaEventCreate(&b->t1);
    if (e != cudaSuccess) {
        free_batch(b);
        delete b;
        return cuda_error(e, "vxr_batch_create");
    }
    *out = b;
    return VXR_OK;
}

int vxr_batch_destroy(vxr_batch* b) {
    if (!b) return VXR_OK;
    cudaStreamSynchronize(b->stream);
    free_batch(b);
    delete b;
    return VXR_OK;
}

int vxr_batch_render(vxr_batch* b) {
    VXR_CHECK_ARG(b, "vxr_batch_render: null batch");
    const size_t n = b->views.size();
    for (vxr_view* v : b->views) {
        if (v->useProposal) return vxr::set_error(VXR_E_INVALID, "vxr_batch_render: a view uses a learned proposal");
        if (v->frameOpen) return vxr::set_error(VXR_E_STATE, "vxr_batch_render: a view has a frame in progress");
    }
    const int slot = (int)(b->frames & 1u);
    if (b->slotUsed[slot]) {
        const cudaError_t e = cudaEventSynchronize(b->slotDone[slot]);
        if (e != cudaSuccess) return cuda_error(e, "vxr_batch_render: wait for staging slot");
    }
    // the shading kernel has a sky-dome variant: recorded graphs follow the views' skies
    int sky = 0;
    for (vxr_view* v : b->views) sky |= v->skyDev != nullptr ? 1 : 0;
    if (sky != b->sky) {
        const cudaError_t e = cudaStreamSynchronize(b->stream);
        if (e != cudaSuccess) return cuda_error(e, "vxr_batch_render: wait before re-recording");
        for (int i = 0; i < 2; i++) {
            if (b->graph[i]) cudaGraphExecDestroy(b->graph[i]);
            b->graph[i] = nullptr;
        }
        b->sky = sky;
        for (BatchChain& c : b->chains) c.bd.sky = sky;
    }
    // begin every view's frame (camera, frame constants, G-buffer swap) and fill the table
    // (slot s holds view order[s]; tiles and hit-list view numbers count within a chain)
    for (size_t i = 0; i < n; i++) {
        if (int r = vxr_view_begin_frame(b->views[i], nullptr)) {
            for (size_t j = 0; j < i; j++) vxr_view_end_frame(b->views[j]);
            return r;
        }
    }
    uint32_t tileBase = 0;
    for (size_t s = 0, c = 0; s < n; s++) {
        if (s == b->chains[c].first + b->chains[c].count) c++;
        if (s == b->chains[c].first) tileBase = 0;
        vxr_view* v = b->views[b->order[s]];
        vxr::ViewDev& d = b->staging[slot][s];
        d = vxr::ViewDev();
        d.w = vxr::dev_world(v);
        d.k = vxr::dev_frame(v->k);
        d.k.sky = v->skyDev;
        d.b = v->buf;
        d.cur = v->cur;
        d.point = v->desc.light_model == VXR_LIGHTS_POINT ? 1 : 0;
        d.tilesX = (v->desc.width + (uint32_t)b->tx - 1) / (uint32_t)b->tx;
        d.tileBase = tileBase;
        tileBase += d.tilesX * ((v->desc.height + (uint32_t)b->ty - 1) / (uint32_t)b->ty);
    }
    cudaError_t e = cudaSuccess;
    // order after each view's earlier work
    for (size_t i = 0; i < n && e == cudaSuccess; i++) {
        e = cudaEventRecord(b->viewReady[i], b->views[i]->stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(b->stream, b->viewReady[i], 0);
    }
    if (e == cudaSuccess) e = cudaEventRecord(b->t0, b->stream);
    if (e == cudaSuccess && b->useGraph) {
        if (!b->graph[slot]) {
            cudaGraph_t g = nullptr;
            e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                enqueue_frame(b, slot);
                e = cudaStreamEndCapture(b->stream, &g);
            }
            if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph[slot], g, 0);
            if (g) cudaGraphDestroy(g);
        }
        if (e == cudaSuccess) e = cudaGraphLaunch(b->graph[slot], b->stream);
    } else if (e == cudaSuccess) {
        enqueue_frame(b, slot);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(b->t1, b->stream);
    if (e == cudaSuccess) e = cudaEventRecord(b->slotDone[slot], b->stream);
    if (e == cudaSuccess) e = cudaEventRecord(b->frameDone, b->stream);
    // later work on each view's stream waits for the frame
    for (size_t i = 0; i < n && e == cudaSuccess; i++) e = cudaStreamWaitEvent(b->views[i]->stream, b->frameDone, 0);
    for (vxr_view* v : b->views) vxr_view_end_frame(v);
    if (e != cudaSuccess) return cuda_error(e, "vxr_batch_render");
    b->slotUsed[slot] = true;
    b->timed = true;
    b->frames++;
    return VXR_OK;
}

int vxr_batch_set_tuning(vxr_batch* b, const vxr_tuning* t) {
    VXR_CHECK_ARG(b, "vxr_batch_set_tuning: null batch");
    if (int r = vxr::check_tuning(t, "vxr_batch_set_tuning")) return r;
    cudaError_t e = cudaStreamSynchronize(b->stream);   // recorded graphs may still run
    if (e != cudaSuccess) return cuda_error(e, "vxr_batch_set_tuning");
    uint64_t tiles = 0;
    for (vxr_view* v : b->views)
        tiles += (uint64_t)((v->desc.width + t->tile_x - 1) / t->tile_x) * ((v->desc.height + t->tile_y - 1) / t->tile_y);
    VXR_CHECK_ARG(tiles < (1ull << 32), "vxr_batch_set_tuning: batch too large");
    for (BatchChain& c : b->chains) {
        uint64_t tl = 0;
        for (uint32_t s = c.first; s < c.first + c.count; s++) {
            const vxr_view* v = b->views[b->order[s]];
            tl += (uint64_t)((v->desc.width + t->tile_x - 1) / t->tile_x) * ((v->desc.height + t->tile_y - 1) / t->tile_y);
        }
        vxr::apply_tuning(c.bd, vxr::to_tuning(*t));
        c.bd.totalTiles = (uint32_t)tl;
    }
    b->tx = (int)t->tile_x;
    b->ty = (int)t->tile_y;
    for (int i = 0; i < 2; i++) {
        if (b->graph[i]) cudaGraphExecDestroy(b->graph[i]);
        b->graph[i] = nullptr;
    }
    return VXR_OK;
}

int vxr_batch_wait(vxr_batch* b, float* ms) {
    VXR_CHECK_ARG(b, "vxr_batch_wait: null batch");
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return cuda_error(e, "vxr_batch_wait");
    if (ms) {
        *ms = 0.0f;
        if (b->timed && cudaEventElapsedTime(ms, b->t0, b->t1) != cudaSuccess) *ms = 0.0f;
    }
    uint32_t any = 0;
    for (vxr_view* v : b->views) {
        uint32_t err = 0;
        e = cudaMemcpy(&err, v->buf.err, sizeof(err), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_error(e, "vxr_batch_wait: read device error flags");
        if (err) {
            cudaMemset(v->buf.err, 0, sizeof(uint32_t));
            any |= err;
        }
    }
    if (any)
        return vxr::set_error(VXR_E_DEVICE, vxr::device_flags_message(any));
    return VXR_OK;
}

}  // extern "C"
