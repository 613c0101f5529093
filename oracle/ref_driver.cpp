// ref_driver.cpp - host driver that runs the reference's own render-path kernels
// (compiled from cl/*.cl by oracle/ref_build.py) over every pixel on the CPU.
//
// TEST INFRASTRUCTURE ONLY (reference oracle, oracle/_ref). It reproduces the
// dataflow of World::Render (template/world.cpp:2127-2340): the 5 kernels in order,
// the reservoir-buffer ping-pong (world.cpp:2209-2219) and the G-buffer swap
// (world.cpp:2221-2223). Work items run as an OpenMP loop over pixels; every kernel
// only writes its own pixel, so the loop is race-free.
//
// Compiled twice (VXREF_VARIANT 0 = area lights, 1 = point lights); each object
// exports its entry points with a _area / _point suffix.
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>
#include "vxr.h"
#undef isnan
#undef isinf

namespace {
int vxref_scr_width = 0, vxref_scr_height = 0;
#include "ref_shim.inc"
#include "_ref/vxref_gen.inc"

struct Ctx {
    int W = 0, H = 0;
    const uint* grid = nullptr;
    const uchar* uber = nullptr;
    const uint* bricks = nullptr;
    std::vector<Light> lights;
    std::vector<CLRay> gb[2];
    std::vector<Reservoir> res[2];
    std::vector<float4> frame, accum, outimg;
    // World::Render statics (world.cpp:2209-2223)
    int reservoirOut = 0, reservoirIn = 1;
    int gbCurrent = 0, gbPrevious = 1;
    // indices for the current frame
    int candOut = 0, candIn = 1, spatOut = 1, spatIn = 0, shadeOut = 0, shadeIn = 1;
    RenderParams params;
    DebugInfo dbg;
    // sky dome (World::LoadSky / UpdateSkylights, world.cpp:803-923); off when empty
    std::vector<float4> sky;
    std::vector<uint> blueNoise;
    uint skyW = 0, skyH = 0;
    float skyLight[24] = {};
    float skyLightScale = 0.0f;
};

void fill_params(Ctx* c, const vxr_frame_consts* k) {
    RenderParams& p = c->params;
    std::memset(&p, 0, sizeof(p));
    p.E = float3(k->E[0], k->E[1], k->E[2]);
    p.p0 = float3(k->p0[0], k->p0[1], k->p0[2]);
    p.p1 = float3(k->p1[0], k->p1[1], k->p1[2]);
    p.p2 = float3(k->p2[0], k->p2[1], k->p2[2]);
    p.oneOverRes = float2(k->oneOverRes[0], k->oneOverRes[1]);
    p.R0 = k->R0;
    p.frame = k->frame;
    p.framecount = k->framecount;
    p.restirtemporalframe = k->restirtemporalframe;
    p.Nleft = float4(k->Nleft[0], k->Nleft[1], k->Nleft[2], k->Nleft[3]);
    p.Nright = float4(k->Nright[0], k->Nright[1], k->Nright[2], k->Nright[3]);
    p.Ntop = float4(k->Ntop[0], k->Ntop[1], k->Ntop[2], k->Ntop[3]);
    p.Nbottom = float4(k->Nbottom[0], k->Nbottom[1], k->Nbottom[2], k->Nbottom[3]);
    p.accumulate = k->accumulate;
    p.spatial = k->spatial;
    p.temporal = k->temporal;
    p.skyDomeSampling = c->sky.empty() ? 0 : 1;
    p.skyWidth = c->skyW;
    p.skyHeight = c->skyH;
    for (int i = 0; i < 6; i++)
        p.skyLight[i] = float4(c->skyLight[4 * i], c->skyLight[4 * i + 1], c->skyLight[4 * i + 2], c->skyLight[4 * i + 3]);
    p.skyLightScale = c->skyLightScale;
    p.editorEnabled = 0;
    p.drawGrid = 0;
    p.numberOfLights = k->numberOfLights;
    p.numberOfCandidates = k->numberOfCandidates;
    p.numberOfMaxTemporalImportance = k->numberOfMaxTemporalImportance;
    p.spatialRadius = k->spatialRadius;
    p.spatialTaps = k->spatialTaps;
    vxref_scr_width = c->W;
    vxref_scr_height = c->H;
}

int g_y0 = 0, g_y1 = 0;   // row range of the next stage (0, 0 = all rows)

template <class F>
void for_pixels(Ctx* c, F f) {
    const int W = c->W;
    const int y0 = g_y0, y1 = (g_y1 > 0 && g_y1 <= c->H) ? g_y1 : c->H;
#pragma omp parallel for schedule(dynamic, 1)
    for (int y = y0; y < y1; y++)
        for (int x = 0; x < W; x++) {
            vx_gid[0] = x;
            vx_gid[1] = y;
            f();
        }
}

image3d_t grid_image(Ctx* c) { image3d_t g; g.data = c->grid; return g; }

Light* lights_ptr(Ctx* c) {
    static Light dummy = {0, 0, 1};
    return c->lights.empty() ? &dummy : c->lights.data();
}

}  // namespace

#if VXREF_VARIANT == 0
#define VXREF_FN(n) n##_area
#else
#define VXREF_FN(n) n##_point
#endif

extern "C" {

void* VXREF_FN(vxref_create)(int W, int H) {
    Ctx* c = new Ctx();
    c->W = W;
    c->H = H;
    const size_t n = (size_t)W * H;
    for (int i = 0; i < 2; i++) {
        c->gb[i].assign(n, CLRay());
        c->res[i].assign(n, Reservoir());
        std::memset(c->gb[i].data(), 0, n * sizeof(CLRay));
        std::memset(c->res[i].data(), 0, n * sizeof(Reservoir));
    }
    c->frame.assign(n, float4(0.0f));
    c->accum.assign(n, float4(0.0f));
    c->outimg.assign(n, float4(0.0f));
    std::memset(&c->dbg, 0, sizeof(c->dbg));
    return c;
}

void VXREF_FN(vxref_destroy)(void* ctx) { delete (Ctx*)ctx; }

void VXREF_FN(vxref_set_world)(void* ctx, const uint32_t* grid, const uint8_t* uber, const uint32_t* bricks) {
    Ctx* c = (Ctx*)ctx;
    c->grid = grid;
    c->uber = uber;
    c->bricks = bricks;
}

void VXREF_FN(vxref_set_lights)(void* ctx, const vxr_light* l, uint32_t n) {
    Ctx* c = (Ctx*)ctx;
    c->lights.resize(n);
    for (uint32_t i = 0; i < n; i++) {
        c->lights[i].position = l[i].position;
        c->lights[i].voxel = l[i].voxel;
        c->lights[i].size = l[i].size;
    }
}

// updateUberGrid (kernels.cl:498-513) over the 32^3 cells
void VXREF_FN(vxref_update_uber)(const uint32_t* grid, uint8_t* uber) {
#pragma omp parallel for
    for (int task = 0; task < 32 * 32 * 32; task++) {
        vx_gid[0] = task;
        updateUberGrid((const uint*)grid, (uchar*)uber);
    }
}

// Frame prologue: the buffer-index bookkeeping of World::Render (world.cpp:2209-2223).
void VXREF_FN(vxref_begin_frame)(void* ctx) {
    Ctx* c = (Ctx*)ctx;
    c->candOut = c->reservoirOut; c->candIn = c->reservoirIn;
    std::swap(c->reservoirOut, c->reservoirIn);
    c->spatOut = c->reservoirOut; c->spatIn = c->reservoirIn;
    std::swap(c->reservoirOut, c->reservoirIn);
    c->shadeOut = c->reservoirOut; c->shadeIn = c->reservoirIn;
    std::swap(c->reservoirOut, c->reservoirIn);
    std::swap(c->gbCurrent, c->gbPrevious);
}

// stage: 1 albedo, 2 candidates+temporal, 3 spatial, 4 shading, 5 accumulate,
// 6 the path-tracer ground truth (renderPathTracer, kernels.cl:177-260) into the frame
void VXREF_FN(vxref_stage)(void* ctx, const vxr_frame_consts* k, int stage) {
    Ctx* c = (Ctx*)ctx;
    fill_params(c, k);
    CLRay* prevAlbedo = c->gb[c->gbPrevious].data();
    CLRay* albedo = c->gb[c->gbCurrent].data();
    RenderParams* params = &c->params;
    image3d_t grid = grid_image(c);
    const uchar* uber = c->uber;
    const uint* brick0 = c->bricks;
    DebugInfo* dbg = &c->dbg;
    Light* lights = lights_ptr(c);
    float4* sky = c->sky.empty() ? nullptr : c->sky.data();
    const uint* bn = c->blueNoise.empty() ? nullptr : c->blueNoise.data();
    switch (stage) {
    case 1:
        for_pixels(c, [&] { renderAlbedo(dbg, prevAlbedo, albedo, params, grid, uber, brick0); });
        break;
    case 2: {
        Reservoir* out = c->res[c->candOut].data();
        Reservoir* in = c->res[c->candIn].data();
        for_pixels(c, [&] {
            perPixelInitialSampling(dbg, prevAlbedo, albedo, params, lights, out, in, grid, uber, brick0);
        });
        break;
    }
    case 3: {
        Reservoir* out = c->res[c->spatOut].data();
        Reservoir* in = c->res[c->spatIn].data();
        for_pixels(c, [&] {
            perPixelSpatialResampling(dbg, prevAlbedo, albedo, params, lights, out, in, grid, uber, brick0);
        });
        break;
    }
    case 4: {
        Reservoir* out = c->res[c->shadeOut].data();
        Reservoir* in = c->res[c->shadeIn].data();
        float4* frame = c->frame.data();
        for_pixels(c, [&] {
            renderRIS(dbg, prevAlbedo, albedo, frame, params, lights, out, in, grid, sky, bn, uber, brick0);
        });
        break;
    }
    case 5: {
        image2d_t img;
        img.data = c->outimg.data();
        img.width = c->W;
        float4* frame = c->frame.data();
        float4* acc = c->accum.data();
        for_pixels(c, [&] { accumulatorFinalizer(img, frame, acc, params); });
        break;
    }
    case 6: {
        float4* frame = c->frame.data();
        for_pixels(c, [&] { renderPathTracer(frame, params, grid, nullptr, nullptr, uber, brick0); });
        break;
    }
    default:
        std::abort();
    }
}

// Sky dome: texels (w * h float4), skyLight[6] (24 floats), skyLightScale and the
// blue-noise buffer (VXR_BLUE_NOISE_WORDS words, world.cpp:180-189); rgba = null: off.
void VXREF_FN(vxref_set_sky)(void* ctx, const float* rgba, uint32_t w, uint32_t h, const float* light, float scale,
                             const uint32_t* bn) {
    Ctx* c = (Ctx*)ctx;
    c->sky.clear();
    c->blueNoise.clear();
    c->skyW = c->skyH = 0;
    if (!rgba) return;
    c->sky.resize((size_t)w * h);
    for (size_t i = 0; i < (size_t)w * h; i++)
        c->sky[i] = float4(rgba[4 * i], rgba[4 * i + 1], rgba[4 * i + 2], rgba[4 * i + 3]);
    c->blueNoise.assign(bn, bn + VXR_BLUE_NOISE_WORDS);
    c->skyW = w;
    c->skyH = h;
    std::memcpy(c->skyLight, light, sizeof(c->skyLight));
    c->skyLightScale = scale;
}

// Rows [y0, y1) only (a bounded sample of a frame, for CPU timing).
void VXREF_FN(vxref_stage_rows)(void* ctx, const vxr_frame_consts* k, int stage, int y0, int y1) {
    g_y0 = y0;
    g_y1 = y1;
    VXREF_FN(vxref_stage)(ctx, k, stage);
    g_y0 = 0;
    g_y1 = 0;
}

// Frame epilogue is the host counter update (world.cpp:2335-2337), done by the caller
// through the frame constants; nothing to do here.

// Readback helpers. which_gb: 0 = current, 1 = previous.
void VXREF_FN(vxref_read_gbuffer)(void* ctx, int which, vxr_gbuffer_rec* out, float* dirs) {
    Ctx* c = (Ctx*)ctx;
    const CLRay* g = c->gb[which == 0 ? c->gbCurrent : c->gbPrevious].data();
    const size_t n = (size_t)c->W * c->H;
    for (size_t i = 0; i < n; i++) {
        out[i].voxel = g[i].voxelValue;
        out[i].dist = g[i].distance;
        out[i].side = g[i].side;
        out[i].seed = g[i].seed;
        if (dirs) {
            dirs[3 * i + 0] = g[i].rayDirection.x;
            dirs[3 * i + 1] = g[i].rayDirection.y;
            dirs[3 * i + 2] = g[i].rayDirection.z;
        }
    }
}

// role: 0 = candidate-stage output, 1 = spatial-stage output (after the shading
// discard write-back), 2 = shading copy (the next frame's temporal history)
void VXREF_FN(vxref_read_reservoirs)(void* ctx, int role, vxr_reservoir_rec* out) {
    Ctx* c = (Ctx*)ctx;
    const int idx = role == 0 ? c->candOut : (role == 1 ? c->spatOut : c->shadeOut);
    const Reservoir* r = c->res[idx].data();
    const size_t n = (size_t)c->W * c->H;
    for (size_t i = 0; i < n; i++) {
        out[i].sumOfWeights = r[i].sumOfWeights;
        out[i].streamLength = r[i].streamLength;
        out[i].lightIndex = r[i].lightIndex;
        out[i].adjustedWeight = r[i].adjustedWeight;
        out[i].positionOnVoxel[0] = r[i].positionOnVoxel.x;
        out[i].positionOnVoxel[1] = r[i].positionOnVoxel.y;
        out[i].positionOnVoxel[2] = r[i].positionOnVoxel.z;
        out[i].invPositionProbability = r[i].invPositionProbability;
        out[i].Nlight[0] = r[i].Nlight.x;
        out[i].Nlight[1] = r[i].Nlight.y;
        out[i].Nlight[2] = r[i].Nlight.z;
        out[i].pHat = r[i].pHat;
    }
}

// Inject reservoirs into a role's buffer for the current frame (stage isolation).
void VXREF_FN(vxref_write_reservoirs)(void* ctx, int role, const vxr_reservoir_rec* in) {
    Ctx* c = (Ctx*)ctx;
    const int idx = role == 0 ? c->candOut : (role == 1 ? c->spatOut : c->shadeOut);
    Reservoir* r = c->res[idx].data();
    const size_t n = (size_t)c->W * c->H;
    for (size_t i = 0; i < n; i++) {
        std::memset(&r[i], 0, sizeof(Reservoir));
        r[i].sumOfWeights = in[i].sumOfWeights;
        r[i].streamLength = in[i].streamLength;
        r[i].lightIndex = in[i].lightIndex;
        r[i].adjustedWeight = in[i].adjustedWeight;
        r[i].positionOnVoxel = float3(in[i].positionOnVoxel[0], in[i].positionOnVoxel[1], in[i].positionOnVoxel[2]);
        r[i].invPositionProbability = in[i].invPositionProbability;
        r[i].Nlight = float3(in[i].Nlight[0], in[i].Nlight[1], in[i].Nlight[2]);
        r[i].pHat = in[i].pHat;
    }
}

// 0 = frame (rgb, dist), 1 = accumulator, 2 = output image
void VXREF_FN(vxref_read_image)(void* ctx, int which, float* out4) {
    Ctx* c = (Ctx*)ctx;
    const std::vector<float4>& v = which == 0 ? c->frame : (which == 1 ? c->accum : c->outimg);
    std::memcpy(out4, v.data(), v.size() * sizeof(float4));
}

// Single-ray entry points of the three DDA variants (trace.cl:121-362), for
// unit tests of the traversal. mode 0 TraceRay, 1 TraceOpaqueRay, 2 TraceThrough.
uint32_t VXREF_FN(vxref_trace)(void* ctx, int mode, const float* O, const float* D, int steps,
                              uint32_t through, uint32_t mask, float* dist, uint32_t* side) {
    Ctx* c = (Ctx*)ctx;
    image3d_t grid = grid_image(c);
    float d = 0.0f;
    uint s = 0;
    const float4 A(O[0], O[1], O[2], 0.0f), B(D[0], D[1], D[2], 1.0f);
    uint v;
    if (mode == 0) v = TraceRay(A, B, &d, &s, grid, c->uber, c->bricks, steps);
    else if (mode == 1) v = TraceOpaqueRay(A, B, &d, &s, grid, c->uber, c->bricks, steps);
    else v = TraceThrough(through, mask, A, B, &d, &s, grid, c->uber, c->bricks, steps);
    *dist = d;
    *side = s;
    return v;
}

}  // extern "C"
