/*
 * vxr_oracle.h - CPU restatement of the reference's per-frame Voxel ReSTIR path.
 *
 * TEST INFRASTRUCTURE ONLY. This is the oracle that the CUDA path is checked against:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use it, never the
 * product. Plain C11, one work item per pixel (OpenMP over rows when available).
 * Every function cites the reference file:line it restates. Its results are pinned
 * against the reference's own kernel source compiled for the CPU (oracle/_ref).
 */
#ifndef VXR_ORACLE_H
#define VXR_ORACLE_H
#include <stdint.h>
#include "vxr.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_ctx orc_ctx;

/* ---- world -------------------------------------------------------------------- */
/* updateUberGrid (cl/kernels.cl:498-513) */
void orc_build_uber(const uint32_t* grid, uint8_t* uber);
/* World::Get (template/world.h:293-306) */
uint32_t orc_world_get(const uint32_t* grid, const uint32_t* bricks, uint32_t x, uint32_t y, uint32_t z);
/* World::FindLightsInWord (template/world.cpp:438-504); returns the count, writes at most cap */
uint32_t orc_scan_lights(const uint32_t* grid, const uint32_t* bricks, vxr_light* out, uint32_t cap);

/* A restated World::Set store (template/world.h:456-513, 392-445) with its own brick pool. */
typedef struct orc_store orc_store;
orc_store* orc_store_create(void);
void orc_store_destroy(orc_store* s);
void orc_store_set(orc_store* s, uint32_t x, uint32_t y, uint32_t z, uint32_t v);
uint32_t orc_store_get(const orc_store* s, uint32_t x, uint32_t y, uint32_t z);
uint32_t orc_store_optimize(orc_store* s);  /* World::OptimizeBricks (world.cpp:655-683) */
uint32_t orc_store_lights(const orc_store* s, vxr_light* out, uint32_t cap);   /* incremental list */
const uint32_t* orc_store_grid(const orc_store* s);
const uint32_t* orc_store_bricks(const orc_store* s);

/* ---- camera (template/precomp.h:825-835; world.cpp:2144-2191, 2335-2337) ----------- */
typedef struct orc_camera {
    float M[16];
    float E[3], p0[3], p1[3], p2[3];
    int first;
    uint32_t rng, frame, framecount, restirtemporalframe;
} orc_camera;
void orc_camera_init(orc_camera* c, uint32_t rng_seed);
void orc_lookat(orc_camera* c, const float pos[3], const float target[3]);
void orc_begin_frame(orc_camera* c, uint32_t W, uint32_t H, vxr_frame_consts* k);
void orc_end_frame(orc_camera* c);

/* ---- render path ----------------------------------------------------------------- */
orc_ctx* orc_create(int W, int H, int point_lights);
void orc_destroy(orc_ctx* c);
void orc_set_world(orc_ctx* c, const uint32_t* grid, const uint8_t* uber, const uint32_t* bricks);
void orc_set_lights(orc_ctx* c, const vxr_light* l, uint32_t n);
/* candidates from another source pdf for stage 2 (null: uniform, the reference's): light
 * idx[m * stride + pixel] with pdf p[m * stride + pixel], m < min(N, numberOfCandidates);
 * the arrays stay owned by the caller */
void orc_set_candidates(orc_ctx* c, const uint32_t* idx, const float* p, size_t stride);
/* buffer bookkeeping at the start of World::Render (world.cpp:2209-2223) */
void orc_frame_start(orc_ctx* c);
/* 1 renderAlbedo, 2 perPixelInitialSampling, 3 perPixelSpatialResampling, 4 renderRIS,
 * 5 accumulatorFinalizer; rows [y0, y1) only (y1 <= 0 means all rows) */
void orc_stage(orc_ctx* c, const vxr_frame_consts* k, int stage, int y0, int y1);
/* which: 0 current, 1 previous */
void orc_read_gbuffer(const orc_ctx* c, int which, vxr_gbuffer_rec* out);
void orc_write_gbuffer(orc_ctx* c, int which, const vxr_gbuffer_rec* in, const vxr_frame_consts* k);
/* role: 0 candidate output, 1 spatial output (after the shading discard), 2 shading copy */
void orc_read_reservoirs(const orc_ctx* c, int role, vxr_reservoir_rec* out);
void orc_write_reservoirs(orc_ctx* c, int role, const vxr_reservoir_rec* in);
/* 0 frame (rgb, dist), 1 accumulator */
void orc_read_image(const orc_ctx* c, int which, float* rgba);
/* one ray: mode 0 TraceRay, 1 TraceOpaqueRay, 2 TraceThrough (cl/trace.cl:121-362) */
uint32_t orc_trace(const orc_ctx* c, int mode, const float O[3], const float D[3], int steps, uint32_t through,
                   uint32_t mask, float* dist, uint32_t* side);
/* the oracle's sin/cos of the spatial taps (same definition as the product's) */
void orc_sincos(float a, float* s, float* c);

#ifdef __cplusplus
}
#endif
#endif
