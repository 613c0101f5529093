/*
 * vxr.h - C ABI of the GB300-native Voxel ReSTIR renderer (libvxr.so).
 *
 * Drop-in boundary for the per-frame render path of the WrldTmpl8/SmallProject
 * reference: the World class (template/world.h:164-758) and the worldapi free
 * functions (template/worldapi.h:1-102, bodies template/template.cpp:49-341).
 * Every entry point names the reference interface it replaces.
 *
 * Conventions
 *  - Every function returns an int status: VXR_OK (0) or a negative VXR_E_* code.
 *    vxr_last_error() returns a thread-local message for the last failure.
 *    (The reference calls FatalError and exits instead: template.cpp:1161-1224.)
 *  - Plain pointers and sizes only; no C++ or torch types cross the boundary.
 *  - A vxr_world is a host-side voxel store (1024^3 map in 8^3 bricks, exactly the
 *    reference's fixed map: common.h:16-21). A vxr_view renders one camera view of
 *    one world on the GPU. Calls on one view are not thread-safe; separate views
 *    own separate CUDA streams.
 *  - Render calls are asynchronous (like World::Render, world.cpp:2127); vxr_wait
 *    blocks and reports device-side errors (like World::Commit, world.cpp:2357).
 */
#ifndef VXR_H
#define VXR_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------- */
#define VXR_OK             0
#define VXR_E_INVALID     -1   /* bad argument (null pointer, size out of range) */
#define VXR_E_CUDA        -2   /* CUDA runtime error (message in vxr_last_error) */
#define VXR_E_NOMEM       -3   /* host or device allocation failed */
#define VXR_E_STATE       -4   /* call out of order (e.g. render before upload) */
#define VXR_E_DEVICE      -5   /* a kernel raised its device error flag */
#define VXR_E_NODEVICE    -6   /* no CUDA device visible */
#define VXR_E_IO          -7   /* file read/write failed or malformed file */

/* ---- map geometry (fixed, reference common.h:16-21, 176-183) --------------- */
#define VXR_MAPDIM     1024u  /* MAPWIDTH = MAPHEIGHT = MAPDEPTH */
#define VXR_BRICKDIM   8u     /* BRICKDIM */
#define VXR_GRIDDIM    128u   /* GRIDWIDTH = MAPWIDTH / BRICKDIM */
#define VXR_UBERDIM    32u    /* UBERWIDTH = GRIDWIDTH / 4 */
#define VXR_BRICKSIZE  512u   /* BRICKSIZE = 8^3 voxels */
/* Words of the blue-noise buffer (world.cpp:180-189): the 8-bit entries of E. Heitz's
 * sampler tables, one per uint32: sequence at [0, 65536), scrambling at
 * [65536, 196608), ranking at [196608, 327680). */
#define VXR_BLUE_NOISE_WORDS 327680u

/* Voxel payload: 32-bit 0x00MMARGB (common.h:32-37, tools.cl:294-322):
 * B bits 0-3, G 4-7, R 8-11, alpha 12-15 (0xF = opaque), emitter strength M 16-23. */
#define VXR_VOXEL(r4, g4, b4, a4, m8) \
    ((((uint32_t)(m8) & 255u) << 16) | (((uint32_t)(a4) & 15u) << 12) | \
     (((uint32_t)(r4) & 15u) << 8) | (((uint32_t)(g4) & 15u) << 4) | ((uint32_t)(b4) & 15u))

/* ---- records shared with the reference -------------------------------------- */

/* Emitter record, identical to the reference struct Light (common.h:134-139):
 * position = x + z*1024 + y*1024*1024, voxel = payload, size = 1 (voxel) or 8 (solid brick). */
typedef struct vxr_light {
    uint32_t position;
    uint32_t voxel;
    uint32_t size;
} vxr_light;

/* Canonical G-buffer record: the reference CLRay (common.h:125-132) without the
 * ray direction, which is a pure function of the camera and the pixel. */
typedef struct vxr_gbuffer_rec {
    uint32_t voxel;   /* re-encoded albedo voxel (ris.cl:381) */
    float    dist;    /* hit distance along the primary ray */
    uint32_t side;    /* axis of the hit face, 0..2 */
    uint32_t seed;    /* per-pixel xorshift32 state after the stage that last advanced it */
} vxr_gbuffer_rec;

/* Canonical reservoir record: the fields of the reference struct Reservoir
 * (common.h:141-151) in declaration order, float3 members unpacked. */
typedef struct vxr_reservoir_rec {
    float    sumOfWeights;
    uint32_t streamLength;          /* M */
    uint32_t lightIndex;
    float    adjustedWeight;        /* W */
    float    positionOnVoxel[3];
    float    invPositionProbability;
    float    Nlight[3];
    float    pHat;
} vxr_reservoir_rec;

/* Per-frame constants of the render path: the subset of RenderParams
 * (common.h:100-118) read by the five stage kernels, plus the resolution
 * (a compile-time constant in the reference, common.h:2-3). Filled by
 * vxr_view_begin_frame from the camera exactly as World::Render does
 * (world.cpp:2144-2191); exposed so tests can drive stages with explicit inputs. */
typedef struct vxr_frame_consts {
    float    E[3];                  /* camera position */
    float    p0[3], p1[3], p2[3];   /* screen-plane corners */
    float    oneOverRes[2];         /* 1/W, 1/H */
    uint32_t R0;                    /* per-frame random seed (world.cpp:2184) */
    uint32_t frame;                 /* (frame+1) & 255 */
    uint32_t framecount;
    uint32_t restirtemporalframe;   /* temporal reuse is skipped when 0 (ris.cl:85) */
    float    Nleft[4], Nright[4], Ntop[4], Nbottom[4];  /* previous-frame frustum planes */
    int32_t  accumulate, spatial, temporal;
    uint32_t numberOfLights;
    uint32_t numberOfCandidates;    /* NUMBEROFCANDIDATES (32) */
    uint32_t numberOfMaxTemporalImportance;  /* TEMPORALMAXIMPORTANCE (20) */
    uint32_t spatialRadius;         /* SPATIALRADIUS (30) */
    uint32_t spatialTaps;           /* SPATIALTAPS (5) */
    uint32_t width, height;         /* SCRWIDTH, SCRHEIGHT */
} vxr_frame_consts;

/* Light model, the reference's compile-time VOXELSAREPOINTLIGHTS (common.h:70). */
#define VXR_LIGHTS_AREA   0   /* solid-angle voxel-side importance sampling (tools.cl:499-577) */
#define VXR_LIGHTS_POINT  1   /* emitter = point at the voxel centre (tools.cl:609-616) */

/* ---- library ------------------------------------------------------------------ */

/* Message of the last failing call on this thread ("" if none). */
const char* vxr_last_error(void);
/* Library version string. */
const char* vxr_version(void);

/* ---- world: host voxel store (World, template/world.h:164-758) ------------------ */
typedef struct vxr_world vxr_world;

/* World::World + World::Clear (world.cpp:47-193, 726-745): an empty 1024^3 map. */
int vxr_world_create(vxr_world** out);
int vxr_world_destroy(vxr_world* w);
/* World::Clear (world.cpp:726-745) / ClearWorld (template.cpp:60). */
int vxr_world_clear(vxr_world* w);
/* World::Set (world.h:456-513) / Plot (template.cpp:64). Out-of-map coordinates are
 * ignored like the reference. When light tracking is on (the default), an emitter
 * voxel is appended to the light list (World::AddLight, world.cpp:228-246) and an
 * overwritten emitter is removed (World::RemoveLight, world.cpp:506-561). */
int vxr_world_set(vxr_world* w, uint32_t x, uint32_t y, uint32_t z, uint32_t voxel);
/* World::AddBrick (world.h:308-352): grid cell (bx, by, bz) becomes solid with value
 * voxel; a brick stored there is recycled. With light tracking on, the cell's old
 * emitters leave the light list and an emitter voxel joins it as one brick light
 * (size 8, position = the cell's lowest corner). Out-of-grid cells are ignored. */
int vxr_world_add_brick(vxr_world* w, uint32_t bx, uint32_t by, uint32_t bz, uint32_t voxel);
/* World::StampSpriteTo (world.cpp:1545-1563): vxr_world_set(x + ox, y + oy, z + oz,
 * voxels[i] | or_mask) for i = 0 .. n-1 in order, with pos[i] = x | y << 10 | z << 20
 * (a sprite's draw list; the reference stamps with or_mask 0xF000). The bulk path for
 * loading scene files. */
int vxr_world_stamp(vxr_world* w, const uint32_t* pos, const uint32_t* voxels, uint32_t n, uint32_t ox, uint32_t oy,
                    uint32_t oz, uint32_t or_mask);
/* World::Get (world.h:293-306) / Read (template.cpp:67). Out-of-map reads wrap like
 * the reference's masking. */
int vxr_world_get(const vxr_world* w, uint32_t x, uint32_t y, uint32_t z, uint32_t* voxel);
/* Box (template.cpp:98-101): Plot over [x1,x2) x [y1,y2) x [z1,z2). */
int vxr_world_box(vxr_world* w, int x1, int y1, int z1, int x2, int y2, int z2, uint32_t voxel);
/* Enable/disable incremental light tracking in vxr_world_set (AddLight/RemoveLight). */
int vxr_world_track_lights(vxr_world* w, int enable);
/* World::OptimizeBricks (world.cpp:655-683): collapse single-valued bricks into solid
 * grid cells. Returns the number of bricks replaced in *replaced (may be NULL). */
int vxr_world_optimize(vxr_world* w, uint32_t* replaced);
/* World::FindLightsInWord + SetupLightBuffer (world.cpp:438-504, 563-612): rebuild the
 * light list by scanning the map (brick cells y->z->x, voxels y->z->x; a solid emitter
 * cell is one light of size 8). Returns the count in *count (may be NULL). */
int vxr_world_scan_lights(vxr_world* w, uint32_t* count);
/* World::SetupLightBuffer (world.cpp:563-612) with an explicit list (replaces the list). */
int vxr_world_set_lights(vxr_world* w, const vxr_light* lights, uint32_t n);
/* World::MoveLights for one light (world.cpp:268-305): move voxel light `index` of the
 * light list to (x, y, z). The voxel it covered is restored (0 if none was remembered),
 * its emitter voxel is drawn at the new position and the non-emitter voxel there is
 * remembered; the list keeps its order. Views restart temporal reuse for a moved light
 * only when their spatial reuse is off, as the reference does (world.cpp:300-301).
 * Brick lights (size 8) do not move: VXR_E_INVALID. */
int vxr_world_move_light(vxr_world* w, uint32_t index, uint32_t x, uint32_t y, uint32_t z);
/* Read-only views of the host arrays (valid until the next edit): top-level grid
 * (128^3 uint32, index x + z*128 + y*16384; 0 empty, even = solid colour << 1,
 * odd = brick index << 1 | 1), brick pool (nbricks * 512 uint32, voxel lx + ly*8 + lz*64),
 * light list. Any out-pointer may be NULL. */
int vxr_world_arrays(const vxr_world* w, const uint32_t** grid, const uint32_t** bricks,
                     uint32_t* nbricks, const vxr_light** lights, uint32_t* nlights);
/* Number of bricks in use (allocated minus recycled). */
int vxr_world_brick_count(const vxr_world* w, uint32_t* in_use);

/* ---- emitter clusters (no reference counterpart: the learned candidate proposal
 * chooses a cluster, then an emitter inside it) ---------------------------------------- */
/* Seeded k-means over light centres: k clusters (clamped to the light count),
 * `iters` Lloyd iterations. Deterministic for a given light list and seed. Any later
 * change of the light list invalidates the clustering (re-run it). */
int vxr_world_cluster_lights(vxr_world* w, uint32_t k, uint32_t seed, uint32_t iters);
/* Cluster id per light (valid until the next light-list change) and the cluster count. */
int vxr_world_light_clusters(const vxr_world* w, const uint32_t** ids, uint32_t* k);

/* ---- procedural scenes (no reference counterpart: the thesis scenes need assets
 * that are not available; these generate the benchmark worlds) -------------------- */
#define VXR_EMIT_ABOVE_SURFACE 0  /* uniform (x,z), 1..8 voxels above the terrain */
#define VXR_EMIT_AIR           1  /* uniform through the air volume above the terrain */
#define VXR_EMIT_BLOBS         2  /* blob_fraction in Gaussian blobs, rest uniform in air */
#define VXR_EMIT_LAYER         3  /* a glowing stratum [layer_lo, layer_hi] plus scattered */

typedef struct vxr_scene_desc {
    uint32_t extent;          /* world side in voxels (256, 512 or 1024), at the map origin */
    uint32_t seed;
    uint32_t octaves;         /* fBm octaves */
    float    base_freq;       /* lattice frequency at extent 256 (1/64) */
    float    gain;            /* fBm amplitude gain (0.5) */
    float    height_base;     /* h = s*(height_base + height_amp*fbm), s = extent/256 */
    float    height_amp;
    float    albedo_lo, albedo_hi;   /* per-voxel RGB uniform range, quantised to 4 bit */
    float    cave_threshold;  /* carve where 3D value noise > threshold; 0 disables */
    uint32_t emitters;        /* number of emitter voxels */
    uint32_t emitter_mode;    /* VXR_EMIT_* */
    float    radiance_lo, radiance_hi;   /* emitter RGB uniform range */
    uint32_t blob_count;      /* VXR_EMIT_BLOBS */
    float    blob_sigma;
    float    blob_fraction;
    uint32_t layer_lo, layer_hi;         /* VXR_EMIT_LAYER */
    float    scatter_fraction;
} vxr_scene_desc;

/* Fill desc with the preset of benchmark configuration `config` (0..4). */
int vxr_scene_preset(int config, vxr_scene_desc* desc);
/* Clear the world and generate the scene; ends with OptimizeBricks and a light scan. */
int vxr_scene_generate(vxr_world* w, const vxr_scene_desc* desc);
/* Terrain height (first empty y) of the generated heightfield at column (x, z). */
int vxr_scene_height(const vxr_scene_desc* desc, uint32_t x, uint32_t z, uint32_t* height);
/* Seeded Catmull-Rom camera path through 8 control points above the terrain:
 * position and look-at target for frame f of n_frames. */
int vxr_camera_path(const vxr_scene_desc* desc, uint32_t path_seed, uint32_t f, uint32_t n_frames,
                    float pos[3], float target[3]);
/* 64-bit FNV-1a checksum of the world's canonical content (voxel values by map
 * position, independent of brick numbering) and of its light list. */
int vxr_world_checksum(const vxr_world* w, uint64_t* voxels, uint64_t* lights);

/* ---- camera (host only) ------------------------------------------------------------ */
/* The camera state World::Render keeps between frames (camMat + previous corners +
 * RandomUInt state + frame counters); every view owns one. Exposed on its own so the
 * per-frame constants can be produced and checked without a GPU. */
typedef struct vxr_camera vxr_camera;
int vxr_camera_create(uint32_t rng_seed, vxr_camera** out);
int vxr_camera_destroy(vxr_camera* c);
int vxr_camera_lookat(vxr_camera* c, const float pos[3], const float target[3]);   /* mat4::LookAt */
int vxr_camera_set_matrix(vxr_camera* c, const float m[16]);
/* world.cpp:2144-2191: corners, previous-frame planes, R0, counters -> *k (resolution W x H).
 * Only the camera-derived fields of *k are written; the knobs are the caller's. */
int vxr_camera_begin_frame(vxr_camera* c, uint32_t W, uint32_t H, vxr_frame_consts* k);
int vxr_camera_end_frame(vxr_camera* c);                                           /* world.cpp:2335-2337 */

/* ---- host memory for end-to-end transfers ------------------------------------------- */
/* Page-locked host buffer (cudaHostAlloc) for vxr_view_render_to_host outputs. */
int vxr_host_alloc(size_t bytes, void** p);
int vxr_host_free(void* p);

/* ---- GPU copy of a world --------------------------------------------------------- */
/* World::ForceSyncAllBricks + the updateUberGrid kernel + SetupLightBuffer's device copy
 * (world.cpp:639-651, kernels.cl:498-513, world.cpp:563-612): upload all of the grid, the
 * bricks and the light list to the current CUDA device, build the 32^3 uber grid and
 * the per-light table there, and the traversal's skip tables (per brick the boxes of
 * its opaque and of its non-zero voxels, 8 bytes; per uber cell the box of its non-zero
 * voxels). Re-upload after edits; views pick up the new copy at their next frame.
 * Synchronous. */
int vxr_world_upload(vxr_world* w);
/* World::Commit + the commit kernel (world.cpp:2357-2420, kernels.cl:448-477): bring the
 * device copy up to date with the edits since the last commit. Only the bricks whose
 * voxels changed are sent (gathered in page-locked memory, copied once, scattered into
 * the device pool by a kernel), the grid only when it changed, the light table only when
 * the light list changed; the uber grid and the skip tables are rebuilt for what changed.
 * Everything is sent when there is no device copy yet, after vxr_world_clear or a scene
 * build, or when new bricks outgrow the device pool (it is then reallocated with 1/8
 * headroom). Unlike the reference there is no per-commit brick limit. Waits for all
 * device work first (frames in flight read these buffers) and is synchronous. Rendering
 * a view commits its world's pending edits the same way. Optional outputs: bricks sent,
 * full = 1 when everything was sent. */
int vxr_world_commit(vxr_world* w, uint32_t* bricks_sent, int* full);
/* What the next commit would send (no reference counterpart: the reference's dirty
 * marks, world.h:565-613, are internal): changed bricks (all bricks when everything is
 * due), whether the grid changed, whether everything is due. Host-only. */
int vxr_world_pending(const vxr_world* w, uint32_t* dirty_bricks, int* grid_changed, int* full);
/* Device bytes held by the world's GPU copy. */
int vxr_world_device_bytes(const vxr_world* w, uint64_t* bytes);

/* ---- views: one camera on one world (World::Render / Commit path) ------------------ */
typedef struct vxr_view vxr_view;

typedef struct vxr_view_desc {
    uint32_t width, height;                /* SCRWIDTH, SCRHEIGHT */
    uint32_t light_model;                  /* VXR_LIGHTS_AREA or VXR_LIGHTS_POINT */
    uint32_t num_candidates;               /* NUMBEROFCANDIDATES, default 32 */
    uint32_t spatial_taps;                 /* SPATIALTAPS, default 5 */
    uint32_t spatial_radius;               /* SPATIALRADIUS, default 30 */
    uint32_t temporal_max_importance;      /* TEMPORALMAXIMPORTANCE, default 20 */
    int32_t  spatial, temporal, accumulate;/* RenderParams toggles (defaults 1, 1, 0) */
    uint32_t rng_seed;                     /* host RandomUInt seed for R0, default 0x12345678 */
    uint32_t tile_x, tile_y;               /* threads per pixel-stage block (<= 256); 0 = library default */
} vxr_view_desc;

int vxr_view_default_desc(vxr_view_desc* d);
/* World::InitReSTIR + SetupReservoirBuffers (world.cpp:195-226): allocate the view's
 * G-buffers, reservoirs and frame buffers on the current device, own CUDA stream. */
int vxr_view_create(vxr_world* w, const vxr_view_desc* d, vxr_view** out);
int vxr_view_destroy(vxr_view* v);
/* LookAt (template.cpp:204-207) -> World::SetCameraMatrix(mat4::LookAt(pos, target)). */
int vxr_view_lookat(vxr_view* v, const float pos[3], const float target[3]);
/* World::SetCameraMatrix with an explicit row-major 4x4 camera-to-world matrix. */
int vxr_view_set_camera_matrix(vxr_view* v, const float m[16]);
/* Change the toggles/knobs of an existing view (RenderParams console knobs,
 * mygame.cpp:112-121); resolution and light model are fixed at creation. */
int vxr_view_set_params(vxr_view* v, const vxr_view_desc* d);

/* Sky dome (RenderParams.skyDomeSampling, common.h:105-112; ris.cl:199-210, 254-290):
 * rgba = NULL turns it off (the default). Otherwise rgba holds w * h texels of 4
 * floats, row by row, as World::LoadSky leaves them (scale * (r, g, b, 1), world.cpp:
 * 861-870); sky_light the 6 integrated sky colours of the axis normals, 4 floats each,
 * in skyLight order (-x, +x, -z, +z, -y, +y of the sky's z-up frame, i.e. selected
 * by the world normals -x, +x, -y, +y, -z, +z; vxr_sky_lights computes them);
 * light_scale skyLightScale; blue_noise VXR_BLUE_NOISE_WORDS words. With the sky on,
 * background pixels take the sky colour, translucent voxels (alpha < 15) blend it in,
 * and shading adds one cosine-weighted ray (10-step budget, opaque voxels only) lit by
 * the sky light of the normal it ends on. Copies everything to the device (blocking).
 * w, h in [1, 65536], w * h < 2^31. */
int vxr_view_set_sky(vxr_view* v, const float* rgba, uint32_t w, uint32_t h, const float sky_light[24],
                     float light_scale, const uint32_t* blue_noise);
/* World::UpdateSkylights (world.cpp:897-922): for each of the 6 normals of skyLight,
 * the mean of 4,096 cosine-weighted samples of the sky (16 x 16 strata, 16 jittered
 * samples each), bilinear like World::SampleSky (world.cpp:878-895). The jitter comes
 * from an xorshift32 stream seeded with `seed` (the reference draws it from its global
 * host RNG, so its values differ by that Monte Carlo noise). Host only. */
int vxr_sky_lights(const float* rgba, uint32_t w, uint32_t h, uint32_t seed, float sky_light[24]);

/* Host part of World::Render (world.cpp:2144-2223): frame constants from the camera,
 * R0, G-buffer swap. Writes the constants to *k when k is not NULL. */
int vxr_view_begin_frame(vxr_view* v, vxr_frame_consts* k);
/* Replace the constants of the frame in progress (stage-isolated testing). */
int vxr_view_set_frame_consts(vxr_view* v, const vxr_frame_consts* k);
/* Launch one stage asynchronously on the view's stream:
 * VXR_STAGE_ALBEDO renderAlbedo, VXR_STAGE_CANDIDATES perPixelInitialSampling,
 * VXR_STAGE_SPATIAL perPixelSpatialResampling, VXR_STAGE_SHADE renderRIS,
 * VXR_STAGE_ACCUMULATE accumulatorFinalizer (world.cpp:2263-2307). */
#define VXR_STAGE_ALBEDO      1
#define VXR_STAGE_CANDIDATES  2
#define VXR_STAGE_SPATIAL     3
#define VXR_STAGE_SHADE       4
#define VXR_STAGE_ACCUMULATE  5
/* renderPathTracer with render_di_gfxexp (kernels.cl:177-260): the reference's
 * ground-truth mode, one hemisphere sample per pixel into the frame buffer (follow with
 * VXR_STAGE_ACCUMULATE, or vxr_view_sum64_add, to converge); not timed per stage. */
#define VXR_STAGE_PATH_TRACE  6
int vxr_view_stage(vxr_view* v, int stage);
/* Frame counters (world.cpp:2335-2337). */
int vxr_view_end_frame(vxr_view* v);
/* World::Render: begin_frame, the five stages (shading and accumulation fused in one
 * kernel), end_frame. Asynchronous. When the previous frame was also rendered by this
 * call with no other call on the view in between, this frame's primary rays, candidates
 * and candidate visibility run on the view's second stream beside the previous frame's
 * shading (same results). */
int vxr_view_render(vxr_view* v);
/* World::Commit's wait (world.cpp:2432-2438): block until the view's work is done,
 * read the stage timings, and report device-side errors as VXR_E_DEVICE. */
int vxr_view_wait(vxr_view* v);
/* Per-stage GPU milliseconds of the last waited frame: albedo, candidates+temporal,
 * spatial, shading, accumulate (GetAlbedoTime ... GetShadingTime, world.h:215-220).
 * A fused shading+accumulate frame reports accumulate as 0. */
int vxr_view_stage_times(vxr_view* v, float ms[5]);

/* Readback / injection in the canonical record formats. which: 0 = current G-buffer,
 * 1 = previous. role: 0 = candidate-stage reservoirs, 1 = spatial-stage reservoirs
 * (after shading's discard write-back, i.e. the next frame's temporal history). */
int vxr_view_read_gbuffer(vxr_view* v, int which, vxr_gbuffer_rec* out);
int vxr_view_write_gbuffer(vxr_view* v, int which, const vxr_gbuffer_rec* in);
int vxr_view_read_reservoirs(vxr_view* v, int role, vxr_reservoir_rec* out);
int vxr_view_write_reservoirs(vxr_view* v, int role, const vxr_reservoir_rec* in);
/* Shaded frame (rgb, primary-hit distance) and accumulator (rgb, 1): float4 per pixel. */
int vxr_view_read_frame(vxr_view* v, float* rgba);
int vxr_view_read_accum(vxr_view* v, float* rgba);
/* Per-stage GPU time summed over every frame finished since the last reset (CUDA
 * events around each stage launch, kept for the last 256 frames between waits), and
 * the number of launches timed; reset != 0 clears the sums after reading. */
int vxr_view_stage_stats(vxr_view* v, double sum_ms[5], uint32_t count[5], int reset);
/* Device-side timer on the view's stream: events recorded before / after the work
 * enqueued in between; vxr_view_timer_end waits and returns the elapsed milliseconds. */
int vxr_view_timer_begin(vxr_view* v);
int vxr_view_timer_end(vxr_view* v, float* ms);
/* Per-kernel timing (no reference counterpart): CUDA events around every kernel the
 * view launches, while on. Kernel ids 0..VXR_KERNEL_COUNT-1 (names from
 * vxr_kernel_name): albedo, compact_hits, proposal_infer, ris_candidates,
 * shadow_candidates, temporal, spatial, shade_request, shadow_shading, shade_finish,
 * accumulate, proposal_train (a frame's online training steps, gather to Adam, as one
 * timed unit). Stats: summed milliseconds and launch counts since the last reset. */
#define VXR_KERNEL_COUNT 12
int vxr_view_kernel_timing(vxr_view* v, int on);
int vxr_view_kernel_stats(vxr_view* v, double sum_ms[VXR_KERNEL_COUNT], uint32_t count[VXR_KERNEL_COUNT], int reset);
const char* vxr_kernel_name(int id);
/* Work of the view's last frame (waits for it): counts[0] hit pixels, counts[1] shadow
 * rays of the candidate stage, counts[2] shadow rays of shading. */
int vxr_view_work_counts(vxr_view* v, uint32_t counts[3]);
/* End-to-end frame through host memory: LookAt(pos, target), render, copy the
 * accumulated image into host_rgba (W*H float4; page-locked memory is fastest), wait. */
int vxr_view_render_to_host(vxr_view* v, const float pos[3], const float target[3], float* host_rgba);
/* The same, pipelined: enqueues the frame and the image copy and returns at once with
 * *ticket; vxr_view_image_wait(v, ticket) returns once that image is in host_rgba (and
 * reports device error flags like vxr_view_wait). Up to 4 images may be in flight (a
 * fifth call first waits for the oldest); give each in-flight image its own host buffer
 * (page-locked, vxr_host_alloc, for the copy to overlap). Rendering frame f + 1 while the
 * host reads image f hides the host's per-frame work behind the device's. */
int vxr_view_render_to_host_async(vxr_view* v, const float pos[3], const float target[3], float* host_rgba,
                                  uint64_t* ticket);
int vxr_view_image_wait(vxr_view* v, uint64_t ticket);

/* ---- learned candidate proposal (no reference counterpart) ------------------------------
 * Replaces the uniform source pdf of RIS (GenerateLightCandidate, tools.cl:593-598) by a
 * small network over the world's emitter clusters (vxr_world_cluster_lights): input =
 * 2-level hash-grid encoding of the shading point + one-hot voxel side, 3 hidden ReLU
 * layers, softmax over K clusters. A candidate is, with probability epsilon, an emitter
 * drawn uniformly, else an emitter drawn uniformly from a cluster c ~ softmax; RIS weighs
 * it with p_hat / p_src, p_src(e) = (1 - epsilon) softmax_c(e) / |c(e)| + epsilon / N.
 * Inference: BF16 tensor cores, FP32 accumulation.
 * Training: online, weighted cross-entropy towards the cluster of each final reservoir's
 * emitter (weight W * p_hat), Adam on FP32 master parameters. The default step runs on
 * the tensor cores (BF16 operands, FP32 accumulation; hidden 64, at most 256 clusters);
 * the FP32 CUDA-core trainer stays selectable. */
typedef struct vxr_proposal_desc {
    uint32_t hidden;          /* hidden width (64) */
    uint32_t table_log2;      /* hash-table entries per level, log2 (16) */
    uint32_t res0, res1;      /* grid resolution of the two levels over the 1024^3 map (32, 128) */
    float    epsilon;         /* weight of the uniform (defensive) emitter mixture (0.1) */
    float    learning_rate;   /* Adam (1e-3) */
    uint32_t batch;           /* training samples per step (65536) */
    uint32_t seed;            /* parameter initialisation */
    uint32_t inference;       /* 0 auto (tcgen05 when hidden = 64 and 256 clusters, else mma.sync), 1 mma.sync, 2 tcgen05 */
    uint32_t training;        /* 0 auto (tensor cores when hidden = 64 and clusters <= 256, else FP32), 1 FP32, 2 tensor cores */
    uint32_t pixels_per_eval; /* tcgen05 inference: 1 = one network evaluation per hit pixel; 2, 4 or 8 = one per run of up to
                                 that many consecutive hit pixels whose shading points lie on the same voxel side as the
                                 run's first within share_distance (all sample from the first one's distribution; still
                                 unbiased) */
    float share_distance;     /* pixels_per_eval > 1: largest per-coordinate distance (voxels) within a shared run */
    uint32_t training_lag;    /* online training (vxr_view_proposal_online): 0 = a frame's inference uses the weights of
                                 the previous frame's training step; 1 = of the step before that, so each step can
                                 overlap the whole next frame */
} vxr_proposal_desc;
int vxr_proposal_default_desc(vxr_proposal_desc* d);
/* Allocate and initialise the network for this view; K = the world's cluster count. */
int vxr_view_proposal_enable(vxr_view* v, const vxr_proposal_desc* d);
/* on = 1: candidates come from the learned proposal; on = 0: uniform (the plain method). */
int vxr_view_proposal_use(vxr_view* v, int on);
/* `steps` Adam steps, each on a batch gathered from the view's current frame (hit
 * pixels, final reservoirs); the last step's loss in *loss (may be NULL). */
int vxr_view_proposal_train(vxr_view* v, uint32_t steps, float* loss);
/* Online training inside the frame: every vxr_view_render (and vxr_view_render_to_host)
 * of a view that samples from the proposal ends with `steps_per_frame` (0..16) training
 * steps on that frame's own final reservoirs, enqueued on the view's stream after
 * shading, so the frame's time includes them. 0 turns it off. */
int vxr_view_proposal_online(vxr_view* v, uint32_t steps_per_frame);
/* Test hook for the device error path (no reference counterpart): on = 1 makes the
 * tcgen05 inference issue no MMA and give each tensor-core wait 64 tries, so every wait
 * runs out with nothing in flight; the kernel raises error flag 16, skips its remaining
 * tiles, frees its tensor memory and returns, the candidate stage falls back to uniform
 * candidates for the entries it did not write, and vxr_view_wait reports VXR_E_DEVICE.
 * on = 0 restores normal operation. */
int vxr_view_proposal_test_timeout(vxr_view* v, int on);
/* The candidates the proposal drew for the view's current frame (after
 * VXR_STAGE_CANDIDATES, before the next frame; no reference counterpart): *nhits hit
 * pixels, hits[j] = pixel of hit-list entry j, cand[(m * nhits + j) * 2 + {0, 1}] = light
 * index and bits(source pdf) of candidate m of entry j, m < min(candidates, lights).
 * hits and cand may be NULL (then only *nhits is written). */
int vxr_view_proposal_read_candidates(vxr_view* v, uint32_t* nhits, uint32_t* hits, uint32_t* cand);
/* Network evaluations of the view's current frame (no reference counterpart): one per hit
 * pixel, or with pixels_per_eval > 1 one per run of pixels sharing an evaluation. */
int vxr_view_proposal_rows(vxr_view* v, uint32_t* rows);
int vxr_view_proposal_param_count(vxr_view* v, uint64_t* n, uint32_t* clusters, uint32_t* hidden);
int vxr_view_proposal_get_params(vxr_view* v, float* out);
int vxr_view_proposal_set_params(vxr_view* v, const float* in);
/* Loss and gradient (no update) on caller samples: samples = B x (x, y, z, side code as
 * uint32 bits; code = axis * 2 + (normal negative)), target cluster, weight. */
int vxr_view_proposal_grad(vxr_view* v, uint32_t B, const float* samples, const uint32_t* target,
                           const float* weight, float* loss, float* grad);
/* softmax probabilities (B x K) of the inference path for caller samples */
int vxr_view_proposal_probs(vxr_view* v, uint32_t n, const float* samples, float* probs);
/* Checkpoint: parameters, Adam moments and step count (versioned binary). */
int vxr_view_proposal_save(vxr_view* v, const char* path);
int vxr_view_proposal_load(vxr_view* v, const char* path);

/* ---- converged reference and error metric --------------------------------------------
 * No counterpart on the reference's GPU path: its validation compared dumped frames
 * offline against a path-traced ground truth (mse.cpp:252-391). Here a view keeps an
 * optional FP64 running sum of its shaded frames (rgb). A converged reference is a view
 * rendered with spatial and temporal reuse off (the unbiased RIS + visibility estimator,
 * same shading) and summed over many frames with distinct seeds. */
/* Clear the view's FP64 sum (allocates it on first use: width*height*3 doubles). */
int vxr_view_sum64_reset(vxr_view* v);
/* Add the current shaded frame (after VXR_STAGE_SHADE / vxr_view_render) to the sum. */
int vxr_view_sum64_add(vxr_view* v);
/* Frames summed so far, and the FP64 mean (width*height*3 doubles) when mean != NULL. */
int vxr_view_sum64_mean(vxr_view* v, uint32_t* count, double* mean);
/* CalculateMSE and CalculateRMAE (mse.cpp:33-65) of view img's image against view ref's
 * FP64 mean (rounded to float as the reference's float images are): which = 0 the
 * shaded frame, 1 the accumulator. Same resolution required. FP64 accumulation. */
int vxr_view_error(vxr_view* img, int which, vxr_view* ref, double* mse, double* mae);

/* ---- launch tuning ---------------------------------------------------------------------
 * No counterpart in the reference (its work-group size is fixed, template.cpp:1700-1754).
 * Parameters that change speed but never results: every setting renders the same bits.
 * The autotuner (smallproject_gb300/autotune.py) times them per configuration. */
typedef struct vxr_tuning {
    uint32_t tile_x, tile_y;       /* threads of a pixel-stage block; tile_x * tile_y a multiple of 32, <= 256 */
    uint32_t persistent;           /* pixel stages: 1 = resident blocks pull tiles from a queue, 0 = one block per tile */
    uint32_t shadow_refill;        /* shadow tracer: idle lanes of a warp (1..32) that trigger a refill from the queue */
    uint32_t shadow_burst;         /* shadow tracer: cell visits per lane between refill checks (1..64) */
    uint32_t list_blocks_per_sm;   /* hit-list kernels (candidates, temporal, shading requests): blocks per SM (1..64) */
    uint32_t occupancy;            /* 1: shadow tracer and candidate kernels capped in registers for more warps per SM */
    uint32_t shadow_schedule;      /* shadow tracer: 0 every lane steps each round, 1 only the lanes at the DDA level most lanes are at */
    uint32_t shadow_early_out;     /* shadow tracer: 1 stops a walk, as occluded, once its step budget cannot reach the emitter */
    uint32_t brick_cache;          /* shadow tracer: bricks whose opacity masks each CTA keeps in shared memory (0 off, 128..2048 a power of two) */
} vxr_tuning;
int vxr_default_tuning(vxr_tuning* t);
/* Current CUDA device: name (NUL-terminated, truncated to n bytes), SM count and compute
 * capability; the autotuner's cache key. */
int vxr_device_info(char* name, size_t n, int* sms, int* cc_major, int* cc_minor);
/* Replaces the view's launch parameters (including vxr_view_desc tile_x / tile_y). */
int vxr_view_set_tuning(vxr_view* v, const vxr_tuning* t);
int vxr_view_get_tuning(vxr_view* v, vxr_tuning* t);

/* ---- batches: several views rendered as one frame -------------------------------------
 * No counterpart in the reference: World::Render (world.cpp:2127-2340) draws one camera
 * per call, so several views are rendered one after another. A batch renders one frame of
 * up to VXR_BATCH_MAX_VIEWS views - each with its own world, resolution, light model and
 * parameters - with every stage as one launch over all of them: the pixel stages pull
 * (view, tile) work items from a device queue, and the candidate loop, the temporal step
 * and the shadow rays run over one list of every view's hit pixels. Each view's images,
 * G-buffers and reservoirs are bit-identical to rendering it alone with vxr_view_render.
 * Views must be on one device, hold at most 2^27 - 1 pixels each and not use a learned
 * proposal. tile_x * tile_y = threads of a pixel-stage block (0, 0 = 16 x 8), a multiple
 * of 32 up to 256. flags: VXR_BATCH_GRAPH records the frame once as a CUDA graph and
 * replays it: one graph launch per frame. VXR_BATCH_CHAINS(c), c in [1, min(n, 15)]:
 * the views are split into c groups of about equal pixel count, each group's stages one
 * launch over its views, on a branch stream of its own (parallel branches of the graph),
 * so that different groups can be in different stages at once. */
#define VXR_BATCH_MAX_VIEWS 16u
#define VXR_BATCH_GRAPH     1u
#define VXR_BATCH_CHAINS(c) (((uint32_t)(c) & 15u) << 8)
typedef struct vxr_batch vxr_batch;
int vxr_batch_create(vxr_view* const* views, uint32_t n, uint32_t tile_x, uint32_t tile_y, uint32_t flags,
                     vxr_batch** out);
int vxr_batch_destroy(vxr_batch* b);
/* One frame of every view: vxr_view_begin_frame, stages 1-4 with the accumulator fused
 * into shading, vxr_view_end_frame. Asynchronous; ordered after earlier work on each
 * view's stream and before later work on it (read results with the view calls). */
int vxr_batch_render(vxr_batch* b);
/* Wait for the batch's frames. ms (may be NULL): GPU time of the last frame. A device
 * error flag raised in any view -> VXR_E_DEVICE. */
int vxr_batch_wait(vxr_batch* b, float* ms);
/* Replaces the batch's launch parameters (tile shape included); recorded graphs are
 * re-recorded on the next frame. */
int vxr_batch_set_tuning(vxr_batch* b, const vxr_tuning* t);

/* ---- rendering without allocation ---------------------------------------------------
 * No counterpart in the reference. For callers that cannot call cudaMalloc - an
 * application that owns all GPU memory through its own pool, a plugin that must not
 * bypass its host's allocator - this renders ONE frame from device buffers the caller
 * already owns into a device image the caller owns, and allocates nothing: no
 * cudaMalloc, cudaFree or allocating library call. The G-buffer, seeds, reservoirs, the
 * hit list, the shadow-ray queue, the uber grid, the light table and the error word live in one fixed file-scope device
 * array of VXR_NOALLOC_SCRATCH_BYTES that every GPU loading libvxr.so holds until exit.
 *   grid      device uint32[128^3] top-level cells (layout of vxr_world_arrays)
 *   bricks    device uint32[nbricks * 512]; every brick cell must index below nbricks
 *             (checked on the device first; VXR_E_INVALID otherwise)
 *   lights    device vxr_light[nlights], nlights <= VXR_NOALLOC_MAX_LIGHTS
 *   k         host frame constants (e.g. from vxr_camera_begin_frame); width*height
 *             <= VXR_NOALLOC_MAX_PIXELS, numberOfLights == nlights; larger sizes are
 *             rejected with VXR_E_INVALID
 *   out_rgba  device float4[width*height]: shaded rgb and primary-hit distance
 *   stream    cudaStream_t to run on (NULL = the legacy default stream)
 * The frame is rendered without temporal reuse, accumulation or sky dome (no history is
 * kept between calls; skyDomeSampling 0). The call is synchronous. On its first call on a device it looks up
 * the device address of its scratch array (cudaGetSymbolAddress), so make that first
 * call before any stream capture on that device. All calls share the one scratch
 * array per device and it keeps the last call's contents: calls that overlap on the
 * GPU (different streams or threads at once) race and must be serialised by the
 * caller. */
#define VXR_NOALLOC_MAX_PIXELS    65536u     /* e.g. 256 x 256 */
#define VXR_NOALLOC_MAX_LIGHTS    65536u
#define VXR_NOALLOC_SCRATCH_BYTES 10518784u
int vxr_render_frame_noalloc(const uint32_t* grid, const uint32_t* bricks, uint32_t nbricks,
                             const vxr_light* lights, uint32_t nlights, uint32_t light_model,
                             const vxr_frame_consts* k, float* out_rgba, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* VXR_H */
