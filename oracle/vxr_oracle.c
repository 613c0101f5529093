/*
 * vxr_oracle.c - CPU restatement of the reference's per-frame Voxel ReSTIR path.
 *
 * TEST INFRASTRUCTURE ONLY (see vxr_oracle.h). Builds with -ffp-contract=off
 * -fno-fast-math: every float op is one IEEE binary32 rounding, in the order the
 * reference kernels (-cl-single-precision-constant) write it. Conventions where the
 * reference is undefined or implementation-defined:
 *   - normalize(v) = v * (1 / sqrt(dot(v, v)))      (reference host: precomp.h:283,656)
 *   - float -> integer conversions truncate and saturate, NaN -> 0 (GPU cvt.rzi)
 *   - uninitialised dist2/side2 after a shadow-ray miss read as 0 (ris.cl:74, 234)
 *   - a NaN reprojected screen coordinate is out of bounds (tools.cl:487)
 *   - cos/sin: orc_sincos below (OpenCL leaves the accuracy to the implementation)
 * Structure deliberately follows the reference: packed-coordinate DDA, full
 * six-face solid-angle evaluation, two reservoir buffers cycling through three roles.
 */
#include "vxr_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ---- scalar helpers ---------------------------------------------------------------- */
typedef struct { float x, y, z; } v3;
static inline v3 mk(float x, float y, float z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
static inline v3 vadd(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vmul(v3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
static inline v3 vsmul(float s, v3 a) { return mk(s * a.x, s * a.y, s * a.z); }
static inline v3 vmulv(v3 a, v3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline v3 vneg(v3 a) { return mk(-a.x, -a.y, -a.z); }
static inline float vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 vcross(v3 a, v3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static inline v3 vnorm(v3 v) { const float inv = 1.0f / sqrtf(vdot(v, v)); return vmul(v, inv); }
static inline float vlen(v3 v) { return sqrtf(vdot(v, v)); }
static inline v3 ld3(const float* p) { return mk(p[0], p[1], p[2]); }

static inline uint32_t f2u(float f) {
    if (!(f > 0.0f)) return 0u;
    if (f >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)f;
}
static inline int32_t f2i(float f) {
    if (f != f) return 0;
    if (f >= 2147483648.0f) return 2147483647;
    if (f <= -2147483648.0f) return (int32_t)0x80000000u;
    return (int32_t)f;
}
static inline uint32_t clampu(uint32_t v, uint32_t lo, uint32_t hi) { return v < lo ? lo : (v > hi ? hi : v); }
static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* tools.cl:17-19 */
static inline uint32_t wang_hash(uint32_t s) {
    s = (s ^ 61u) ^ (s >> 16);
    s *= 9u;
    s = s ^ (s >> 4);
    s *= 0x27d4eb2du;
    s = s ^ (s >> 15);
    return s;
}
static inline uint32_t rnd_int(uint32_t* s) {
    *s ^= *s << 13;
    *s ^= *s >> 17;
    *s ^= *s << 5;
    return *s;
}
static inline float rnd(uint32_t* s) { return (float)rnd_int(s) * 2.3283064365387e-10f; }

/* voxel payload, tools.cl:294-322 and common.h:203-211 */
static inline uint32_t alpha4(uint32_t v) { return (v & 0xf000u) >> 12; }
static inline float alphaf(uint32_t v) { return (float)alpha4(v) / (float)0xF; }
static inline v3 to_rgb(uint32_t v) {
    return mk((float)((v >> 8) & 15u) * (1.0f / 15.0f), (float)((v >> 4) & 15u) * (1.0f / 15.0f),
              (float)(v & 15u) * (1.0f / 15.0f));
}
static inline uint32_t from_rgba(v3 c, float a, uint32_t m) {
    return (m << 16) + (f2u(a * 15) << 12) + (f2u(c.x * 15) << 8) + (f2u(c.y * 15) << 4) + f2u(c.z * 15);
}
static inline float strength(uint32_t v) { return (float)((v & 0xff0000u) >> 16) * 1; }
static inline int is_emitter(uint32_t v) { return ((v >> 16) & 255u) > 0; }
/* tools.cl:416-421 (side is always 0..2 here) */
static inline v3 voxel_normal(uint32_t side, v3 D) {
    if (side == 0) return mk(D.x > 0 ? -1.0f : 1.0f, 0, 0);
    if (side == 1) return mk(0, D.y > 0 ? -1.0f : 1.0f, 0);
    return mk(0, 0, D.z > 0 ? -1.0f : 1.0f);
}

/* Cody-Waite reduction by pi/2 with the three-part constant of the Cephes library,
 * Taylor polynomials on [-pi/4, pi/4], every op a separate rounding. */
void orc_sincos(float a, float* s, float* c) {
    const float q = rintf(a * 0.636619772367581343f);
    const int qi = (int)q;
    const float r = ((a - q * 1.5703125f) - q * 4.83751296997070312e-4f) - q * 7.54978995489188216e-8f;
    const float r2 = r * r;
    const float ps = r + (r * r2) * (-1.0f / 6.0f + r2 * (1.0f / 120.0f + r2 * (-1.0f / 5040.0f + r2 * (1.0f / 362880.0f))));
    const float pc = 1.0f + r2 * (-0.5f + r2 * (1.0f / 24.0f + r2 * (-1.0f / 720.0f + r2 * (1.0f / 40320.0f + r2 * (-1.0f / 3628800.0f)))));
    switch (qi & 3) {
    case 0: *s = ps; *c = pc; break;
    case 1: *s = pc; *c = -ps; break;
    case 2: *s = -ps; *c = -pc; break;
    default: *s = -pc; *c = ps; break;
    }
}

/* ---- world ------------------------------------------------------------------------ */
typedef struct {
    const uint32_t* grid;
    const uint8_t* uber;
    const uint32_t* bricks;
} o_world;

/* kernels.cl:498-513 */
void orc_build_uber(const uint32_t* grid, uint8_t* uber) {
    for (int task = 0; task < 32 * 32 * 32; task++) {
        const int x = task & 31, z = (task / 32) & 31, y = (task / 1024) & 31;
        int empty = 1;
        for (int a = 0; a < 4; a++)
            for (int b = 0; b < 4; b++)
                for (int c = 0; c < 4; c++)
                    if (grid[(x * 4 + a) + (z * 4 + c) * 128 + (y * 4 + b) * 128 * 128]) empty = 0;
        uber[x + z * 32 + y * 1024] = empty ? 0 : 1;
    }
}

/* world.h:293-306 */
uint32_t orc_world_get(const uint32_t* grid, const uint32_t* bricks, uint32_t x, uint32_t y, uint32_t z) {
    const uint32_t bx = (x / 8) & 127, by = (y / 8) & 127, bz = (z / 8) & 127;
    const uint32_t g = grid[bx + bz * 128 + by * 128 * 128];
    if ((g & 1) == 0) return g >> 1;
    return bricks[(g >> 1) * 512 + (x & 7) + (y & 7) * 8 + (z & 7) * 64];
}

/* world.cpp:438-504 */
uint32_t orc_scan_lights(const uint32_t* grid, const uint32_t* bricks, vxr_light* out, uint32_t cap) {
    uint32_t n = 0;
    for (uint32_t by = 0; by < 128; by++)
        for (uint32_t bz = 0; bz < 128; bz++)
            for (uint32_t bx = 0; bx < 128; bx++) {
                const uint32_t g = grid[bx + bz * 128 + by * 128 * 128];
                if ((g & 1) == 0) {
                    if (strength(g >> 1) > 0) {
                        if (n < cap) {
                            out[n].position = bx * 8 + bz * 8 * 1024 + by * 8 * 1024 * 1024;
                            out[n].voxel = g >> 1;
                            out[n].size = 8;
                        }
                        n++;
                    }
                    continue;
                }
                for (uint32_t ly = 0; ly < 8; ly++)
                    for (uint32_t lz = 0; lz < 8; lz++)
                        for (uint32_t lx = 0; lx < 8; lx++) {
                            const uint32_t v = bricks[(g >> 1) * 512 + lx + ly * 8 + lz * 64];
                            if (strength(v) > 0) {
                                if (n < cap) {
                                    const uint32_t x = lx + bx * 8, y = ly + by * 8, z = lz + bz * 8;
                                    out[n].position = x + z * 1024 + y * 1024 * 1024;
                                    out[n].voxel = v;
                                    out[n].size = 1;
                                }
                                n++;
                            }
                        }
            }
    return n;
}

/* ---- restated World::Set store ------------------------------------------------------ */
struct orc_store {
    uint32_t* grid;
    uint32_t* bricks;
    uint32_t* zeroes;
    uint32_t nb, cap;
    uint32_t* trash;
    uint32_t ntrash, trashcap;
    vxr_light* lights;
    uint32_t nl, lcap;
};

orc_store* orc_store_create(void) {
    orc_store* s = (orc_store*)calloc(1, sizeof(orc_store));
    s->grid = (uint32_t*)calloc(128 * 128 * 128, sizeof(uint32_t));
    return s;
}
void orc_store_destroy(orc_store* s) {
    if (!s) return;
    free(s->grid); free(s->bricks); free(s->zeroes); free(s->trash); free(s->lights);
    free(s);
}
static uint32_t st_new_brick(orc_store* s) {
    if (s->ntrash) return s->trash[--s->ntrash];
    if (s->nb == s->cap) {
        s->cap = s->cap ? s->cap * 2 : 256;
        s->bricks = (uint32_t*)realloc(s->bricks, (size_t)s->cap * 512 * sizeof(uint32_t));
        s->zeroes = (uint32_t*)realloc(s->zeroes, (size_t)s->cap * sizeof(uint32_t));
    }
    return s->nb++;
}
static void st_free_brick(orc_store* s, uint32_t b) {
    if (s->ntrash == s->trashcap) {
        s->trashcap = s->trashcap ? s->trashcap * 2 : 256;
        s->trash = (uint32_t*)realloc(s->trash, s->trashcap * sizeof(uint32_t));
    }
    s->trash[s->ntrash++] = b;
}
static void st_remove_light(orc_store* s, uint32_t pos) {   /* world.cpp:506-561 */
    uint32_t j = 0;
    for (uint32_t i = 0; i < s->nl; i++)
        if (s->lights[i].position != pos) s->lights[j++] = s->lights[i];
    s->nl = j;
}
static void st_add_light(orc_store* s, uint32_t pos, uint32_t v) {   /* world.cpp:228-246 */
    if (s->nl == s->lcap) {
        s->lcap = s->lcap ? s->lcap * 2 : 64;
        s->lights = (vxr_light*)realloc(s->lights, s->lcap * sizeof(vxr_light));
    }
    s->lights[s->nl].position = pos;
    s->lights[s->nl].voxel = v;
    s->lights[s->nl].size = 1;
    s->nl++;
}
void orc_store_set(orc_store* s, uint32_t x, uint32_t y, uint32_t z, uint32_t v) {
    const uint32_t bx = x / 8, by = y / 8, bz = z / 8;
    if (bx >= 128 || by >= 128 || bz >= 128) return;
    const uint32_t ci = bx + bz * 128 + by * 128 * 128;
    uint32_t cell = s->grid[ci], b = cell >> 1;
    if ((cell & 1) == 0) {
        if (v == (cell >> 1)) return;
        const uint32_t colour = cell >> 1;
        b = st_new_brick(s);
        for (int i = 0; i < 512; i++) s->bricks[(size_t)b * 512 + i] = colour;
        s->zeroes[b] = (colour == 0) * 512;
        s->grid[ci] = (b << 1) | 1;
    }
    const size_t vi = (size_t)b * 512 + (x & 7) + (y & 7) * 8 + (z & 7) * 64;
    const uint32_t orig = s->bricks[vi];
    const uint32_t pos = x + z * 1024 + y * 1024 * 1024;
    if (is_emitter(orig)) st_remove_light(s, pos);
    if (is_emitter(v)) st_add_light(s, pos, v);
    const int change = (orig != 0 && v == 0) - (orig == 0 && v != 0);
    s->zeroes[b] = (uint32_t)((int)s->zeroes[b] + change);
    if (s->zeroes[b] < 512) s->bricks[vi] = v;
    else {
        s->grid[ci] = 0;
        st_free_brick(s, b);
    }
}
uint32_t orc_store_get(const orc_store* s, uint32_t x, uint32_t y, uint32_t z) {
    return orc_world_get(s->grid, s->bricks, x, y, z);
}
uint32_t orc_store_optimize(orc_store* s) {
    uint32_t replaced = 0;
    for (uint32_t i = 0; i < 128 * 128 * 128; i++) {
        const uint32_t c = s->grid[i];
        if (!(c & 1)) continue;
        const uint32_t* br = s->bricks + (size_t)(c >> 1) * 512;
        int solid = 1;
        for (int j = 1; j < 512 && solid; j++) solid = br[j] == br[0];
        if (solid) {
            s->grid[i] = br[0] << 1;
            st_free_brick(s, c >> 1);
            replaced++;
        }
    }
    return replaced;
}
uint32_t orc_store_lights(const orc_store* s, vxr_light* out, uint32_t cap) {
    for (uint32_t i = 0; i < s->nl && i < cap; i++) out[i] = s->lights[i];
    return s->nl;
}
const uint32_t* orc_store_grid(const orc_store* s) { return s->grid; }
const uint32_t* orc_store_bricks(const orc_store* s) { return s->bricks; }

/* ---- camera --------------------------------------------------------------------------- */
void orc_camera_init(orc_camera* c, uint32_t rng_seed) {
    memset(c, 0, sizeof(*c));
    for (int i = 0; i < 16; i++) c->M[i] = (i % 5 == 0) ? 1.0f : 0.0f;
    c->first = 1;
    c->rng = rng_seed;
}
/* mat4::LookAt (precomp.h:825-835) */
void orc_lookat(orc_camera* c, const float pos[3], const float target[3]) {
    const v3 P = ld3(pos), T = ld3(target);
    const v3 z = vnorm(vsub(T, P));
    const v3 x = vnorm(vcross(z, mk(0, 1, 0)));
    const v3 y = vcross(x, z);
    for (int i = 0; i < 16; i++) c->M[i] = (i % 5 == 0) ? 1.0f : 0.0f;
    c->M[3] = P.x; c->M[7] = P.y; c->M[11] = P.z;
    c->M[0] = x.x; c->M[4] = x.y; c->M[8] = x.z;
    c->M[1] = y.x; c->M[5] = y.y; c->M[9] = y.z;
    c->M[2] = z.x; c->M[6] = z.y; c->M[10] = z.z;
}
/* TransformPosition (template.cpp:1045-1062) */
static v3 xform(const float* m, v3 a) {
    return mk(m[0] * a.x + m[1] * a.y + m[2] * a.z + m[3] * 1.0f, m[4] * a.x + m[5] * a.y + m[6] * a.z + m[7] * 1.0f,
              m[8] * a.x + m[9] * a.y + m[10] * a.z + m[11] * 1.0f);
}
static void put_plane(float* out, v3 n, v3 E) { out[0] = n.x; out[1] = n.y; out[2] = n.z; out[3] = vdot(E, n); }
static void st3(float* p, v3 v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }
/* World::Render host part (world.cpp:2144-2191) */
void orc_begin_frame(orc_camera* c, uint32_t W, uint32_t H, vxr_frame_consts* k) {
    v3 prevE = ld3(c->E), prevP0 = ld3(c->p0), prevP1 = ld3(c->p1), prevP2 = ld3(c->p2);
    const v3 prevP3 = vadd(prevP1, vsub(prevP2, prevP0));
    const float aspect = (float)W / H;
    const v3 E = xform(c->M, mk(0, 0, 0));
    const v3 p0 = xform(c->M, mk(aspect, 1, 2.2f));
    const v3 p1 = xform(c->M, mk(-aspect, 1, 2.2f));
    const v3 p2 = xform(c->M, mk(aspect, -1, 2.2f));
    if (c->first) { prevE = E; prevP0 = p0; prevP1 = p1; prevP2 = p2; c->first = 0; }
    st3(c->E, E); st3(c->p0, p0); st3(c->p1, p1); st3(c->p2, p2);
    memset(k, 0, sizeof(*k));
    st3(k->E, E); st3(k->p0, p0); st3(k->p1, p1); st3(k->p2, p2);
    k->oneOverRes[0] = 1.0f / W;
    k->oneOverRes[1] = 1.0f / H;
    put_plane(k->Nleft, vnorm(vcross(vsub(prevP0, prevE), vsub(prevP2, prevE))), prevE);
    put_plane(k->Nright, vnorm(vcross(vsub(prevP3, prevE), vsub(prevP1, prevE))), prevE);
    put_plane(k->Ntop, vnorm(vcross(vsub(prevP0, prevE), vsub(prevP1, prevE))), prevE);
    put_plane(k->Nbottom, vnorm(vcross(vsub(prevP3, prevE), vsub(prevP2, prevE))), prevE);
    k->R0 = rnd_int(&c->rng);
    k->frame = c->frame;
    k->framecount = c->framecount;
    k->restirtemporalframe = c->restirtemporalframe;
    k->width = W;
    k->height = H;
}
void orc_end_frame(orc_camera* c) {
    c->frame = (c->frame + 1) & 255;
    c->framecount++;
    c->restirtemporalframe++;
}

/* ---- brick-grid DDA (trace.cl:121-362) ---------------------------------------------- */
#define TOPMASK3 ((1016u << 20) + (1016u << 10) + 1016u)
#define UBERMASK3 ((1020u << 20) + (1020u << 10) + 1020u)

static inline int dda_hit(int mode, uint32_t v, uint32_t through, uint32_t mask) {
    if (mode == 0) return v != 0;                               /* TraceRay: v != 0 */
    if (mode == 1) return alpha4(v) == 0xF;                     /* TraceOpaqueRay */
    return (v & mask) != (through & mask);                      /* TraceThrough */
}

static uint32_t o_trace(const o_world* w, int mode, v3 A, v3 B, int steps, uint32_t through, uint32_t mask,
                        float* dist, uint32_t* side) {
    v3 V = B;                                                    /* FixZeroDeltas, trace.cl:37-43 */
    if (fabsf(V.x) < 1e-8f) V.x = V.x < 0 ? -1e-8f : 1e-8f;
    if (fabsf(V.y) < 1e-8f) V.y = V.y < 0 ? -1e-8f : 1e-8f;
    if (fabsf(V.z) < 1e-8f) V.z = V.z < 0 ? -1e-8f : 1e-8f;
    const v3 rV = mk(1.0f / V.x, 1.0f / V.y, 1.0f / V.z);
    float to = 0;
    const int bits = (V.x > 0 ? 34 : 4) + (V.y > 0 ? 10752 : 3072) + (V.z > 0 ? 3276800 : 1310720);
    const uint32_t OX = (bits >> 5) & 1, OY = (bits >> 13) & 1, OZ = (uint32_t)bits >> 21;
    const int DX = (bits & 3) - 1, DY = ((bits >> 8) & 3) - 1, DZ = ((bits >> 16) & 3) - 1;
    const uint32_t dx = (uint32_t)DX << 20, dy = (uint32_t)DY << 10, dz = (uint32_t)DZ;
    uint32_t last = 0;
    if (A.x < 0 || A.y < 0 || A.z < 0 || A.x > 1024.0f || A.y > 1024.0f || A.z > 1024.0f) {
        const float tx1 = -A.x * rV.x, tx2 = (1024.0f - A.x) * rV.x;
        float tmin = fminf(tx1, tx2), tmax = fmaxf(tx1, tx2);
        const float ty1 = -A.y * rV.y, ty2 = (1024.0f - A.y) * rV.y;
        tmin = fmaxf(tmin, fminf(ty1, ty2)), tmax = fminf(tmax, fmaxf(ty1, ty2));
        const float tz1 = -A.z * rV.z, tz2 = (1024.0f - A.z) * rV.z;
        tmin = fmaxf(tmin, fminf(tz1, tz2)), tmax = fminf(tmax, fmaxf(tz1, tz2));
        if (tmax < tmin || tmax <= 0) return 0;
        A = mk(A.x + tmin * V.x, A.y + tmin * V.y, A.z + tmin * V.z);
        to = tmin;
        if (A.y < 0.01f || A.y > (1024.0f - 1.01f)) last = 1;
        if (A.z < 0.01f || A.z > (1024.0f - 1.01f)) last = 2;
    }
    uint32_t up = (clampu(f2u(A.x) >> 5, 0, 31) << 20) + (clampu(f2u(A.y) >> 5, 0, 31) << 10) + clampu(f2u(A.z) >> 5, 0, 31);
    float tmx = ((float)((up >> 20) + OX) - A.x * 0.03125f) * rV.x;
    float tmy = ((float)(((up >> 10) & 31) + OY) - A.y * 0.03125f) * rV.y;
    float tmz = ((float)((up & 31) + OZ) - A.z * 0.03125f) * rV.z;
    float t = 0;
    const float tdx = (float)DX * rV.x, tdy = (float)DY * rV.y, tdz = (float)DZ * rV.z;
    uint32_t o = w->uber[(up >> 20) + ((up & 31) << 5) + (((up >> 10) & 31) << 10)];
    for (;;) {
        if ((steps -= 4) <= 0) break;
        if (mode == 2 ? (o != 0 || through != 0) : (o != 0)) {
            const float ux_ = tmx, uy_ = tmy, uz_ = tmz;
            t *= 4;
            const uint32_t qx = f2u(0.125f * A.x + V.x * t), qy = f2u(0.125f * A.y + V.y * t), qz = f2u(0.125f * A.z + V.z * t);
            uint32_t tp = (clampu(qx, up >> 18, (up >> 18) + 3) << 20) +
                          (clampu(qy, (up >> 8) & 1023, ((up >> 8) & 1023) + 3) << 10) +
                          clampu(qz, (up << 2) & 1023, ((up << 2) & 1023) + 3);
            const uint32_t tq = tp & UBERMASK3;
            tmx = ((float)((tp >> 20) + OX) - A.x * 0.125f) * rV.x;
            tmy = ((float)(((tp >> 10) & 127) + OY) - A.y * 0.125f) * rV.y;
            tmz = ((float)((tp & 127) + OZ) - A.z * 0.125f) * rV.z;
            o = w->grid[(tp >> 20) + (tp & 127) * 128 + ((tp >> 10) & 127) * 16384];
            for (;;) {
                if (!--steps) break;
                const uint32_t v = o >> 1;
                if ((dda_hit(mode, v, through, mask) && (o & 1) == 0) || (o & 1) == 1) {
                    if ((o & 1) == 0) {
                        *dist = t * 8.0f + to;
                        *side = last;
                        return v;
                    }
                    const float gx_ = tmx, gy_ = tmy, gz_ = tmz;
                    t *= 8;
                    const uint32_t px = f2u(A.x + V.x * t), py = f2u(A.y + V.y * t), pz = f2u(A.z + V.z * t);
                    uint32_t p = (clampu(px, tp >> 17, (tp >> 17) + 7) << 20) +
                                 (clampu(py, (tp >> 7) & 1023, ((tp >> 7) & 1023) + 7) << 10) +
                                 clampu(pz, (tp << 3) & 1023, ((tp << 3) & 1023) + 7);
                    tmx = ((float)((p >> 20) + OX) - A.x) * rV.x;
                    tmy = ((float)(((p >> 10) & 1023) + OY) - A.y) * rV.y;
                    tmz = ((float)((p & 1023) + OZ) - A.z) * rV.z;
                    p &= 7 + (7 << 10) + (7 << 20);
                    const uint32_t base = (o - 1) << 8;               /* o = --o << 8 */
                    for (int i = 0; i < 24; i++) {                    /* 24 x BRICKSTEP */
                        const uint32_t bv = w->bricks[base + (p >> 20) + ((p >> 7) & 56) + (p & 7) * 64];
                        if (dda_hit(mode, bv, through, mask)) {
                            *dist = t + to;
                            *side = last;
                            return bv;
                        }
                        t = fminf(tmx, fminf(tmy, tmz)), last = 0;
                        if (t == tmx) tmx += tdx, p += dx;
                        if (t == tmy) tmy += tdy, p += dy, last = 1;
                        if (t == tmz) tmz += tdz, p += dz, last = 2;
                        if (p & TOPMASK3) break;
                    }
                    tmx = gx_, tmy = gy_, tmz = gz_;
                }
                t = fminf(tmx, fminf(tmy, tmz)), last = 0;
                if (t == tmx) tmx += tdx, tp += dx;
                if (t == tmy) tmy += tdy, tp += dy, last = 1;
                if (t == tmz) tmz += tdz, tp += dz, last = 2;
                if ((tp & UBERMASK3) - tq) break;
                o = w->grid[(tp >> 20) + (tp & 127) * 128 + ((tp >> 10) & 127) * 16384];
            }
            tmx = ux_, tmy = uy_, tmz = uz_;
        }
        t = fminf(tmx, fminf(tmy, tmz)), last = 0;
        if (t == tmx) tmx += tdx, up += dx;
        if (t == tmy) tmy += tdy, up += dy, last = 1;
        if (t == tmz) tmz += tdz, up += dz, last = 2;
        if (up & 0xfe0f83e0u) break;
        o = w->uber[(up >> 20) + ((up & 31) << 5) + (((up >> 10) & 31) << 10)];
    }
    return 0;
}

/* ---- render path ----------------------------------------------------------------------- */
typedef struct {
    uint32_t voxel;
    float dist;
    uint32_t side;
    uint32_t seed;
    v3 dir;
} o_ray;
typedef struct {
    float sumW;
    uint32_t M;
    uint32_t idx;
    float W;
    v3 pos;
    float inv;
    v3 nl;
    float pHat;
} o_res;

struct orc_ctx {
    int W, H, point;
    o_world w;
    vxr_light* lights;
    uint32_t nl;
    o_ray* gb[2];
    o_res* res[2];
    float* frame;   /* float4 */
    float* accum;   /* float4 */
    int resOut, resIn, gbCur, gbPrev;
    int candOut, candIn, spatOut, spatIn, shadeOut, shadeIn;
    /* explicit candidates (the learned proposal's draws), or null: candidate m of pixel i
     * is light candIdx[m * candStride + i] with source pdf candP[...] */
    const uint32_t* candIdx;
    const float* candP;
    size_t candStride;
};

void orc_set_candidates(orc_ctx* c, const uint32_t* idx, const float* p, size_t stride) {
    c->candIdx = idx;
    c->candP = p;
    c->candStride = stride;
}

orc_ctx* orc_create(int W, int H, int point_lights) {
    orc_ctx* c = (orc_ctx*)calloc(1, sizeof(orc_ctx));
    const size_t n = (size_t)W * H;
    c->W = W; c->H = H; c->point = point_lights;
    for (int i = 0; i < 2; i++) {
        c->gb[i] = (o_ray*)calloc(n, sizeof(o_ray));
        c->res[i] = (o_res*)calloc(n, sizeof(o_res));
    }
    c->frame = (float*)calloc(n * 4, sizeof(float));
    c->accum = (float*)calloc(n * 4, sizeof(float));
    c->resOut = 0; c->resIn = 1; c->gbCur = 0; c->gbPrev = 1;
    return c;
}
void orc_destroy(orc_ctx* c) {
    if (!c) return;
    for (int i = 0; i < 2; i++) { free(c->gb[i]); free(c->res[i]); }
    free(c->frame); free(c->accum); free(c->lights);
    free(c);
}
void orc_set_world(orc_ctx* c, const uint32_t* grid, const uint8_t* uber, const uint32_t* bricks) {
    c->w.grid = grid; c->w.uber = uber; c->w.bricks = bricks;
}
void orc_set_lights(orc_ctx* c, const vxr_light* l, uint32_t n) {
    free(c->lights);
    c->lights = (vxr_light*)malloc((n ? n : 1) * sizeof(vxr_light));
    if (n) memcpy(c->lights, l, n * sizeof(vxr_light));
    else { c->lights[0].position = 0; c->lights[0].voxel = 0; c->lights[0].size = 1; }
    c->nl = n;
}
static inline void swapi(int* a, int* b) { int t = *a; *a = *b; *b = t; }
/* world.cpp:2209-2223 */
void orc_frame_start(orc_ctx* c) {
    c->candOut = c->resOut; c->candIn = c->resIn; swapi(&c->resOut, &c->resIn);
    c->spatOut = c->resOut; c->spatIn = c->resIn; swapi(&c->resOut, &c->resIn);
    c->shadeOut = c->resOut; c->shadeIn = c->resIn; swapi(&c->resOut, &c->resIn);
    swapi(&c->gbCur, &c->gbPrev);
}

/* GenerateCameraRay (tools.cl:102-127) */
static v3 camera_ray(const vxr_frame_consts* k, int x, int y) {
    const float u = (float)x * k->oneOverRes[0], v = (float)y * k->oneOverRes[1];
    const v3 p0 = ld3(k->p0), p1 = ld3(k->p1), p2 = ld3(k->p2);
    const v3 P = vadd(vadd(p0, vmul(vsub(p1, p0), u)), vmul(vsub(p2, p0), v));
    return vnorm(vsub(P, ld3(k->E)));
}

/* reservoir.cl:3-42 */
static void res_update(o_res* r, float w, float pHat, uint32_t idx, float r0, v3 pos, float inv, v3 nl) {
    r->M += 1;
    r->sumW += w;
    if (r0 < w / fmaxf(10e-6f, r->sumW)) {
        r->idx = idx; r->pos = pos; r->inv = inv; r->nl = nl; r->pHat = pHat;
    }
}
static void res_reweigh(o_res* r, float newPHat, uint32_t M) {
    r->sumW = r->W * M * newPHat;
    r->M = M;
    r->pHat = newPHat;
}
static void res_combine(o_res* r, const o_res* o, float r0) {
    const uint32_t m1 = r->M, m2 = o->M;
    res_update(r, o->sumW, o->pHat, o->idx, r0, o->pos, o->inv, o->nl);
    r->M = m1 + m2;
}
static void res_adjust(o_res* r, float pHat) { r->W = r->sumW / fmaxf(10e-6f, pHat * r->M); }

/* phat.cl:2-41 */
static v3 phat_full(const orc_ctx* c, v3 pl, v3 nl, v3 sp, v3 N, v3 brdf, uint32_t lvox, uint32_t lsize) {
    const float size = (float)lsize;
    v3 em = vmul(to_rgb(lvox), strength(lvox));
    em = vmul(em, 0.31830988618379067153777f);
    const v3 R = vsub(pl, sp);
    const v3 L = vnorm(R);
    const float ndotl = fmaxf(vdot(N, L), 0.0f);
    const float dsq = fmaxf(10e-6f, vdot(R, R));
    const float area = size * size;
    const float nldotl = c->point ? 1.0f : fmaxf(vdot(nl, vneg(L)), 0.0f);
    const float solid = (nldotl * area) / dsq;
    return vmul(vmul(vmulv(brdf, em), ndotl), solid);
}
static float phat(const orc_ctx* c, v3 pl, v3 nl, v3 sp, v3 N, v3 brdf, uint32_t lvox, uint32_t lsize) {
    const float r = vlen(phat_full(c, pl, nl, sp, N, brdf, lvox, lsize));
    if (isnan(r) || isinf(r)) return 0.0f;
    return r;
}

static const float NORMALS[6][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {-1, 0, 0}, {0, -1, 0}, {0, 0, -1}};
static const int TIDX[6] = {1, 2, 0, 4, 5, 3};
static const int BIDX[6] = {2, 0, 1, 5, 3, 4};

/* RandomPointOnVoxel (tools.cl:499-577) */
static v3 random_point_on_voxel(v3 center, v3 sp, int isize, uint32_t* seed, float* invp, v3* nlight) {
    const float size = (float)isize;
    float sa[6];
    v3 pts[6];
    float total = 0;
    for (int i = 0; i < 6; i++) {
        const v3 N = ld3(NORMALS[i]), T = ld3(NORMALS[TIDX[i]]), B = ld3(NORMALS[BIDX[i]]);
        const float r0 = rnd(seed), r1 = rnd(seed);
        v3 p = vadd(center, vmul(N, 0.5f * size));
        p = vsub(p, vmul(T, 0.5f * size));
        p = vsub(p, vmul(B, 0.5f * size));
        p = vadd(p, vmul(T, r0 * size));
        p = vadd(p, vmul(B, r1 * size));
        const v3 R = vsub(p, sp);
        const v3 L = vnorm(R);
        const float dsq = fmaxf(10e-6f, vdot(R, R));
        const float nl = vdot(N, vneg(L));
        const float area = size * size;
        const float s = nl * area / dsq;
        pts[i] = p;
        sa[i] = fmaxf(0.0f, s);
        total += fmaxf(0.0f, s);
    }
    float pdf[6], cdf[6];
    const float r2 = rnd(seed);
    int index = 0;
    pdf[0] = sa[0] / total;
    cdf[0] = pdf[0];
    if (cdf[0] < r2) {
        for (int i = 1; i < 6; i++) {
            pdf[i] = sa[i] / total;
            cdf[i] = cdf[i - 1] + pdf[i];
            index = i;
            if (cdf[i] >= r2) break;
        }
    }
    float wgt = 1.0f / pdf[index];
    if (isinf(wgt) || isnan(wgt)) wgt = 0.0f;
    *invp = wgt;
    *nlight = ld3(NORMALS[index]);
    return pts[index];
}

/* indexToCoordinates (tools.cl:428-434) */
static void light_coords(uint32_t p, uint32_t* x, uint32_t* y, uint32_t* z) {
    *y = p / (1024u * 1024u);
    *z = (p / 1024u) % 1024u;
    *x = p % 1024u;
}

/* isLightOccluded (ris.cl:1-17) with GridCoordinatesFromHit / Uint3CubeEquals
 * (tools.cl:452-472) */
static int occluded(const orc_ctx* c, const vxr_light* l, v3 o, v3 L) {
    uint32_t ex, ey, ez;
    light_coords(l->position, &ex, &ey, &ez);
    float d2 = 0.0f;
    uint32_t s2 = 0;
    o_trace(&c->w, 1, o, L, 128, 0, 0, &d2, &s2);
    const v3 N = voxel_normal(s2, L);
    const v3 hp = vadd(vmul(L, d2), o);
    const v3 q = vsub(hp, vmul(N, 0.1f));
    const uint32_t hx = f2u(q.x), hy = f2u(q.y), hz = f2u(q.z);
    const uint32_t sz = l->size;
    const int inside = ex <= hx && ex + sz > hx && ey <= hy && ey + sz > hy && ez <= hz && ez + sz > hz;
    return !inside;
}

/* renderAlbedo (ris.cl:295-389) */
static void px_albedo(orc_ctx* c, const vxr_frame_consts* k, int x, int y) {
    const uint32_t seed = wang_hash((uint32_t)(x * 171 + y * 1773) + k->R0);
    const v3 D = camera_ray(k, x, y);
    const v3 E = ld3(k->E);
    uint32_t side = 0;
    float dist = 0;
    uint32_t voxel = o_trace(&c->w, 0, E, D, 999999, 0, 0, &dist, &side);
    float alpha = alphaf(voxel);
    v3 outc = vmul(to_rgb(voxel), alpha);
    float total = 0.0f;
    int iter = 0;
    float remvis = 1.0f - alphaf(voxel);
    uint32_t prevSide = 0, prevHit = 0;
    while (prevHit != voxel && remvis > 0.0f) {
        prevHit = voxel;
        prevSide = side;
        total += dist + 0.01f;
        const v3 o = vadd(E, vsmul(total, D));
        voxel = o_trace(&c->w, 2, o, D, 999999, voxel, 0x00FFFF, &dist, &side);
        const v3 col = to_rgb(voxel);
        alpha = alphaf(voxel);
        outc = vadd(outc, vmul(vsmul(remvis, col), alpha));
        remvis = remvis * (1 - alpha);
        if (++iter == 25) remvis = 0.0f;
        if (dist <= 0.001f) break;
    }
    if (voxel != 0) total += dist;
    else side = prevSide;
    voxel = from_rgba(outc, 1.0f - remvis, (uint32_t)strength(voxel));
    o_ray* r = &c->gb[c->gbCur][(size_t)y * c->W + x];
    r->voxel = voxel;
    r->side = side;
    r->seed = seed;
    r->dist = total;
    r->dir = D;
}

/* perPixelInitialSampling (ris.cl:20-124) */
static void px_candidates(orc_ctx* c, const vxr_frame_consts* k, int x, int y) {
    o_ray* ray = &c->gb[c->gbCur][(size_t)y * c->W + x];
    const o_ray* prevAlbedo = c->gb[c->gbPrev];
    const o_res* prevRes = c->res[c->candIn];
    const float dist = ray->dist;
    const uint32_t voxel = ray->voxel;
    o_res res;
    memset(&res, 0, sizeof(res));
    if (voxel != 0) {
        uint32_t* seed = &ray->seed;
        const v3 D = ray->dir;
        const uint32_t side = ray->side;
        const v3 N = voxel_normal(side, D);
        const v3 brdf = vmul(to_rgb(voxel), 0.31830988618379067153777f);
        const v3 sp = vadd(vmul(D, dist), ld3(k->E));
        const v3 spo = vadd(sp, vsmul(0.1f, N));
        const uint32_t nL = k->numberOfLights;
        const uint32_t K = nL < k->numberOfCandidates ? nL : k->numberOfCandidates;
        const size_t pi = (size_t)y * c->W + x;
        for (uint32_t i = 0; i < K; i++) {
            /* GenerateLightCandidate (tools.cl:593-598): uniform index, p = 1/N; or the
             * candidate and pdf a caller-supplied source drew (no draw from the pixel seed) */
            uint32_t li;
            float p;
            if (c->candIdx) {
                li = c->candIdx[i * c->candStride + pi];
                p = c->candP[i * c->candStride + pi];
            } else {
                li = (uint32_t)clampi(f2i(rnd(seed) * (int)nL), 0, (int)nL - 1);
                p = 1.0f / nL;
            }
            const vxr_light* L = &c->lights[li];
            uint32_t ex, ey, ez;
            light_coords(L->position, &ex, &ey, &ez);
            const v3 center = vadd(mk((float)ex, (float)ey, (float)ez), vsmul(0.5f, mk((float)(int)L->size, (float)(int)L->size, (float)(int)L->size)));
            v3 pos, nl;
            float inv;
            if (c->point) {
                inv = 1;
                pos = center;
                nl = mk(0, 0, 0);
            } else {
                pos = random_point_on_voxel(center, spo, (int)L->size, seed, &inv, &nl);
            }
            const float ph = phat(c, pos, nl, sp, N, brdf, L->voxel, L->size) * inv;
            res_update(&res, ph / p, ph, li, rnd(seed), pos, inv, nl);
        }
        res_adjust(&res, res.pHat);
        {
            const vxr_light light = c->lights[res.idx];
            const v3 R = vsub(res.pos, spo);
            const v3 L = vnorm(R);
            if (occluded(c, &light, spo, L)) {
                res.W = 0;
                res.sumW = 0;
            }
        }
        if (k->restirtemporalframe > 0 && k->temporal) {
            const float dl = vdot(sp, ld3(k->Nleft)) - k->Nleft[3];
            const float dr = vdot(sp, ld3(k->Nright)) - k->Nright[3];
            const float dt = vdot(sp, ld3(k->Ntop)) - k->Ntop[3];
            const float db = vdot(sp, ld3(k->Nbottom)) - k->Nbottom[3];
            const float up = (float)c->W * (dl / (dl + dr));
            const float vp = (float)c->H * (dt / (dt + db));
            const float ru = roundf(up), rv = roundf(vp);
            if (ru == ru && rv == rv) {
                const int px = f2i(ru), py = f2i(rv);
                if (px >= 0 && py >= 0 && px < c->W && py < c->H) {
                    const o_ray* pr = &prevAlbedo[(size_t)py * c->W + px];
                    if (pr->side == side && fabsf(dist - pr->dist) <= 0.1f * dist) {
                        o_res prev = prevRes[(size_t)py * c->W + px];
                        const uint32_t pm = k->numberOfMaxTemporalImportance * K < prev.M ? k->numberOfMaxTemporalImportance * K : prev.M;
                        if (pm > 0) {
                            const vxr_light* pl = &c->lights[prev.idx < c->nl ? prev.idx : 0];
                            const float pph = phat(c, prev.pos, prev.nl, sp, N, brdf, pl->voxel, pl->size) * prev.inv;
                            res_reweigh(&prev, pph, pm);
                            res_combine(&res, &prev, rnd(seed));
                            const vxr_light* sl = &c->lights[res.idx < c->nl ? res.idx : 0];
                            const float sph = phat(c, res.pos, res.nl, sp, N, brdf, sl->voxel, sl->size) * res.inv;
                            res_adjust(&res, sph);
                        }
                    }
                }
            }
        }
    }
    c->res[c->candOut][(size_t)y * c->W + x] = res;
}

/* perPixelSpatialResampling (ris.cl:126-151) + _perPixelSpatialResampling (spatialSampling.cl:2-66) */
static void px_spatial(orc_ctx* c, const vxr_frame_consts* k, int x, int y) {
    const o_res* in = c->res[c->spatIn];
    o_res res = in[(size_t)y * c->W + x];
    o_ray* ray = &c->gb[c->gbCur][(size_t)y * c->W + x];
    if (ray->voxel != 0 && k->spatial) {
        uint32_t* seed = &ray->seed;
        const float dist = ray->dist;
        const v3 D = ray->dir;
        const uint32_t side = ray->side;
        const v3 N = voxel_normal(side, D);
        const v3 brdf = vmul(to_rgb(ray->voxel), 0.31830988618379067153777f);
        const v3 sp = vadd(vmul(D, dist), ld3(k->E));
        for (uint32_t i = 0; i < k->spatialTaps; i++) {
            const float angle = rnd(seed) * 6.28318530717958647692528f;
            const float radius = (float)(k->spatialRadius - 1) * sqrtf(rnd(seed)) + 1.0f;
            float sn, cs;
            orc_sincos(angle, &sn, &cs);
            const int nx = (int)((uint32_t)x + (uint32_t)f2i(cs * radius));
            const int ny = (int)((uint32_t)y + (uint32_t)f2i(sn * radius));
            if ((nx == x && ny == y) || nx < 0 || ny < 0 || nx >= c->W || ny >= c->H) continue;
            const size_t ni = (size_t)ny * c->W + nx;
            o_res nb = in[ni];
            if (nb.M > 0) {
                const o_ray* nr = &c->gb[c->gbCur][ni];
                if (nr->side == side && fabsf(dist - nr->dist) <= 0.1f * dist) {
                    const vxr_light* nl = &c->lights[nb.idx < c->nl ? nb.idx : 0];
                    const float ph = phat(c, nb.pos, nb.nl, sp, N, brdf, nl->voxel, nl->size) * nb.inv;
                    res_reweigh(&nb, ph, nb.M);
                    res_combine(&res, &nb, rnd(seed));
                }
            }
        }
        res_adjust(&res, res.pHat);
    }
    c->res[c->spatOut][(size_t)y * c->W + x] = res;
}

/* renderRIS (ris.cl:391-413) + render_di_ris (ris.cl:155-293), sky and editor off */
static void px_shade(orc_ctx* c, const vxr_frame_consts* k, int x, int y) {
    const size_t i = (size_t)y * c->W + x;
    const o_ray* hit = &c->gb[c->gbCur][i];
    o_res* prev = c->res[c->shadeIn];
    o_res res = prev[i];
    const float dist = hit->dist;
    const v3 D = hit->dir;
    const v3 N = voxel_normal(hit->side, D);
    const uint32_t voxel = hit->voxel;
    v3 color = mk(0, 0, 0);
    if (voxel != 0) {
        const v3 sky = mk(0, 0, 0);
        if (is_emitter(voxel)) {
            v3 ec = vmul(to_rgb(voxel), strength(voxel));
            ec = vmul(ec, 0.31830988618379067153777f);
            color = vadd(color, ec);
        }
        if (res.W > 0 && res.M > 0) {
            const v3 sp = vadd(vmul(D, dist), ld3(k->E));
            const v3 spo = vadd(sp, vsmul(0.1f, N));
            const vxr_light light = c->lights[res.idx < c->nl ? res.idx : 0];
            const v3 L = vnorm(vsub(res.pos, spo));
            if (!occluded(c, &light, spo, L)) {
                const v3 brdf = vmul(to_rgb(voxel), 0.31830988618379067153777f);
                const v3 inc0 = phat_full(c, res.pos, res.nl, sp, N, brdf, light.voxel, light.size);
                color = vadd(color, vmul(vmul(inc0, res.W), res.inv));
            } else {
                res.W = 0;
                res.sumW = 0;
                prev[i] = res;
            }
        }
        const float a = alphaf(voxel);
        color = vadd(color, vadd(vsmul(a, color), vsmul(1 - a, sky)));
    }
    float* f = c->frame + 4 * i;
    f[0] = color.x; f[1] = color.y; f[2] = color.z; f[3] = dist;
    c->res[c->shadeOut][i] = prev[i];
}

/* accumulatorFinalizer (kernels.cl:304-326) */
static void px_accumulate(orc_ctx* c, const vxr_frame_consts* k, int x, int y) {
    const size_t i = (size_t)y * c->W + x;
    const float* f = c->frame + 4 * i;
    float* a = c->accum + 4 * i;
    const int n = (int)(k->framecount * (uint32_t)k->accumulate);
    float pr[3] = {0, 0, 0};
    if (n > 0) { pr[0] = a[0]; pr[1] = a[1]; pr[2] = a[2]; }
    const float w = 1.0f / (1 + n);
    for (int j = 0; j < 3; j++) a[j] = (1 - w) * pr[j] + w * f[j];
    a[3] = 1.0f;
}

void orc_stage(orc_ctx* c, const vxr_frame_consts* k, int stage, int y0, int y1) {
    if (y1 <= 0 || y1 > c->H) y1 = c->H;
    if (y0 < 0) y0 = 0;
    int y;
#pragma omp parallel for schedule(dynamic, 1)
    for (y = y0; y < y1; y++)
        for (int x = 0; x < c->W; x++) {
            switch (stage) {
            case 1: px_albedo(c, k, x, y); break;
            case 2: px_candidates(c, k, x, y); break;
            case 3: px_spatial(c, k, x, y); break;
            case 4: px_shade(c, k, x, y); break;
            case 5: px_accumulate(c, k, x, y); break;
            default: break;
            }
        }
}

void orc_read_gbuffer(const orc_ctx* c, int which, vxr_gbuffer_rec* out) {
    const o_ray* g = c->gb[which == 0 ? c->gbCur : c->gbPrev];
    for (size_t i = 0; i < (size_t)c->W * c->H; i++) {
        out[i].voxel = g[i].voxel; out[i].dist = g[i].dist; out[i].side = g[i].side; out[i].seed = g[i].seed;
    }
}
void orc_write_gbuffer(orc_ctx* c, int which, const vxr_gbuffer_rec* in, const vxr_frame_consts* k) {
    o_ray* g = c->gb[which == 0 ? c->gbCur : c->gbPrev];
    for (int y = 0; y < c->H; y++)
        for (int x = 0; x < c->W; x++) {
            const size_t i = (size_t)y * c->W + x;
            g[i].voxel = in[i].voxel; g[i].dist = in[i].dist; g[i].side = in[i].side; g[i].seed = in[i].seed;
            g[i].dir = camera_ray(k, x, y);
        }
}
static int role_index(const orc_ctx* c, int role) { return role == 0 ? c->candOut : (role == 1 ? c->spatOut : c->shadeOut); }
void orc_read_reservoirs(const orc_ctx* c, int role, vxr_reservoir_rec* out) {
    const o_res* r = c->res[role_index(c, role)];
    for (size_t i = 0; i < (size_t)c->W * c->H; i++) {
        out[i].sumOfWeights = r[i].sumW; out[i].streamLength = r[i].M; out[i].lightIndex = r[i].idx;
        out[i].adjustedWeight = r[i].W;
        out[i].positionOnVoxel[0] = r[i].pos.x; out[i].positionOnVoxel[1] = r[i].pos.y; out[i].positionOnVoxel[2] = r[i].pos.z;
        out[i].invPositionProbability = r[i].inv;
        out[i].Nlight[0] = r[i].nl.x; out[i].Nlight[1] = r[i].nl.y; out[i].Nlight[2] = r[i].nl.z;
        out[i].pHat = r[i].pHat;
    }
}
void orc_write_reservoirs(orc_ctx* c, int role, const vxr_reservoir_rec* in) {
    o_res* r = c->res[role_index(c, role)];
    for (size_t i = 0; i < (size_t)c->W * c->H; i++) {
        r[i].sumW = in[i].sumOfWeights; r[i].M = in[i].streamLength; r[i].idx = in[i].lightIndex;
        r[i].W = in[i].adjustedWeight; r[i].pos = ld3(in[i].positionOnVoxel);
        r[i].inv = in[i].invPositionProbability; r[i].nl = ld3(in[i].Nlight); r[i].pHat = in[i].pHat;
    }
}
void orc_read_image(const orc_ctx* c, int which, float* rgba) {
    memcpy(rgba, which == 0 ? c->frame : c->accum, (size_t)c->W * c->H * 4 * sizeof(float));
}
uint32_t orc_trace(const orc_ctx* c, int mode, const float O[3], const float D[3], int steps, uint32_t through,
                   uint32_t mask, float* dist, uint32_t* side) {
    return o_trace(&c->w, mode, ld3(O), ld3(D), steps, through, mask, dist, side);
}
