// devhost.cpp - compiles the product's device header (device.cuh) for the host CPU so
// its DDA traversal (recursive and resumable forms) and its sin/cos can be compared
// with the oracle without a GPU. Test infrastructure only.
//
// Host stand-ins for the CUDA intrinsics device.cuh uses; each has the semantics the
// device instruction has (round-toward-zero saturating conversions, raw bit casts).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

static inline unsigned __float2uint_rz(float f) {
    if (!(f > 0.0f)) return 0u;
    if (f >= 4294967296.0f) return 0xFFFFFFFFu;
    return (unsigned)f;
}
static inline int __float2int_rz(float f) {
    if (f != f) return 0;
    if (f >= 2147483648.0f) return 2147483647;
    if (f <= -2147483648.0f) return (int)0x80000000u;
    return (int)f;
}
static inline float __uint_as_float(unsigned u) { float f; std::memcpy(&f, &u, 4); return f; }
static inline unsigned __float_as_uint(float f) { unsigned u; std::memcpy(&u, &f, 4); return u; }
static inline float __uint2float_rn(unsigned u) { return (float)u; }
template <class T> static inline T __ldg(const T* p) { return *p; }
using std::max;
using std::min;
#ifndef __noinline__
#define __noinline__ __attribute__((noinline))
#endif

#include "device.cuh"

using namespace vxr::dev;

static World make_world(const uint32_t* grid, const uint8_t* uber, const uint32_t* bricks) {
    World w;
    w.grid = grid; w.uber = uber; w.bricks = bricks; w.lgeom = nullptr; w.lemit = nullptr; w.nlights = 0;
    return w;
}

extern "C" {

uint32_t dh_trace(int mode, const uint32_t* grid, const uint8_t* uber, const uint32_t* bricks, const float* O,
                  const float* D, int steps, uint32_t through, uint32_t mask, float* dist, uint32_t* side) {
    const World w = make_world(grid, uber, bricks);
    float d = 0.0f;
    uint32_t s = 0;
    uint32_t v;
    if (mode == 0) v = trace<0>(w, O[0], O[1], O[2], D[0], D[1], D[2], steps, through, mask, &d, &s);
    else if (mode == 1) v = trace<1>(w, O[0], O[1], O[2], D[0], D[1], D[2], steps, through, mask, &d, &s);
    else v = trace<2>(w, O[0], O[1], O[2], D[0], D[1], D[2], steps, through, mask, &d, &s);
    *dist = d;
    *side = s;
    return v;
}

// resumable walker run to completion; *status: 1 hit, 2 miss; *visits: cells visited
uint32_t dh_walk(const uint32_t* grid, const uint8_t* uber, const uint32_t* bricks, const float* O, const float* D,
                 int steps, float* dist, uint32_t* side, int* status, int* visits) {
    const World w = make_world(grid, uber, bricks);
    Walker k;
    int st = walk_init(k, w, O[0], O[1], O[2], D[0], D[1], D[2], steps);
    int n = 0;
    while (st == WALK_CONTINUE) {
        st = walk_step(k, w);
        n++;
    }
    *status = st;
    *visits = n;
    if (st == WALK_HIT) {
        *dist = k.dist;
        *side = k.side;
        return k.voxel;
    }
    *dist = 0.0f;
    *side = 0;
    return 0u;
}

void dh_sincos(float a, float* s, float* c) { sincos_vx(a, s, c); }

}  // extern "C"
