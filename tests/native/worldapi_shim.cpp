// worldapi_shim.cpp - the worldapi.h shim a maintainer adds on top of libvxr (the same
// code as the integration guide shows), compiled and linked by tests/test_capi.py with a
// prelude standing in for the reference's types, and driven through its world calls
// (which need no GPU) and, with the argument "render", through LookAt / RenderFrame /
// CommitFrame on the GPU (tests/test_gpu_shim.py).
#include <cstdio>
#include <cstdlib>

#include "vxr.h"

// ---- prelude: what the reference's precomp.h provides to worldapi.h callers ----------
typedef unsigned int uint;
struct float3 {
    float x, y, z;
};
static void FatalError(const char* m) {
    std::fprintf(stderr, "%s\n", m);
    std::exit(1);
}

// ---- the shim ------------------------------------------------------------------------
static vxr_world* g_world;
static vxr_view* g_view;
static void ok(int r) { if (r) FatalError(vxr_last_error()); }

void InitVxr(uint w, uint h) {
    ok(vxr_world_create(&g_world));
    vxr_view_desc d; vxr_view_default_desc(&d); d.width = w; d.height = h;
    ok(vxr_view_create(g_world, &d, &g_view));
}
void Plot(const uint x, const uint y, const uint z, const uint c) { ok(vxr_world_set(g_world, x, y, z, c)); }
uint Read(const int x, const int y, const int z) { uint v; ok(vxr_world_get(g_world, x, y, z, &v)); return v; }
void Box(const int x1, const int y1, const int z1, const int x2, const int y2, const int z2, const uint c)
{ ok(vxr_world_box(g_world, x1, y1, z1, x2, y2, z2, c)); }
void ClearWorld() { ok(vxr_world_clear(g_world)); }
void LookAt(const float3 pos, const float3 target)
{ const float p[3] = {pos.x, pos.y, pos.z}, t[3] = {target.x, target.y, target.z}; ok(vxr_view_lookat(g_view, p, t)); }
// main loop: was world->Render(); game->Tick(dt); world->Commit();
void RenderFrame() { ok(vxr_view_render(g_view)); }
void CommitFrame() { ok(vxr_view_wait(g_view)); }

// ---- driver ----------------------------------------------------------------------------
// "render": a ground slab and one emitter voxel through Plot / Box, the camera through
// LookAt, three frames through RenderFrame / CommitFrame (needs a GPU), then the frame
// read back; prints lit pixels, non-finite values and the brightest value. Without
// arguments: the world half alone (no device needed).
static int render_demo() {
    InitVxr(96, 64);
    Box(0, 0, 0, 64, 4, 64, 0xF888);
    Plot(32, 10, 32, (10u << 16) | 0xFFFFu);        // strength 10, opaque, white
    const float3 pos = {32.0f, 30.0f, -20.0f}, tgt = {32.0f, 4.0f, 32.0f};
    for (int f = 0; f < 3; f++) {
        LookAt(pos, tgt);
        RenderFrame();
        CommitFrame();
    }
    static float rgba[96 * 64 * 4];
    ok(vxr_view_read_frame(g_view, rgba));
    int lit = 0, bad = 0;
    float mx = 0.0f;
    for (int i = 0; i < 96 * 64; i++) {
        for (int c = 0; c < 3; c++) {
            const float v = rgba[i * 4 + c];
            if (!(v == v) || v > 1e30f || v < -1e30f) bad++;
            if (v > mx) mx = v;
        }
        if (rgba[i * 4] + rgba[i * 4 + 1] + rgba[i * 4 + 2] > 0.0f) lit++;
    }
    std::printf("%d %d %g\n", lit, bad, mx);
    ok(vxr_view_destroy(g_view));
    ok(vxr_world_destroy(g_world));
    return (lit > 100 && bad == 0 && mx > 0.0f) ? 0 : 2;
}

int main(int argc, char** argv) {
    if (argc > 1 && argv[1][0] == 'r') return render_demo();
    ok(vxr_world_create(&g_world));
    Plot(10, 20, 30, 0xF888);
    Box(0, 0, 0, 4, 4, 4, 0xF123);
    const uint a = Read(10, 20, 30), b = Read(3, 3, 3), c = Read(4, 4, 4);
    ClearWorld();
    const uint d = Read(10, 20, 30);
    std::printf("%x %x %x %x\n", a, b, c, d);
    ok(vxr_world_destroy(g_world));
    return (a == 0xF888 && b == 0xF123 && c == 0 && d == 0) ? 0 : 2;
}
