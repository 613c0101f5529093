// capi_world.cpp - C ABI of the host voxel store and the scene generator.
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "internal.hpp"
#include "world.hpp"

namespace vxr {
int scene_preset(int config, vxr_scene_desc* d);
int scene_generate(World& w, const vxr_scene_desc& d);
int scene_height(const vxr_scene_desc* d, uint32_t x, uint32_t z, uint32_t* h);
int camera_path(const vxr_scene_desc* d, uint32_t seed, uint32_t f, uint32_t n, float pos[3], float target[3]);
void release_device_world(World& w);
int cluster_lights(World& w, uint32_t k, uint32_t seed, uint32_t iters);

static thread_local std::string g_err;
int set_error(int code, const std::string& msg) {
    g_err = msg;
    return code;
}
void clear_error() { g_err.clear(); }

std::string device_flags_message(uint32_t flags) {
    static const char* const names[] = {"bit 0", "temporal light index", "spatial light index", "shading light index",
                                         "tensor-core wait gave up"};
    char hex[16];
    std::snprintf(hex, sizeof(hex), "0x%x", flags);
    std::string m = std::string("device error flags ") + hex + " (";
    bool first = true;
    for (int b = 0; b < 32; b++) {
        if (!(flags >> b & 1u)) continue;
        if (!first) m += ", ";
        first = false;
        m += std::to_string(1u << b) + ": " + (b < 5 ? names[b] : "unknown");
    }
    return m + ")";
}
}  // namespace vxr

using vxr::set_error;

extern "C" {

const char* vxr_last_error(void) { return vxr::g_err.c_str(); }
const char* vxr_version(void) { return "vxr 0.1 (sm_103a)"; }

int vxr_world_create(vxr_world** out) {
    VXR_CHECK_ARG(out, "vxr_world_create: null out");
    try {
        *out = new vxr_world();
    } catch (const std::bad_alloc&) {
        return set_error(VXR_E_NOMEM, "vxr_world_create: out of host memory");
    }
    return VXR_OK;
}

int vxr_world_destroy(vxr_world* w) {
    if (!w) return VXR_OK;
    vxr::release_device_world(w->w);
    delete w;
    return VXR_OK;
}

int vxr_world_clear(vxr_world* w) {
    VXR_CHECK_ARG(w, "vxr_world_clear: null world");
    w->w.clear();
    return VXR_OK;
}

int vxr_world_set(vxr_world* w, uint32_t x, uint32_t y, uint32_t z, uint32_t voxel) {
    VXR_CHECK_ARG(w, "vxr_world_set: null world");
    try {
        w->w.set(x, y, z, voxel);
    } catch (const std::bad_alloc&) {
        return set_error(VXR_E_NOMEM, "vxr_world_set: brick pool allocation failed");
    }
    return VXR_OK;
}

int vxr_world_add_brick(vxr_world* w, uint32_t bx, uint32_t by, uint32_t bz, uint32_t voxel) {
    VXR_CHECK_ARG(w, "vxr_world_add_brick: null world");
    w->w.add_brick(bx, by, bz, voxel);
    return VXR_OK;
}

int vxr_world_stamp(vxr_world* w, const uint32_t* pos, const uint32_t* voxels, uint32_t n, uint32_t ox, uint32_t oy,
                    uint32_t oz, uint32_t or_mask) {
    VXR_CHECK_ARG(w && ((pos && voxels) || n == 0), "vxr_world_stamp: null argument");
    try {
        for (uint32_t i = 0; i < n; i++) {
            const uint32_t p = pos[i];
            w->w.set((p & 1023u) + ox, ((p >> 10) & 1023u) + oy, ((p >> 20) & 1023u) + oz, voxels[i] | or_mask);
        }
    } catch (const std::bad_alloc&) {
        return set_error(VXR_E_NOMEM, "vxr_world_stamp: brick pool allocation failed");
    }
    return VXR_OK;
}

int vxr_world_get(const vxr_world* w, uint32_t x, uint32_t y, uint32_t z, uint32_t* voxel) {
    VXR_CHECK_ARG(w && voxel, "vxr_world_get: null argument");
    *voxel = w->w.get(x, y, z);
    return VXR_OK;
}

int vxr_world_box(vxr_world* w, int x1, int y1, int z1, int x2, int y2, int z2, uint32_t voxel) {
    VXR_CHECK_ARG(w, "vxr_world_box: null world");
    try {
        for (int y = y1; y < y2; y++)
            for (int z = z1; z < z2; z++)
                for (int x = x1; x < x2; x++) w->w.set((uint32_t)x, (uint32_t)y, (uint32_t)z, voxel);
    } catch (const std::bad_alloc&) {
        return set_error(VXR_E_NOMEM, "vxr_world_box: brick pool allocation failed");
    }
    return VXR_OK;
}

int vxr_world_track_lights(vxr_world* w, int enable) {
    VXR_CHECK_ARG(w, "vxr_world_track_lights: null world");
    w->w.trackLights = enable != 0;
    return VXR_OK;
}

int vxr_world_optimize(vxr_world* w, uint32_t* replaced) {
    VXR_CHECK_ARG(w, "vxr_world_optimize: null world");
    const uint32_t r = w->w.optimize();
    if (replaced) *replaced = r;
    return VXR_OK;
}

int vxr_world_scan_lights(vxr_world* w, uint32_t* count) {
    VXR_CHECK_ARG(w, "vxr_world_scan_lights: null world");
    const uint32_t n = w->w.scan_lights();
    if (count) *count = n;
    return VXR_OK;
}

int vxr_world_set_lights(vxr_world* w, const vxr_light* lights, uint32_t n) {
    VXR_CHECK_ARG(w && (lights || n == 0), "vxr_world_set_lights: null argument");
    for (uint32_t i = 0; i < n; i++) {
        VXR_CHECK_ARG(lights[i].position < VXR_MAPDIM * VXR_MAPDIM * VXR_MAPDIM, "vxr_world_set_lights: position outside the map");
        VXR_CHECK_ARG(lights[i].size >= 1 && lights[i].size <= VXR_MAPDIM, "vxr_world_set_lights: size out of range");
    }
    w->w.lights.assign(lights, lights + n);
    w->w.lightVersion++;
    w->w.touch();
    return VXR_OK;
}

int vxr_world_move_light(vxr_world* w, uint32_t index, uint32_t x, uint32_t y, uint32_t z) {
    VXR_CHECK_ARG(w, "vxr_world_move_light: null world");
    const int r = w->w.move_light(index, x, y, z);
    VXR_CHECK_ARG(r != -1, "vxr_world_move_light: light index or position out of range");
    VXR_CHECK_ARG(r != -2, "vxr_world_move_light: only voxel lights (size 1) move");
    return VXR_OK;
}

int vxr_world_arrays(const vxr_world* w, const uint32_t** grid, const uint32_t** bricks, uint32_t* nbricks,
                     const vxr_light** lights, uint32_t* nlights) {
    VXR_CHECK_ARG(w, "vxr_world_arrays: null world");
    if (grid) *grid = w->w.grid.data();
    if (bricks) *bricks = w->w.bricks.empty() ? nullptr : w->w.bricks.data();
    if (nbricks) *nbricks = w->w.brickHigh;
    if (lights) *lights = w->w.lights.empty() ? nullptr : w->w.lights.data();
    if (nlights) *nlights = (uint32_t)w->w.lights.size();
    return VXR_OK;
}

int vxr_world_brick_count(const vxr_world* w, uint32_t* in_use) {
    VXR_CHECK_ARG(w && in_use, "vxr_world_brick_count: null argument");
    *in_use = w->w.bricks_in_use();
    return VXR_OK;
}

int vxr_world_cluster_lights(vxr_world* w, uint32_t k, uint32_t seed, uint32_t iters) {
    VXR_CHECK_ARG(w, "vxr_world_cluster_lights: null world");
    VXR_CHECK_ARG(k >= 1 && k <= 65536, "vxr_world_cluster_lights: k must be in [1, 65536]");
    try {
        return vxr::cluster_lights(w->w, k, seed, iters);
    } catch (const std::bad_alloc&) {
        return set_error(VXR_E_NOMEM, "vxr_world_cluster_lights: out of host memory");
    }
}

int vxr_world_light_clusters(const vxr_world* w, const uint32_t** ids, uint32_t* k) {
    VXR_CHECK_ARG(w && ids && k, "vxr_world_light_clusters: null argument");
    const bool valid = w->w.clusterCount > 0 && w->w.lightCluster.size() == w->w.lights.size();
    *ids = valid ? w->w.lightCluster.data() : nullptr;
    *k = valid ? w->w.clusterCount : 0;
    return VXR_OK;
}

int vxr_scene_preset(int config, vxr_scene_desc* desc) {
    VXR_CHECK_ARG(desc, "vxr_scene_preset: null desc");
    const int r = vxr::scene_preset(config, desc);
    if (r != VXR_OK) return set_error(r, "vxr_scene_preset: unknown configuration");
    return VXR_OK;
}

int vxr_scene_generate(vxr_world* w, const vxr_scene_desc* desc) {
    VXR_CHECK_ARG(w && desc, "vxr_scene_generate: null argument");
    VXR_CHECK_ARG(desc->extent >= 8 && desc->extent <= VXR_MAPDIM, "vxr_scene_generate: extent must be in [8, 1024]");
    VXR_CHECK_ARG(desc->gain > 0.0f && desc->base_freq > 0.0f, "vxr_scene_generate: gain and base_freq must be positive");
    try {
        return vxr::scene_generate(w->w, *desc);
    } catch (const std::bad_alloc&) {
        return set_error(VXR_E_NOMEM, "vxr_scene_generate: out of host memory");
    }
}

int vxr_scene_height(const vxr_scene_desc* desc, uint32_t x, uint32_t z, uint32_t* height) {
    VXR_CHECK_ARG(desc && height, "vxr_scene_height: null argument");
    const int r = vxr::scene_height(desc, x, z, height);
    if (r != VXR_OK) return set_error(r, "vxr_scene_height: column outside the scene extent");
    return VXR_OK;
}

int vxr_camera_path(const vxr_scene_desc* desc, uint32_t path_seed, uint32_t f, uint32_t n_frames, float pos[3],
                    float target[3]) {
    VXR_CHECK_ARG(desc && pos && target, "vxr_camera_path: null argument");
    return vxr::camera_path(desc, path_seed, f, n_frames, pos, target);
}

int vxr_world_checksum(const vxr_world* w, uint64_t* voxels, uint64_t* lights) {
    VXR_CHECK_ARG(w, "vxr_world_checksum: null world");
    const uint64_t P = 1099511628211ull;
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](uint32_t v) {
        for (int b = 0; b < 4; b++) {
            h ^= (v >> (8 * b)) & 255u;
            h *= P;
        }
    };
    const vxr::World& W = w->w;
    for (uint32_t i = 0; i < vxr::kGridSize; i++) {
        const uint32_t c = W.grid[i];
        if (c == 0) continue;
        mix(i);
        if ((c & 1u) == 0) {
            mix(0xFFFFFFFFu);
            mix(c >> 1);
        } else {
            const uint32_t* br = &W.bricks[(size_t)(c >> 1) * vxr::kBrick];
            for (uint32_t j = 0; j < vxr::kBrick; j++) mix(br[j]);
        }
    }
    if (voxels) *voxels = h;
    h = 1469598103934665603ull;
    for (const vxr_light& l : W.lights) {
        mix(l.position);
        mix(l.voxel);
        mix(l.size);
    }
    if (lights) *lights = h;
    return VXR_OK;
}

}  // extern "C"
