// scene_host.cpp - the seeded procedural scenes and camera paths for the reference arm
// of the benchmark (test and benchmark infrastructure, not the product).
//
// The reference arm times the reference's own kernels on the host CPU (oracle/_ref) on the
// same inputs the CUDA arm renders. Those inputs come from the project's scene generator
// (smallproject_gb300/csrc/scene.cpp, world.cpp: terrain, emitters, camera spline). This
// file gives that generator a small C ABI and is compiled together with those two host
// sources into oracle/_build/libscenehost.so, so the reference arm builds its scene
// without loading the CUDA library. Frame constants come from the oracle's camera
// restatement (orc_begin_frame in vxr_oracle.c).
#include <cstring>
#include <new>

#include "world.hpp"

namespace vxr {
int scene_preset(int config, vxr_scene_desc* d);
int scene_generate(World& w, const vxr_scene_desc& d);
int camera_path(const vxr_scene_desc* d, uint32_t seed, uint32_t f, uint32_t n, float pos[3], float target[3]);
}  // namespace vxr

extern "C" {

int osh_preset(int config, vxr_scene_desc* d) { return d ? vxr::scene_preset(config, d) : VXR_E_INVALID; }

// a generated world (null on failure); free with osh_free
void* osh_generate(const vxr_scene_desc* d) {
    if (!d) return nullptr;
    vxr::World* w = new (std::nothrow) vxr::World();
    if (!w) return nullptr;
    try {
        if (vxr::scene_generate(*w, *d) != VXR_OK) {
            delete w;
            return nullptr;
        }
    } catch (const std::bad_alloc&) {
        delete w;
        return nullptr;
    }
    return w;
}

// the arrays the renderer reads: grid (128^3 cells), bricks (n x 512 voxels), lights
void osh_sizes(const void* h, uint32_t* nbricks, uint32_t* nlights) {
    const vxr::World* w = static_cast<const vxr::World*>(h);
    *nbricks = w->brickHigh;
    *nlights = (uint32_t)w->lights.size();
}

void osh_copy(const void* h, uint32_t* grid, uint32_t* bricks, vxr_light* lights) {
    const vxr::World* w = static_cast<const vxr::World*>(h);
    std::memcpy(grid, w->grid.data(), w->grid.size() * sizeof(uint32_t));
    if (w->brickHigh) std::memcpy(bricks, w->bricks.data(), (size_t)w->brickHigh * 512 * sizeof(uint32_t));
    if (!w->lights.empty()) std::memcpy(lights, w->lights.data(), w->lights.size() * sizeof(vxr_light));
}

int osh_camera_path(const vxr_scene_desc* d, uint32_t seed, uint32_t f, uint32_t n, float pos[3], float target[3]) {
    return vxr::camera_path(d, seed, f, n, pos, target);
}

void osh_free(void* h) { delete static_cast<vxr::World*>(h); }

}  // extern "C"
