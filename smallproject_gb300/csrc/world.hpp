// world.hpp - host-side brick-grid voxel store.
//
// Same storage semantics as the reference World (template/world.h:164-758): a fixed
// 1024^3 map split into 128^3 cells of 8^3 voxels. A cell is 0 (empty), an even value
// (solid colour << 1) or an odd value (brick index << 1 | 1) into a pool of 512-voxel
// bricks. The brick pool grows on demand instead of the reference's fixed 2 GB
// allocation (common.h:186-189); freed bricks are recycled LIFO. Brick numbering never
// affects rendering (only the cell -> brick mapping is read by the DDA).
#pragma once
#include <cstdint>
#include <unordered_map>
#include <vector>
#include "vxr.h"

namespace vxr {

constexpr uint32_t kMap = VXR_MAPDIM;
constexpr uint32_t kGrid = VXR_GRIDDIM;
constexpr uint32_t kGridSize = kGrid * kGrid * kGrid;
constexpr uint32_t kBrick = VXR_BRICKSIZE;

inline uint32_t cell_index(uint32_t bx, uint32_t by, uint32_t bz) { return bx + bz * kGrid + by * kGrid * kGrid; }
inline bool is_emitter(uint32_t v) { return ((v >> 16) & 255u) > 0; }  // common.h:203-206

struct DeviceWorld;  // GPU copy (runtime.cu)

struct World {
    std::vector<uint32_t> grid;        // kGridSize cells
    std::vector<uint32_t> bricks;      // brickCap * 512 voxels
    std::vector<uint32_t> zeroes;      // per brick: number of zero voxels (world.h:440, 500-512)
    std::vector<uint32_t> freeList;    // recycled brick indices
    uint32_t brickHigh = 0;            // bricks ever allocated (pool high-water mark)
    std::vector<vxr_light> lights;
    std::vector<uint32_t> lightCluster;   // cluster id per light (cluster_lights)
    uint32_t clusterCount = 0;
    uint64_t clusterVersion = 0;
    bool trackLights = true;
    uint64_t version = 1;              // bumps on every edit (device copy stale when different)
    uint64_t lightVersion = 1;         // bumps on every light-list change (temporal reset)
    uint64_t lightMoveVersion = 1;     // bumps when a light moves (list order kept)
    std::unordered_map<uint32_t, uint32_t> covered;   // voxel under a moved light (defaultVoxel)
    DeviceWorld* dev = nullptr;
    // device commit state (World::Commit / IsDirty / Mark, world.cpp:2357-2420,
    // world.h:565-613): bricks whose content changed since the last commit (1 bit each),
    // whether the top-level grid changed, whether everything must be sent again
    std::vector<uint32_t> dirty;
    uint32_t dirtyCount = 0;
    bool gridDirty = true;
    uint32_t gridRows[kGrid / 32] = {};   // grid y-layers (128^2 cells each) that changed
    bool fullDirty = true;
    void mark_row(uint32_t by) {
        gridDirty = true;
        gridRows[by >> 5] |= 1u << (by & 31);
    }
    void mark_brick(uint32_t b) {
        if ((b >> 5) >= dirty.size()) dirty.resize((b >> 5) + 1 + dirty.size() / 2, 0u);
        const uint32_t m = 1u << (b & 31);
        if (!(dirty[b >> 5] & m)) {
            dirty[b >> 5] |= m;
            dirtyCount++;
        }
    }
    void mark_all() {
        fullDirty = true;
        gridDirty = true;
    }

    World();
    ~World();
    void clear();
    uint32_t get(uint32_t x, uint32_t y, uint32_t z) const;
    void set(uint32_t x, uint32_t y, uint32_t z, uint32_t v);
    void add_brick(uint32_t bx, uint32_t by, uint32_t bz, uint32_t v);
    uint32_t optimize();
    uint32_t scan_lights();
    uint32_t new_brick();
    void free_brick(uint32_t idx);
    uint32_t bricks_in_use() const { return brickHigh - (uint32_t)freeList.size(); }
    void add_light(uint32_t x, uint32_t y, uint32_t z, uint32_t size, uint32_t v);
    void remove_light(uint32_t x, uint32_t y, uint32_t z);
    int move_light(uint32_t index, uint32_t x, uint32_t y, uint32_t z);
    void touch() { version++; }
};

}  // namespace vxr

// The opaque C handle of the C ABI.
struct vxr_world {
    vxr::World w;
};
