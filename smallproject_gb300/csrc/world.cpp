// world.cpp - host voxel store operations (World::Set/Get/OptimizeBricks/lights).
#include "world.hpp"

#include <algorithm>
#include <cstring>

namespace vxr {

World::World() { clear(); }

World::~World() = default;

// World::Clear (world.cpp:726-745): empty grid, all bricks recycled, no lights.
void World::clear() {
    grid.assign(kGridSize, 0u);
    bricks.clear();
    bricks.shrink_to_fit();
    zeroes.clear();
    freeList.clear();
    brickHigh = 0;
    lights.clear();
    covered.clear();
    dirty.clear();
    dirtyCount = 0;
    mark_all();
    touch();
    lightVersion++;
}

uint32_t World::new_brick() {
    if (!freeList.empty()) {
        const uint32_t b = freeList.back();
        freeList.pop_back();
        return b;
    }
    const uint32_t b = brickHigh++;
    if ((size_t)brickHigh * kBrick > bricks.size()) {
        const size_t cap = std::max<size_t>((size_t)brickHigh * 2, 1024);
        bricks.resize(cap * kBrick, 0u);
        zeroes.resize(cap, 0u);
    }
    return b;
}

void World::free_brick(uint32_t idx) { freeList.push_back(idx); }

// World::Get (world.h:293-306)
uint32_t World::get(uint32_t x, uint32_t y, uint32_t z) const {
    const uint32_t bx = (x / 8) & (kGrid - 1), by = (y / 8) & (kGrid - 1), bz = (z / 8) & (kGrid - 1);
    const uint32_t c = grid[cell_index(bx, by, bz)];
    if ((c & 1u) == 0) return c >> 1;
    const uint32_t lx = x & 7, ly = y & 7, lz = z & 7;
    return bricks[(size_t)(c >> 1) * kBrick + lx + ly * 8 + lz * 64];
}

// World::AddLight (world.cpp:228-246): append; any light change resets temporal reuse.
void World::add_light(uint32_t x, uint32_t y, uint32_t z, uint32_t size, uint32_t v) {
    vxr_light l;
    l.position = x + z * kMap + y * kMap * kMap;
    l.voxel = v;
    l.size = size;
    lights.push_back(l);
    lightVersion++;
}

// World::RemoveLight (world.cpp:506-561): drop every entry at this position, keep order.
void World::remove_light(uint32_t x, uint32_t y, uint32_t z) {
    const uint32_t p = x + z * kMap + y * kMap * kMap;
    lights.erase(std::remove_if(lights.begin(), lights.end(), [p](const vxr_light& l) { return l.position == p; }),
                 lights.end());
    lightVersion++;
}

// World::MoveLights for one light (world.cpp:268-305): restore the voxel the light
// covered (0 when none was remembered), draw its emitter voxel at (x, y, z) and remember
// the non-emitter voxel it covers there; the list entry keeps its index. Voxel lights
// (size 1) only. Returns 0, or -1 for an index or position out of range, -2 for a
// brick light.
int World::move_light(uint32_t index, uint32_t x, uint32_t y, uint32_t z) {
    if (index >= lights.size() || x >= kMap || y >= kMap || z >= kMap) return -1;
    vxr_light& l = lights[index];
    if (l.size != 1u) return -2;
    const uint32_t from = l.position, to = x + z * kMap + y * kMap * kMap;
    if (from == to) return 0;
    const uint32_t fx = from % kMap, fz = (from / kMap) % kMap, fy = from / (kMap * kMap);
    const uint32_t under = get(x, y, z);
    uint32_t restore = 0u;
    const auto it = covered.find(from);
    if (it != covered.end()) {
        restore = it->second;
        covered.erase(it);
    }
    if (!is_emitter(under)) covered[to] = under;
    const bool track = trackLights;
    trackLights = false;
    set(fx, fy, fz, restore);
    set(x, y, z, l.voxel);
    trackLights = track;
    l.position = to;
    lightMoveVersion++;
    touch();
    return 0;
}

// World::Set (world.h:456-513): split a solid cell into a brick when needed, keep the
// per-brick zero count, free the brick when it becomes all-empty.
void World::set(uint32_t x, uint32_t y, uint32_t z, uint32_t v) {
    const uint32_t bx = x / 8, by = y / 8, bz = z / 8;
    if (bx >= kGrid || by >= kGrid || bz >= kGrid) return;
    const uint32_t ci = cell_index(bx, by, bz);
    uint32_t c = grid[ci];
    uint32_t b = c >> 1;
    if ((c & 1u) == 0) {
        const uint32_t colour = c >> 1;
        if (v == colour) return;
        // World::SplitSolidBrick (world.h:392-445)
        b = new_brick();
        std::fill(bricks.begin() + (size_t)b * kBrick, bricks.begin() + (size_t)(b + 1) * kBrick, colour);
        zeroes[b] = (colour == 0) ? kBrick : 0u;
        grid[ci] = (b << 1) | 1u;
        mark_brick(b);
        mark_row(by);
    }
    const size_t vi = (size_t)b * kBrick + (x & 7) + (y & 7) * 8 + (z & 7) * 64;
    const uint32_t orig = bricks[vi];
    if (trackLights) {
        if (is_emitter(orig)) remove_light(x, y, z);
        if (is_emitter(v)) add_light(x, y, z, 1, v);
    }
    const int zeroChange = (int)(orig != 0 && v == 0) - (int)(orig == 0 && v != 0);
    zeroes[b] = (uint32_t)((int)zeroes[b] + zeroChange);
    if (zeroes[b] < kBrick) {
        bricks[vi] = v;
        mark_brick(b);
    } else {
        grid[ci] = 0;
        free_brick(b);
        mark_row(by);
    }
    touch();
}

// World::AddBrick (world.h:308-352): the cell becomes solid with value v. A brick that
// was there is freed and its emitter voxels leave the light list; a solid emitter cell
// that was there leaves it as a brick light; an emitter v joins it as a brick light
// (size 8, at the cell's lowest corner).
void World::add_brick(uint32_t bx, uint32_t by, uint32_t bz, uint32_t v) {
    if (bx >= kGrid || by >= kGrid || bz >= kGrid) return;
    const uint32_t ci = cell_index(bx, by, bz);
    const uint32_t c = grid[ci];
    if (c & 1u) {
        const uint32_t b = c >> 1;
        free_brick(b);
        if (trackLights)
            for (uint32_t ly = 0; ly < 8; ly++)
                for (uint32_t lz = 0; lz < 8; lz++)
                    for (uint32_t lx = 0; lx < 8; lx++)
                        if (is_emitter(bricks[(size_t)b * kBrick + lx + ly * 8 + lz * 64]))
                            remove_light(bx * 8 + lx, by * 8 + ly, bz * 8 + lz);
    } else if (trackLights && is_emitter(c >> 1)) {
        remove_light(bx * 8, by * 8, bz * 8);
    }
    if (trackLights && is_emitter(v)) add_light(bx * 8, by * 8, bz * 8, 8, v);
    grid[ci] = v << 1;
    mark_row(by);
    touch();
}

// World::OptimizeBricks (world.cpp:655-683)
uint32_t World::optimize() {
    uint32_t replaced = 0;
    for (uint32_t i = 0; i < kGridSize; i++) {
        const uint32_t c = grid[i];
        if (!(c & 1u)) continue;
        const uint32_t* br = &bricks[(size_t)(c >> 1) * kBrick];
        const uint32_t first = br[0];
        bool solid = true;
        for (uint32_t j = 1; j < kBrick; j++)
            if (br[j] != first) { solid = false; break; }
        if (solid) {
            grid[i] = first << 1;
            free_brick(c >> 1);
            mark_row(i / (kGrid * kGrid));
            replaced++;
        }
    }
    if (replaced) touch();
    return replaced;
}

// World::FindLightsInWord + SetupLightBuffer (world.cpp:438-504, 563-612)
uint32_t World::scan_lights() {
    lights.clear();
    for (uint32_t by = 0; by < kGrid; by++)
        for (uint32_t bz = 0; bz < kGrid; bz++)
            for (uint32_t bx = 0; bx < kGrid; bx++) {
                const uint32_t g = grid[cell_index(bx, by, bz)];
                if ((g & 1u) == 0) {
                    const uint32_t vox = g >> 1;
                    if (is_emitter(vox)) {
                        vxr_light l;
                        l.position = bx * 8 + bz * 8 * kMap + by * 8 * kMap * kMap;
                        l.voxel = vox;
                        l.size = 8;
                        lights.push_back(l);
                    }
                } else {
                    const uint32_t* br = &bricks[(size_t)(g >> 1) * kBrick];
                    for (uint32_t ly = 0; ly < 8; ly++)
                        for (uint32_t lz = 0; lz < 8; lz++)
                            for (uint32_t lx = 0; lx < 8; lx++) {
                                const uint32_t vox = br[lx + ly * 8 + lz * 64];
                                if (is_emitter(vox)) {
                                    const uint32_t x = lx + bx * 8, y = ly + by * 8, z = lz + bz * 8;
                                    vxr_light l;
                                    l.position = x + z * kMap + y * kMap * kMap;
                                    l.voxel = vox;
                                    l.size = 1;
                                    lights.push_back(l);
                                }
                            }
                }
            }
    lightVersion++;
    touch();
    return (uint32_t)lights.size();
}

}  // namespace vxr
