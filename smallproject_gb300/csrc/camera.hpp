// camera.hpp - host camera and per-frame constants of the render path.
#pragma once
#include <cstdint>
#include "vxr.h"

namespace vxr {

struct Mat4 {
    float cell[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
};

// mat4::LookAt (template/precomp.h:825-835)
Mat4 look_at(const float P[3], const float T[3]);

// Host state that World::Render keeps between frames (world.cpp:2144-2191, 2335-2337).
struct CameraState {
    Mat4 M;
    float E[3] = {0, 0, 0}, p0[3] = {0, 0, 0}, p1[3] = {0, 0, 0}, p2[3] = {0, 0, 0};
    bool firstFrame = true;
    uint32_t rng = 0x12345678u;   // RandomUInt state (template.cpp:933-941)
    uint32_t frame = 0, framecount = 0, restirtemporalframe = 0;
};

// Fill the frame constants for the next frame from the camera (the host part of
// World::Render); updates the stored previous-frame corners and draws R0.
void begin_frame(CameraState& st, uint32_t W, uint32_t H, vxr_frame_consts* k);
// Frame counters (world.cpp:2335-2337).
void end_frame(CameraState& st);

}  // namespace vxr
