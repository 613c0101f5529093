// ogt_ref.cpp - the reference's vendored opengametools .vox reader (lib/ogt_vox.h of
// marsicplusplus/SmallProject), compiled where it lies into oracle/_ref/libogtref.so by
// oracle/ref_build.py.
//
// TEST INFRASTRUCTURE ONLY: the checker for the large-model .vox reader of the package
// (LoadSprite(path, true) parses files with ogt_vox_read_scene, template/world.cpp:1041-
// 1049). Nothing in the product links it.
#define OGT_VOX_IMPLEMENTATION
#include "ogt_vox.h"

#include <cstring>

extern "C" {

// Parse a file image. Returns the scene (free with ogtref_free) or null.
const void* ogtref_read(const uint8_t* buf, uint32_t n) { return ogt_vox_read_scene(buf, n); }
void ogtref_free(const void* s) { ogt_vox_destroy_scene((const ogt_vox_scene*)s); }

// counts[0] = instances, counts[1] = models
void ogtref_counts(const void* s, uint32_t counts[2]) {
    const ogt_vox_scene* sc = (const ogt_vox_scene*)s;
    counts[0] = sc->num_instances;
    counts[1] = sc->num_models;
}

// instance i: model index and the 16 floats of its transform (m00, m01, ..., m33)
uint32_t ogtref_instance(const void* s, uint32_t i, float out[16]) {
    const ogt_vox_instance& in = ((const ogt_vox_scene*)s)->instances[i];
    std::memcpy(out, &in.transform, 16 * sizeof(float));
    return in.model_index;
}

// model m: size (x, y, z); with voxels non-null, its size_x * size_y * size_z indices
void ogtref_model(const void* s, uint32_t m, uint32_t size[3], uint8_t* voxels) {
    const ogt_vox_model* md = ((const ogt_vox_scene*)s)->models[m];
    size[0] = md->size_x;
    size[1] = md->size_y;
    size[2] = md->size_z;
    if (voxels) std::memcpy(voxels, md->voxel_data, (size_t)md->size_x * md->size_y * md->size_z);
}

// the 256 RGBA palette entries
void ogtref_palette(const void* s, uint8_t out[1024]) {
    std::memcpy(out, &((const ogt_vox_scene*)s)->palette, 1024);
}

}  // extern "C"
