/* stb_ref.c - the reference's vendored stb_image / stb_image_write (lib/stb_image.h,
 * lib/stb_image_write.h of marsicplusplus/SmallProject), compiled where they lie into
 * oracle/_ref/libstbref.so by oracle/ref_build.py.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the .hdr reader of the scene-file module
 * (World::LoadSky reads sky domes through stbi_loadf, template/world.cpp:808). Nothing
 * in the product links it. */
#define STB_IMAGE_IMPLEMENTATION
#define STBI_ONLY_HDR
#define STBI_NO_THREAD_LOCALS
#include "stb_image.h"
#define STB_IMAGE_WRITE_IMPLEMENTATION
#include "stb_image_write.h"

/* stbi_loadf(path, &w, &h, &comp, 0): pixels (w * h * comp floats) or NULL */
float* stbref_loadf(const char* path, int* w, int* h, int* comp) { return stbi_loadf(path, w, h, comp, 0); }
void stbref_free(void* p) { stbi_image_free(p); }
/* stbi_write_hdr: 1 on success */
int stbref_write_hdr(const char* path, int w, int h, int comp, const float* data) {
    return stbi_write_hdr(path, w, h, comp, data);
}
