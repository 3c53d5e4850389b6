/* ref_stb.c — test infrastructure only: the decoder the reference's asset
 * loader calls for PNG / JPEG / HDR textures (core/assets/asset_loader.cpp:109
 * stbi_load with 4 channels, :150 stbi_loadf with 4 channels), i.e. the
 * reference's vendored extern/stb/stb_image.h, compiled from the checkout by
 * oracle/build_ref.sh into oracle/_ref/libref_stb.so (nothing of it is copied
 * here).  The tests compare the library's own image decoders with it. */
#define STB_IMAGE_IMPLEMENTATION
#include "stb/stb_image.h"

/* 8-bit RGBA of an image in memory (malloc'ed; free with ref_stb_free). */
unsigned char* ref_stb_load_rgba8(const unsigned char* data, int size, int* w, int* h) {
    int n = 0;
    return stbi_load_from_memory(data, size, w, h, &n, 4);
}

/* Float RGBA (stbi_loadf: HDR files as stored, 8-bit images through stb's gamma). */
float* ref_stb_load_rgbaf(const unsigned char* data, int size, int* w, int* h) {
    int n = 0;
    return stbi_loadf_from_memory(data, size, w, h, &n, 4);
}

void ref_stb_free(void* p) { stbi_image_free(p); }
