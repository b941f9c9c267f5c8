// Image-loading stand-in for the four stb_image entry points Core/Texture2D.cpp
// calls (Texture2D.cpp:107-195). Test oracle build only.
//
// A ".hdr" file here is the project's raw container, read back bit-exactly:
//   8 bytes "PTRAWF32", uint32 width, uint32 height, width*height*3 float32 (RGB,
//   row-major, top row first). PNG loading is not provided (returns null).
#pragma once
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#ifdef STB_IMAGE_IMPLEMENTATION
static inline void stbi_hdr_to_ldr_scale(float) {}
static inline void stbi_image_free(void* p) { std::free(p); }
static inline unsigned char* stbi_load(const char*, int*, int*, int*, int) { return nullptr; }
static inline float* stbi_loadf(const char* path, int* w, int* h, int* comp, int) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return nullptr;
    char magic[8];
    uint32_t dims[2];
    float* data = nullptr;
    if (std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "PTRAWF32", 8) == 0 &&
        std::fread(dims, 4, 2, f) == 2) {
        const size_t n = (size_t)dims[0] * dims[1] * 3;
        data = (float*)std::malloc(n * sizeof(float));
        if (data && std::fread(data, sizeof(float), n, f) != n) {
            std::free(data);
            data = nullptr;
        }
    }
    std::fclose(f);
    if (data) {
        *w = (int)dims[0];
        *h = (int)dims[1];
        if (comp) *comp = 3;
    }
    return data;
}
#endif
