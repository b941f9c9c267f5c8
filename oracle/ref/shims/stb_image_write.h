// Image-writing stand-in for the two stb_image_write calls in Core/Texture2D.cpp
// (Texture2D.cpp:197-252). Test oracle build only: writes nothing, reports failure.
#pragma once
#ifdef STB_IMAGE_WRITE_IMPLEMENTATION
static inline int stbi_write_png(const char*, int, int, int, const void*, int) { return 0; }
static inline int stbi_write_hdr(const char*, int, int, int, const float*) { return 0; }
#endif
