// Client of the denoiser class of the C++ API (IntelOpenImageDenoiser in
// include/petrichor_gb300/Petrichor.hpp), called as the reference's application calls
// it: Denoise(color, albedo, normal, isHDR) on Texture2D images.
//
//   denoise_client <width> <height> <images.bin> <out.bin> [colour-only]
//
// images.bin holds the colour, albedo and normal images (RGB float32 rows, in that
// order); out.bin receives the denoised image.
#include <petrichor_gb300/Petrichor.hpp>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

using namespace Petrichor::Core;

int main(int argc, char** argv) {
    if (argc < 5) return 2;
    const int W = std::atoi(argv[1]), H = std::atoi(argv[2]);
    const size_t n = (size_t)W * H * 3;
    std::vector<float> buf(3 * n);
    std::ifstream in(argv[3], std::ios::binary);
    if (!in.read(reinterpret_cast<char*>(buf.data()), (std::streamsize)(buf.size() * 4))) return 2;
    Texture2D img[3];
    for (int k = 0; k < 3; k++) {
        img[k] = Texture2D(W, H);
        std::memcpy(img[k].GetRawDataPtr(), buf.data() + k * n, n * 4);
    }
    IntelOpenImageDenoiser denoiser;
    const bool colourOnly = argc > 5 && std::string(argv[5]) == "colour-only";
    const Texture2D out = colourOnly ? denoiser.Denoise(img[0], true)
                                     : denoiser.Denoise(img[0], img[1], img[2], true);
    std::ofstream o(argv[4], std::ios::binary);
    o.write(reinterpret_cast<const char*>(out.GetRawDataPtr()), (std::streamsize)(n * 4));
    return o ? 0 : 1;
}
