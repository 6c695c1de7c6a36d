// Host-side pixel work of the frame readers (slam_gb300/inputs.py): PNG
// scanline filter reconstruction for the TUM-format FileReader
// (src/inputs/FileReader.cpp:43-55 reads its PNG images through OpenCV).
#include <cstddef>
#include <cstdint>
#include <cstdlib>

#include "slam_gb300.h"

namespace {

// The Paeth predictor of the PNG format (ISO/IEC 15948, filter type 4):
// the neighbour (left a, above b, upper-left c) closest to a + b - c, ties
// in the order a, b, c.
inline uint8_t paeth(int a, int b, int c) {
    const int p = a + b - c;
    const int pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
    if (pa <= pb && pa <= pc) return (uint8_t)a;
    if (pb <= pc) return (uint8_t)b;
    return (uint8_t)c;
}

}  // namespace

extern "C" int odo_png_unfilter(const uint8_t *filtered, int height, size_t row_bytes, int bpp, uint8_t *out) {
    if (!filtered || !out || height < 0 || bpp < 1 || bpp > 8 || row_bytes == 0) return ODO_ERR_ARG;
    const uint8_t *prev = nullptr;  // reconstructed row above (none for the first row)
    for (int y = 0; y < height; ++y) {
        const uint8_t *src = filtered + (size_t)y * (row_bytes + 1);
        const int type = src[0];
        ++src;
        uint8_t *dst = out + (size_t)y * row_bytes;
        for (size_t i = 0; i < row_bytes; ++i) {
            const int a = i >= (size_t)bpp ? dst[i - bpp] : 0;
            const int b = prev ? prev[i] : 0;
            const int c = (prev && i >= (size_t)bpp) ? prev[i - bpp] : 0;
            int v;
            switch (type) {
                case 0: v = src[i]; break;
                case 1: v = src[i] + a; break;
                case 2: v = src[i] + b; break;
                case 3: v = src[i] + ((a + b) >> 1); break;
                case 4: v = src[i] + paeth(a, b, c); break;
                default: return ODO_ERR_ARG;
            }
            dst[i] = (uint8_t)v;
        }
        prev = dst;
    }
    return ODO_OK;
}
