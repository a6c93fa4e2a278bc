// image_io.cpp -- host-side image decoding support for the scene loader.
//
// PNG scanline reconstruction (ISO/IEC 15948, section 9: filter types None, Sub,
// Up, Average, Paeth).  Sub, Average and Paeth depend on the byte just
// reconstructed to their left, so the loop runs here rather than in Python.
#include <cstdint>
#include <cstdlib>

#include "../../include/xr.h"

namespace {

inline uint8_t paeth(int a, int b, int c) {
    const int p = a + b - c;
    const int pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
    if (pa <= pb && pa <= pc) return (uint8_t)a;
    if (pb <= pc) return (uint8_t)b;
    return (uint8_t)c;
}

}  // namespace

extern "C" xr_status xr_png_unfilter(const uint8_t* filtered, uint32_t rows, uint32_t row_bytes, uint32_t bpp,
                                     uint8_t* out) {
    if (!filtered || !out || bpp == 0 || bpp > 8) return XR_ERR_INVALID_ARGUMENT;
    const uint8_t* prev = nullptr;
    for (uint32_t y = 0; y < rows; y++) {
        const uint8_t* in = filtered + (size_t)y * (row_bytes + 1);
        uint8_t* cur = out + (size_t)y * row_bytes;
        const uint8_t type = in[0];
        ++in;
        for (uint32_t i = 0; i < row_bytes; i++) {
            const int a = i >= bpp ? cur[i - bpp] : 0;
            const int b = prev ? prev[i] : 0;
            const int c = (prev && i >= bpp) ? prev[i - bpp] : 0;
            int v = in[i];
            switch (type) {
                case 0: break;
                case 1: v += a; break;
                case 2: v += b; break;
                case 3: v += (a + b) >> 1; break;
                case 4: v += paeth(a, b, c); break;
                default: return XR_ERR_INVALID_ARGUMENT;
            }
            cur[i] = (uint8_t)(v & 255);
        }
        prev = cur;
    }
    return XR_OK;
}
