// Host-side helpers of the command-line front end (libbicos_gb300.cli),
// which replaces libBICOS's OpenCV-based bicos-cli (src/cli.cpp).
//
// PNG row reconstruction (ISO/IEC 15948 section 9): each scanline carries
// a filter byte (None, Sub, Up, Average, Paeth) and its bytes are deltas
// against the reconstructed bytes to the left (bpp bytes back) and above.
// The left dependence makes this a sequential byte loop, which is why it
// lives here and not in the Python reader.
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>

#include "../../include/bicos_c.h"

namespace {

inline uint8_t paeth(int a, int b, int c) {
    const int p = a + b - c;
    const int pa = abs(p - a), pb = abs(p - b), pc = abs(p - c);
    if (pa <= pb && pa <= pc)
        return (uint8_t)a;
    return (uint8_t)(pb <= pc ? b : c);
}

}  // namespace

extern "C" int32_t bicos_png_unfilter(uint8_t* out, const uint8_t* raw, int32_t height, size_t stride,
                                      int32_t bpp) {
    if (!out || !raw || height < 0 || bpp < 1)
        return -1;
    const uint8_t* prev = nullptr;
    for (int32_t y = 0; y < height; ++y) {
        const uint8_t f = raw[(size_t)y * (stride + 1)];
        const uint8_t* in = raw + (size_t)y * (stride + 1) + 1;
        uint8_t* cur = out + (size_t)y * stride;
        for (size_t i = 0; i < stride; ++i) {
            const int a = i >= (size_t)bpp ? cur[i - bpp] : 0;
            const int b = prev ? prev[i] : 0;
            const int c = (prev && i >= (size_t)bpp) ? prev[i - bpp] : 0;
            int v;
            switch (f) {
                case 0: v = 0; break;
                case 1: v = a; break;
                case 2: v = b; break;
                case 3: v = (a + b) >> 1; break;
                case 4: v = paeth(a, b, c); break;
                default: return y + 1;  // row y has an unknown filter
            }
            cur[i] = (uint8_t)(in[i] + v);
        }
        prev = cur;
    }
    return 0;
}
