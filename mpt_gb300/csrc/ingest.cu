// ingest.cu - host-side decoding helpers for scene ingestion (no device code).
//
// PNG scanline reconstruction (the five filter types of the PNG
// specification, ISO/IEC 15948 section 9): the row loop of an image decoder,
// which the reference gets from libpng (demo/png_2d_scenario.hpp:198-240) and
// which is too slow as an interpreted loop for demo-sized images.
#include "common.cuh"

static inline int paeth(int a, int b, int c) {
    const int p = a + b - c;
    const int pa = p > a ? p - a : a - p, pb = p > b ? p - b : b - p, pc = p > c ? p - c : c - p;
    return (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
}

extern "C" mptg_status mptg_png_unfilter(const uint8_t* raw, int height, int stride, int bpp, uint8_t* out) {
    if (!raw || !out || height < 0 || stride < 1 || bpp < 1 || bpp > 8) return MPTG_ERR_INVALID_ARG;
    for (int y = 0; y < height; ++y) {
        const uint8_t* in = raw + (size_t)y * (stride + 1);
        const int ft = in[0];
        ++in;
        uint8_t* cur = out + (size_t)y * stride;
        const uint8_t* prev = y ? cur - stride : nullptr;
        for (int x = 0; x < stride; ++x) {
            const int a = x >= bpp ? cur[x - bpp] : 0;
            const int b = prev ? prev[x] : 0;
            const int c = (prev && x >= bpp) ? prev[x - bpp] : 0;
            int p;
            switch (ft) {
                case 0: p = 0; break;
                case 1: p = a; break;
                case 2: p = b; break;
                case 3: p = (a + b) >> 1; break;
                case 4: p = paeth(a, b, c); break;
                default: return MPTG_ERR_INVALID_ARG;
            }
            cur[x] = (uint8_t)(in[x] + p);
        }
    }
    return MPTG_OK;
}
