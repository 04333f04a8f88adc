// Exercises the C++ entry point BICOS::match (include/BICOS/match.hpp) the
// way a libBICOS user does: device images per frame, Config with optionals
// and variants, disparity (re)created by match.  Reads a raw stack from
// argv[1] (n, rows, cols as int32 header, then left and right uint8
// frames), writes the int16/float32 disparity and the corrmap to argv[2].
#include <BICOS/match.hpp>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <vector>

int main(int argc, char** argv) {
    if (argc < 4)
        return 2;
    FILE* f = std::fopen(argv[1], "rb");
    int32_t hdr[3];
    if (!f || std::fread(hdr, 4, 3, f) != 3)
        return 3;
    const int n = hdr[0], rows = hdr[1], cols = hdr[2];
    std::vector<uint8_t> buf((size_t)2 * n * rows * cols);
    if (std::fread(buf.data(), 1, buf.size(), f) != buf.size())
        return 4;
    std::fclose(f);

    std::vector<BICOS::Image> s0, s1;
    for (int t = 0; t < n; ++t) {
        BICOS::Image a(rows, cols, BICOS::IMG_8U), b(rows, cols, BICOS::IMG_8U);
        a.upload(buf.data() + (size_t)t * rows * cols, cols);
        b.upload(buf.data() + (size_t)(n + t) * rows * cols, cols);
        s0.push_back(a);
        s1.push_back(b);
    }
    BICOS::Config cfg;
    cfg.nxcorr_threshold = 0.9f;
    cfg.min_variance = 2.0f;
    const int mode = std::atoi(argv[3]);
    if (mode == 1)
        cfg.subpixel_step = 0.1f;
    if (mode == 2)
        cfg.variant = BICOS::Variant::Consistency {1, true};

    BICOS::Image disp, corr;
    BICOS::match(s0, s1, disp, cfg, &corr);

    const size_t de = disp.elemSize();
    std::vector<uint8_t> dh((size_t)rows * cols * de), ch((size_t)rows * cols * 4);
    disp.download(dh.data(), cols * de);
    corr.download(ch.data(), cols * 4);
    FILE* o = std::fopen(argv[2], "wb");
    std::fwrite(dh.data(), 1, dh.size(), o);
    std::fwrite(ch.data(), 1, ch.size(), o);
    std::fclose(o);

    // error behaviour: too many frames for a 256-bit descriptor
    try {
        std::vector<BICOS::Image> big(66, s0[0]);
        BICOS::match(big, big, disp, cfg);
        return 5;
    } catch (const std::invalid_argument& e) {
        if (std::strstr(e.what(), "would require 257 bits") == nullptr)
            return 6;
    }
    try {
        std::vector<BICOS::Image> one(1, s0[0]);
        BICOS::match(one, one, disp, cfg);
        return 7;
    } catch (const BICOS::Exception& e) {
        if (std::strcmp(e.what(), "need at least two images") != 0)
            return 8;
    }
    return 0;
}
