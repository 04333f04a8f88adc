// C++ API over the C ABI: BICOS::match, BICOS::Image, BICOS::Exception.
// Mirrors libBICOS src/lib.cpp:31-49 and src/exception.cpp:23-27; output
// (re)creation follows src/impl/cuda.cu.in:139-147,190-191,216-217.
#include <cuda_runtime.h>

#include <stdexcept>

#include "../../include/BICOS/match.hpp"
#include "../../include/bicos_c.h"

namespace BICOS {

Exception::Exception(const std::string& message): _message(message) {}
const char* Exception::what() const throw() { return _message.c_str(); }

namespace {
void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess)
        throw Exception(std::string("libBICOS CUDA error in ") + what + ": " + cudaGetErrorString(e));
}
size_t type_bytes(int t) {
    switch (t) {
        case IMG_8U: return 1;
        case IMG_16U:
        case IMG_16S: return 2;
        case IMG_32F: return 4;
        case IMG_64F: return 8;
        default: throw Exception("unsupported image type");
    }
}
bicos_image view(const Image& im) {
    bicos_image v;
    v.data = im.data;
    v.step = im.step;
    v.rows = im.rows;
    v.cols = im.cols;
    v.type = im.type();
    v.reserved = 0;
    return v;
}
}  // namespace

Image::Image(int r, int c, int t) { create(r, c, t); }

Image::Image(int r, int c, int t, void* d, size_t s): data(d), step(s), rows(r), cols(c), _type(t) {
    type_bytes(t);
}

size_t Image::elemSize() const { return type_bytes(_type); }

void Image::create(int r, int c, int t) {
    if (data && rows == r && cols == c && _type == t)
        return;
    release();
    void* p = nullptr;
    size_t pitch = 0;
    check(cudaMallocPitch(&p, &pitch, (size_t)c * type_bytes(t), (size_t)r), "cudaMallocPitch");
    _owner = std::shared_ptr<void>(p, [](void* q) { cudaFree(q); });
    data = p;
    step = pitch;
    rows = r;
    cols = c;
    _type = t;
}

void Image::release() {
    _owner.reset();
    data = nullptr;
    step = 0;
    rows = cols = 0;
}

void Image::upload(const void* host, size_t host_step, Stream s) {
    check(cudaMemcpy2DAsync(data, step, host, host_step, (size_t)cols * elemSize(), rows, cudaMemcpyHostToDevice,
                            reinterpret_cast<cudaStream_t>(s)),
          "cudaMemcpy2DAsync");
}

void Image::download(void* host, size_t host_step, Stream s) const {
    check(cudaMemcpy2DAsync(host, host_step, data, step, (size_t)cols * elemSize(), rows, cudaMemcpyDeviceToHost,
                            reinterpret_cast<cudaStream_t>(s)),
          "cudaMemcpy2DAsync");
    check(cudaStreamSynchronize(reinterpret_cast<cudaStream_t>(s)), "cudaStreamSynchronize");
}

void match(const std::vector<Image>& stack0, const std::vector<Image>& stack1, Image& disparity, Config cfg,
           Image* corrmap, Stream stream) {
    const size_t n = stack0.size();
    if (n < 2)
        throw Exception("need at least two images");
    if (stack1.size() != n)
        throw Exception("both stacks must hold the same number of images");

    bicos_config c;
    bicos_config_default(&c);
    c.has_threshold = cfg.nxcorr_threshold.has_value();
    c.nxcorr_threshold = cfg.nxcorr_threshold.value_or(0.f);
    c.has_subpixel_step = cfg.subpixel_step.has_value();
    c.subpixel_step = cfg.subpixel_step.value_or(0.f);
    c.has_min_variance = cfg.min_variance.has_value();
    c.min_variance = cfg.min_variance.value_or(0.f);
    c.mode = cfg.mode == TransformMode::FULL ? BICOS_MODE_FULL : BICOS_MODE_LIMITED;
    c.precision = cfg.precision == Precision::DOUBLE ? BICOS_PRECISION_DOUBLE : BICOS_PRECISION_SINGLE;
    if (std::holds_alternative<Variant::Consistency>(cfg.variant)) {
        const auto& v = std::get<Variant::Consistency>(cfg.variant);
        c.variant = BICOS_VARIANT_CONSISTENCY;
        c.max_lr_diff = v.max_lr_diff;
        c.no_dupes = v.no_dupes;
    } else {
        c.variant = BICOS_VARIANT_NODUPLICATES;
    }

    int32_t dt = 0, ct = 0;
    bicos_output_types(&c, &dt, &ct);
    const int rows = stack0.front().rows, cols = stack0.front().cols;
    disparity.create(rows, cols, dt);
    if (corrmap && ct >= 0)
        corrmap->create(rows, cols, ct);

    std::vector<bicos_image> v0, v1;
    for (size_t i = 0; i < n; ++i) {
        v0.push_back(view(stack0[i]));
        v1.push_back(view(stack1[i]));
    }
    bicos_image dv = view(disparity);
    bicos_image cv;
    if (corrmap && ct >= 0)
        cv = view(*corrmap);
    const bicos_status s = bicos_match_v1(v0.data(), v1.data(), (uint32_t)n, &dv, (corrmap && ct >= 0) ? &cv : nullptr,
                                          &c, reinterpret_cast<bicos_stream_t>(stream));
    if (s == BICOS_ERR_INVALID_ARGUMENT)
        throw std::invalid_argument(bicos_last_error());
    if (s != BICOS_OK)
        throw Exception(bicos_last_error());
}

}  // namespace BICOS
