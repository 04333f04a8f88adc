// C entry points over libBICOS's own CPU backend, compiled from the
// reference sources in place (see oracle/ref_build.sh).  TEST
// INFRASTRUCTURE ONLY: used to pin the oracle restatement and to produce the
// golden vectors under tests/golden/.  Never part of the product library.
//
// Entry points mirror the reference functions they wrap:
//   ref_match           -> BICOS::impl::cpu::match          src/impl/cpu.cpp:96-155
//   ref_transform       -> cpu::descriptor_transform<...>    include/impl/cpu/descriptor_transform.hpp:125-138
//   ref_search          -> cpu::bicos<TDescriptor, FLAGS>    include/impl/cpu/bicos.hpp:78-113
//   ref_agree           -> cpu::agree<TInput>                include/impl/cpu/agree.hpp:52-92
//   ref_agree_subpixel  -> cpu::agree_subpixel<TInput>       include/impl/cpu/agree.hpp:94-185

#include "common.hpp"
#include "cpu.hpp"
#include "impl/cpu/agree.hpp"
#include "impl/cpu/bicos.hpp"
#include "impl/cpu/descriptor_transform.hpp"

#include <bitset>
#include <cstdio>
#include <cstring>

#include "bicos_oracle.h"

using namespace BICOS;
using namespace BICOS::impl;

namespace {

std::vector<cv::Mat> planes_of(const void* stack, int elem_bytes, int n, int rows, int cols) {
    std::vector<cv::Mat> v;
    const int type = elem_bytes == 1 ? CV_8UC1 : CV_16UC1;
    const size_t plane = (size_t)rows * cols * elem_bytes;
    for (int t = 0; t < n; ++t)
        v.emplace_back(rows, cols, type, (uint8_t*)stack + t * plane);
    return v;
}

template<typename T>
void to_words(const T& d, uint32_t* w, int nwords) {
    std::memset(w, 0, nwords * 4);
    std::memcpy(w, &d, std::min<size_t>(sizeof(T), nwords * 4));
}
template<>
void to_words(const std::bitset<256>& d, uint32_t* w, int nwords) {
    std::memset(w, 0, nwords * 4);
    for (int i = 0; i < 256 && i < nwords * 32; ++i)
        if (d.test(i))
            w[i >> 5] |= 1u << (i & 31);
}

template<typename T>
T from_words(const uint32_t* w, int nwords) {
    T d {};
    std::memcpy(&d, w, std::min<size_t>(sizeof(T), nwords * 4));
    return d;
}
template<>
std::bitset<256> from_words(const uint32_t* w, int nwords) {
    std::bitset<256> d;
    for (int i = 0; i < 256 && i < nwords * 32; ++i)
        if (w[i >> 5] >> (i & 31) & 1u)
            d.set(i);
    return d;
}

template<typename TIn, typename TDesc>
void transform_t(const void* stack, int elem_bytes, int n, int rows, int cols, int full, int nwords,
                 uint32_t* out) {
    cv::Mat merged;
    cv::merge(planes_of(stack, elem_bytes, n, rows, cols), merged);
    const cv::Size sz(cols, rows);
    auto d = full ? cpu::descriptor_transform<TIn, TDesc, cpu::transform_full<TIn, TDesc>>(merged, sz, n)
                  : cpu::descriptor_transform<TIn, TDesc, cpu::transform_limited<TIn, TDesc>>(merged, sz, n);
    for (int r = 0; r < rows; ++r)
        for (int c = 0; c < cols; ++c)
            to_words(d->row(r)[c], out + ((size_t)r * cols + c) * nwords, nwords);
}

template<typename TIn>
int transform_in(const void* stack, int elem_bytes, int n, int rows, int cols, int full, int nwords,
                 uint32_t* out) {
    switch (nwords) {
        case 1: transform_t<TIn, uint32_t>(stack, elem_bytes, n, rows, cols, full, nwords, out); break;
        case 2: transform_t<TIn, uint64_t>(stack, elem_bytes, n, rows, cols, full, nwords, out); break;
        case 4: transform_t<TIn, uint128_t>(stack, elem_bytes, n, rows, cols, full, nwords, out); break;
        case 8: transform_t<TIn, std::bitset<256>>(stack, elem_bytes, n, rows, cols, full, nwords, out); break;
        default: return ORC_ERR_INVALID_ARGUMENT;
    }
    return ORC_OK;
}

template<typename TDesc, int FLAGS>
void search_t(const uint32_t* d0, const uint32_t* d1, int rows, int cols, int nwords, int lr, int16_t* out) {
    const cv::Size sz(cols, rows);
    auto a = std::make_unique<cpu::StepBuf<TDesc>>(sz), b = std::make_unique<cpu::StepBuf<TDesc>>(sz);
    for (int r = 0; r < rows; ++r)
        for (int c = 0; c < cols; ++c) {
            const size_t px = (size_t)r * cols + c;
            a->row(r)[c] = from_words<TDesc>(d0 + px * nwords, nwords);
            b->row(r)[c] = from_words<TDesc>(d1 + px * nwords, nwords);
        }
    cv::Mat o;
    cpu::bicos<TDesc, FLAGS>(a, b, lr, sz, o);
    for (int r = 0; r < rows; ++r)
        std::memcpy(out + (size_t)r * cols, o.ptr<int16_t>(r), cols * sizeof(int16_t));
}

template<typename TDesc>
void search_d(const uint32_t* d0, const uint32_t* d1, int rows, int cols, int nwords, int flags, int lr,
              int16_t* out) {
    switch (flags) {
        case 0: search_t<TDesc, 0>(d0, d1, rows, cols, nwords, lr, out); break;
        case 1: search_t<TDesc, 1>(d0, d1, rows, cols, nwords, lr, out); break;
        case 2: search_t<TDesc, 2>(d0, d1, rows, cols, nwords, lr, out); break;
        default: search_t<TDesc, 3>(d0, d1, rows, cols, nwords, lr, out); break;
    }
}

} // namespace

extern "C" {

int ref_transform(const void* stack, int elem_bytes, int n, int rows, int cols, int full, int nwords,
                  uint32_t* out) {
    return elem_bytes == 1 ? transform_in<uint8_t>(stack, elem_bytes, n, rows, cols, full, nwords, out)
                           : transform_in<uint16_t>(stack, elem_bytes, n, rows, cols, full, nwords, out);
}

int ref_search(const uint32_t* d0, const uint32_t* d1, int rows, int cols, int nwords, int flags,
               int max_lr_diff, int16_t* out) {
    switch (nwords) {
        case 1: search_d<uint32_t>(d0, d1, rows, cols, nwords, flags, max_lr_diff, out); break;
        case 2: search_d<uint64_t>(d0, d1, rows, cols, nwords, flags, max_lr_diff, out); break;
        case 4: search_d<uint128_t>(d0, d1, rows, cols, nwords, flags, max_lr_diff, out); break;
        case 8: search_d<std::bitset<256>>(d0, d1, rows, cols, nwords, flags, max_lr_diff, out); break;
        default: return ORC_ERR_INVALID_ARGUMENT;
    }
    return ORC_OK;
}

int ref_agree(int16_t* disp, const void* s0, const void* s1, int elem_bytes, int n, int rows, int cols,
              float thr, int has_minvar, float minvar, float* corr) {
    cv::Mat l, r;
    cv::merge(planes_of(s0, elem_bytes, n, rows, cols), l);
    cv::merge(planes_of(s1, elem_bytes, n, rows, cols), r);
    cv::Mat d(rows, cols, CV_16SC1, disp);
    cv::Mat c;
    if (corr) {
        c = cv::Mat(rows, cols, CV_32FC1, corr);
        c.setTo(std::numeric_limits<float>::quiet_NaN());
    }
    std::optional<float> mv = has_minvar ? std::optional<float>(minvar) : std::nullopt;
    if (elem_bytes == 1)
        cpu::agree<uint8_t>(d, l, r, n, thr, mv, corr ? &c : nullptr);
    else
        cpu::agree<uint16_t>(d, l, r, n, thr, mv, corr ? &c : nullptr);
    return ORC_OK;
}

int ref_agree_subpixel(const int16_t* disp, const void* s0, const void* s1, int elem_bytes, int n, int rows,
                       int cols, float thr, float step, int has_minvar, float minvar, float* out, float* corr) {
    cv::Mat l, r;
    cv::merge(planes_of(s0, elem_bytes, n, rows, cols), l);
    cv::merge(planes_of(s1, elem_bytes, n, rows, cols), r);
    cv::Mat1s d(cv::Mat(rows, cols, CV_16SC1, (void*)disp));
    cv::Mat c;
    if (corr) {
        c = cv::Mat(rows, cols, CV_32FC1, corr);
        c.setTo(std::numeric_limits<float>::quiet_NaN());
    }
    cv::Mat o;
    std::optional<float> mv = has_minvar ? std::optional<float>(minvar) : std::nullopt;
    if (elem_bytes == 1)
        cpu::agree_subpixel<uint8_t>(d, l, r, n, thr, step, mv, o, corr ? &c : nullptr);
    else
        cpu::agree_subpixel<uint16_t>(d, l, r, n, thr, step, mv, o, corr ? &c : nullptr);
    for (int i = 0; i < rows; ++i)
        std::memcpy(out + (size_t)i * cols, o.ptr<float>(i), cols * sizeof(float));
    return ORC_OK;
}

int ref_match(const void* s0, const void* s1, int elem_bytes, int n, int rows, int cols, const orc_config* cfg,
              void* disp_out, void* corr_out, char* err, int errlen) {
    try {
        if (cfg->precision != 0) {
            std::snprintf(err, errlen, "the reference CPU backend computes in single precision only");
            return ORC_ERR_INVALID_ARGUMENT;
        }
        Config c;
        c.nxcorr_threshold = cfg->has_threshold ? std::optional<float>(cfg->nxcorr_threshold) : std::nullopt;
        c.subpixel_step = cfg->has_subpixel_step ? std::optional<float>(cfg->subpixel_step) : std::nullopt;
        c.min_variance = cfg->has_min_variance ? std::optional<float>(cfg->min_variance) : std::nullopt;
        c.mode = cfg->mode ? TransformMode::FULL : TransformMode::LIMITED;
        if (cfg->variant == 1)
            c.variant = Variant::Consistency {cfg->max_lr_diff, cfg->no_dupes != 0};
        else
            c.variant = Variant::NoDuplicates {};
        cv::Mat disp, corr;
        impl::cpu::match(planes_of(s0, elem_bytes, n, rows, cols), planes_of(s1, elem_bytes, n, rows, cols),
                         disp, c, corr_out ? &corr : nullptr);
        const size_t eb = disp.type() == CV_16SC1 ? 2 : 4;
        for (int i = 0; i < rows; ++i)
            std::memcpy((uint8_t*)disp_out + (size_t)i * cols * eb, disp.ptr<uint8_t>(i), cols * eb);
        if (corr_out && !corr.empty())
            for (int i = 0; i < rows; ++i)
                std::memcpy((uint8_t*)corr_out + (size_t)i * cols * 4, corr.ptr<uint8_t>(i), cols * 4);
        return ORC_OK;
    } catch (const std::invalid_argument& e) {
        std::snprintf(err, errlen, "%s", e.what());
        return ORC_ERR_INVALID_ARGUMENT;
    } catch (const std::exception& e) {
        std::snprintf(err, errlen, "%s", e.what());
        return ORC_ERR_EXCEPTION;
    }
}

} // extern "C"
