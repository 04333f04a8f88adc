// OpenCV adapter for BICOS::match: libBICOS include/match.hpp:30-40 with
// its CUDA build's types (cv::cuda::GpuMat images, cv::cuda::Stream&),
// header-only and active only when OpenCV's CUDA core headers are on the
// include path, so a caller of the reference's CUDA build keeps its call:
//
//     #include <BICOS/opencv.hpp>
//     BICOS::match(stack0, stack1, disparity, cfg, &corrmap, stream);
//
// The GpuMats are wrapped without copies.  `disparity` (and `corrmap`) are
// created with the output type first -- CV_16SC1, or CV_32FC1 with a
// subpixel step; the corrmap CV_32FC1 or CV_64FC1 by precision -- so the
// library writes straight into them (an Image over memory of the right
// size and type is not reallocated).  Asynchronous on `stream`, as the
// rest of this API.
#pragma once

#include "match.hpp"

#if defined(__has_include)
#if __has_include(<opencv2/core/cuda.hpp>) && __has_include(<opencv2/core/cuda_stream_accessor.hpp>)
#define BICOS_HAVE_OPENCV_CUDA 1
#endif
#endif

#ifdef BICOS_HAVE_OPENCV_CUDA
#include <opencv2/core/cuda.hpp>
#include <opencv2/core/cuda_stream_accessor.hpp>

namespace BICOS {

// a borrowing Image over a single-channel GpuMat (OpenCV's depth codes are
// the ImageType codes)
inline Image view(const cv::cuda::GpuMat& m) {
    if (m.channels() != 1)
        throw Exception("single-channel images only");
    return Image(m.rows, m.cols, m.depth(), m.data, m.step);
}

inline void match(const std::vector<cv::cuda::GpuMat>& stack0, const std::vector<cv::cuda::GpuMat>& stack1,
                  cv::cuda::GpuMat& disparity, Config cfg = Config {}, cv::cuda::GpuMat* corrmap = nullptr,
                  cv::cuda::Stream& stream = cv::cuda::Stream::Null()) {
    std::vector<Image> s0, s1;
    s0.reserve(stack0.size());
    s1.reserve(stack1.size());
    for (const cv::cuda::GpuMat& m : stack0)
        s0.push_back(view(m));
    for (const cv::cuda::GpuMat& m : stack1)
        s1.push_back(view(m));
    Image d, c;
    if (!stack0.empty()) {
        const int rows = stack0[0].rows, cols = stack0[0].cols;
        disparity.create(rows, cols, cfg.subpixel_step.has_value() ? CV_32FC1 : CV_16SC1);
        d = view(disparity);
        if (corrmap && cfg.nxcorr_threshold.has_value()) {
            corrmap->create(rows, cols, cfg.precision == Precision::SINGLE ? CV_32FC1 : CV_64FC1);
            c = view(*corrmap);
        }
    }
    match(s0, s1, d, cfg, corrmap ? &c : nullptr, cv::cuda::StreamAccessor::getStream(stream));
}

}  // namespace BICOS

#endif  // BICOS_HAVE_OPENCV_CUDA
