// bicos_gb300 C++ API: the types of libBICOS's public header, GB300 build.
//
// Drop-in counterpart of libBICOS include/common.hpp:30-92 (Config, enums,
// Variant, INVALID_DISP, is_invalid, Exception) with Precision always
// present, as in the reference's CUDA build.  `Image` replaces
// cv::cuda::GpuMat: the same header layout (data, step, rows, cols, type)
// over device memory, without an OpenCV dependency.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <exception>
#include <limits>
#include <memory>
#include <optional>
#include <string>
#include <type_traits>
#include <variant>
#include <vector>

struct CUstream_st;

namespace BICOS {

using uint128_t = __uint128_t;

template<typename T>
constexpr T INVALID_DISP = std::numeric_limits<T>::has_quiet_NaN ? std::numeric_limits<T>::quiet_NaN()
                                                                 : std::numeric_limits<T>::lowest();

template<typename T>
constexpr bool is_invalid(T disparity) {
    if constexpr (std::is_floating_point_v<T>)
        return std::isnan(disparity);
    else
        return disparity == INVALID_DISP<T>;
}

enum class TransformMode { LIMITED, FULL };
enum class Precision { SINGLE, DOUBLE };

namespace Variant {
    struct NoDuplicates {};
    struct Consistency {
        int max_lr_diff = 1;
        bool no_dupes = false;
    };
}  // namespace Variant

using SearchVariant = std::variant<Variant::NoDuplicates, Variant::Consistency>;

struct Config {
    std::optional<float> nxcorr_threshold = 0.5f;
    std::optional<float> subpixel_step = std::nullopt;
    std::optional<float> min_variance = std::nullopt;
    TransformMode mode = TransformMode::LIMITED;
    Precision precision = Precision::SINGLE;
    SearchVariant variant = Variant::NoDuplicates {};
};

class Exception: public std::exception {
    std::string _message;

public:
    Exception(const std::string& message);
    const char* what() const throw() override;
};

// element type codes, as OpenCV's CV_8UC1 ... CV_64FC1
enum ImageType { IMG_8U = 0, IMG_16U = 2, IMG_16S = 3, IMG_32F = 5, IMG_64F = 6 };

using Stream = CUstream_st*;

// A pitched 2-D device image (cv::cuda::GpuMat's header layout).  Owning
// when made by create() (cudaMallocPitch, freed with the last copy),
// borrowing when built over external device memory.
class Image {
public:
    void* data = nullptr;
    size_t step = 0;
    int rows = 0;
    int cols = 0;

    Image() = default;
    Image(int rows, int cols, int type);
    Image(int rows, int cols, int type, void* data, size_t step);

    void create(int rows, int cols, int type);
    void release();
    int type() const { return _type; }
    int depth() const { return _type; }
    size_t elemSize() const;
    bool empty() const { return data == nullptr || rows == 0 || cols == 0; }

    void upload(const void* host, size_t host_step, Stream stream = nullptr);
    void download(void* host, size_t host_step, Stream stream = nullptr) const;

private:
    int _type = IMG_8U;
    std::shared_ptr<void> _owner;
};

}  // namespace BICOS
