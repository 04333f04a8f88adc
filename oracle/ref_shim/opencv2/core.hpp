// Minimal stand-in for the handful of OpenCV core symbols that libBICOS's
// CPU backend uses (cv::Mat, Mat_, Mat1s, Size, Range, DataType, merge,
// parallel_for_).  TEST INFRASTRUCTURE ONLY: it exists so the reference's
// own CPU sources compile unmodified into the oracle/_ref checker library.
// Written from the documented OpenCV semantics of those calls; only the
// behaviour the reference relies on is provided.
#pragma once

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <memory>
#include <stdexcept>
#include <sys/types.h>
#include <atomic>
#include <thread>
#include <vector>

#define CV_8U 0
#define CV_8S 1
#define CV_16U 2
#define CV_16S 3
#define CV_32S 4
#define CV_32F 5
#define CV_64F 6
#define CV_CN_SHIFT 3
#define CV_DEPTH_MASK 7
#define CV_MAKETYPE(depth, cn) (((depth) & CV_DEPTH_MASK) + (((cn) - 1) << CV_CN_SHIFT))
#define CV_8UC1 CV_MAKETYPE(CV_8U, 1)
#define CV_16UC1 CV_MAKETYPE(CV_16U, 1)
#define CV_16SC1 CV_MAKETYPE(CV_16S, 1)
#define CV_32FC1 CV_MAKETYPE(CV_32F, 1)
#define CV_64FC1 CV_MAKETYPE(CV_64F, 1)

namespace cv {

struct Size {
    int width = 0, height = 0;
    Size() = default;
    Size(int w, int h): width(w), height(h) {}
    size_t area() const { return (size_t)width * (size_t)height; }
    bool operator==(const Size& o) const { return width == o.width && height == o.height; }
    bool operator!=(const Size& o) const { return !(*this == o); }
};

struct Range {
    int start = 0, end = 0;
    Range() = default;
    Range(int s, int e): start(s), end(e) {}
};

template<typename T> struct DataType;
template<> struct DataType<uint8_t> { enum { type = CV_8UC1, depth = CV_8U }; };
template<> struct DataType<uint16_t> { enum { type = CV_16UC1, depth = CV_16U }; };
template<> struct DataType<int16_t> { enum { type = CV_16SC1, depth = CV_16S }; };
template<> struct DataType<float> { enum { type = CV_32FC1, depth = CV_32F }; };
template<> struct DataType<double> { enum { type = CV_64FC1, depth = CV_64F }; };

inline size_t depth_bytes(int depth) {
    static const size_t sz[] = {1, 1, 2, 2, 4, 4, 8, 2};
    return sz[depth & CV_DEPTH_MASK];
}

// 2-D matrix header over a shared, refcounted buffer (row pitch `step`).
class Mat {
public:
    int rows = 0, cols = 0;
    uint8_t* data = nullptr;
    size_t step = 0;

    Mat() = default;
    Mat(Size sz, int type) { create(sz, type); }
    Mat(int r, int c, int type) { create(Size(c, r), type); }
    Mat(int r, int c, int type, void* ext, size_t st = 0)
        : rows(r), cols(c), data((uint8_t*)ext), _type(type) {
        step = st ? st : (size_t)c * elemSize();
    }
    virtual ~Mat() = default;

    int type() const { return _type; }
    int depth() const { return _type & CV_DEPTH_MASK; }
    int channels() const { return (_type >> CV_CN_SHIFT) + 1; }
    size_t elemSize() const { return depth_bytes(depth()) * channels(); }
    Size size() const { return Size(cols, rows); }
    bool empty() const { return data == nullptr || rows == 0 || cols == 0; }

    void create(Size sz, int type) {
        if (data && sz.width == cols && sz.height == rows && type == _type)
            return;
        _type = type;
        rows = sz.height;
        cols = sz.width;
        step = (size_t)cols * elemSize();
        _buf = std::shared_ptr<uint8_t>(new uint8_t[step * rows + 1], std::default_delete<uint8_t[]>());
        data = _buf.get();
    }

    template<typename V>
    Mat& setTo(V value) {
        for (int r = 0; r < rows; ++r) {
            uint8_t* p = data + r * step;
            switch (depth()) {
                case CV_8U: fill_row<uint8_t>(p, value); break;
                case CV_16U: fill_row<uint16_t>(p, value); break;
                case CV_16S: fill_row<int16_t>(p, value); break;
                case CV_32F: fill_row<float>(p, value); break;
                case CV_64F: fill_row<double>(p, value); break;
                default: throw std::runtime_error("setTo: unsupported depth");
            }
        }
        return *this;
    }

    Mat row(int r) const {
        Mat m(*this);
        m.rows = 1;
        m.data = data + (size_t)r * step;
        return m;
    }

    template<typename T> T* ptr(int r = 0) { return (T*)(data + (size_t)r * step); }
    template<typename T> const T* ptr(int r = 0) const { return (const T*)(data + (size_t)r * step); }
    template<typename T> T* ptr(int r, int c) { return (T*)(data + (size_t)r * step + (size_t)c * elemSize()); }
    template<typename T> const T* ptr(int r, int c) const {
        return (const T*)(data + (size_t)r * step + (size_t)c * elemSize());
    }
    template<typename T> T& at(int r, int c) { return *ptr<T>(r, c); }
    template<typename T> const T& at(int r, int c) const { return *ptr<T>(r, c); }
    // single index: along the row of a one-row matrix, else down the column
    template<typename T> T& at(int i) { return rows == 1 ? *ptr<T>(0, i) : *ptr<T>(i, 0); }
    template<typename T> const T& at(int i) const { return rows == 1 ? *ptr<T>(0, i) : *ptr<T>(i, 0); }

protected:
    int _type = CV_8UC1;
    std::shared_ptr<uint8_t> _buf;

    template<typename T, typename V>
    void fill_row(uint8_t* p, V value) {
        T* q = (T*)p;
        const size_t cnt = (size_t)cols * channels();
        for (size_t i = 0; i < cnt; ++i)
            q[i] = (T)value;
    }
};

template<typename T>
class Mat_: public Mat {
public:
    Mat_() { _type = DataType<T>::type; }
    Mat_(Size sz) { create(sz, DataType<T>::type); }
    Mat_(const Mat& m): Mat(m) {
        if (!m.empty() && m.type() != DataType<T>::type)
            throw std::runtime_error("Mat_: type mismatch");
        _type = DataType<T>::type;
    }
    Mat_& operator=(const Mat& m) {
        Mat::operator=(m);
        _type = DataType<T>::type;
        return *this;
    }
    T& at(int i) { return Mat::at<T>(i); }
    const T& at(int i) const { return Mat::at<T>(i); }
    template<typename U> U& at(int i) { return Mat::at<U>(i); }
    template<typename U> const U& at(int i) const { return Mat::at<U>(i); }
    template<typename U> U& at(int r, int c) { return Mat::at<U>(r, c); }
    template<typename U> const U& at(int r, int c) const { return Mat::at<U>(r, c); }
};

using Mat1s = Mat_<int16_t>;

// channel interleave: out(r, c)[k] = planes[k](r, c)
inline void merge(const std::vector<Mat>& planes, Mat& out) {
    if (planes.empty())
        throw std::runtime_error("merge: no planes");
    const int cn = (int)planes.size();
    const int depth = planes[0].depth();
    const size_t eb = depth_bytes(depth);
    Mat m(planes[0].size(), CV_MAKETYPE(depth, cn));
    if (cn > 512)
        throw std::runtime_error("merge: too many planes");
    for (int r = 0; r < m.rows; ++r)
        for (int c = 0; c < m.cols; ++c)
            for (int k = 0; k < cn; ++k)
                std::memcpy(m.ptr<uint8_t>(r, c) + k * eb, planes[k].ptr<uint8_t>(r) + c * eb, eb);
    out = m;
}

// Parallel loop over all hardware threads that hands the body one index at
// a time, as OpenCV's stripes do for row loops: the reference's bodies
// allocate per-pixel scratch on the stack (alloca), released only when the
// body returns, so a body call must not span many image rows.
inline void parallel_for_(const Range& range, const std::function<void(const Range&)>& body) {
    const int total = range.end - range.start;
    if (total <= 0)
        return;
    int nt = (int)std::thread::hardware_concurrency();
    if (nt < 1)
        nt = 1;
    if (nt > total)
        nt = total;
    std::atomic<int> next(range.start);
    std::vector<std::thread> pool;
    for (int i = 0; i < nt; ++i)
        pool.emplace_back([&]() {
            for (int r = next++; r < range.end; r = next++)
                body(Range(r, r + 1));
        });
    for (auto& t: pool)
        t.join();
}

} // namespace cv
