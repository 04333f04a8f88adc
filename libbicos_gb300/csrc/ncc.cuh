// Per-pixel NCC helpers shared by the agreement kernels (agree.cu) and the
// learned subpixel kernel (learned.cu).  Arithmetic follows libBICOS
// include/impl/cuda/agree.cuh:35-97 (nxcorrd / nxcorrf) with explicit IEEE
// round-to-nearest intrinsics in the reference's order.
#pragma once

#include "kernels.cuh"

namespace bicos_gb300 {

template<typename T>
__device__ __forceinline__ int ld_px(const StackParams& p, int side, int t, int row, int col) {
    const T* r = reinterpret_cast<const T*>(p.frame[side][t] + (long long)row * p.pitch[side][t]);
    return (int)__ldg(r + col);
}

template<bool DBL>
struct Prec;
template<>
struct Prec<false> {
    using T = float;
};
template<>
struct Prec<true> {
    using T = double;
};

// (T)__float2int_rn(v): round half to even, wrap modulo 2^bits
template<typename T>
__device__ __forceinline__ int round_wrap(float v) {
    return (int)(T)__float2int_rn(v);
}

// The reference NCC of the left pixel against the right column col1 (QUAD
// false) or against the rounded interpolants of columns col1-1..col1+1 at
// x (QUAD true), streamed over the frames twice instead of held in
// registers: the same operations in the same order as nxc_full, so the same
// result (each accumulator still runs in frame order).
template<typename T, bool DBL, bool QUAD>
__device__ __forceinline__ typename Prec<DBL>::T nxc_stream(const StackParams& s, int row, int col, int col1,
                                                             float x, bool mv, float minvar) {
    using TP = typename Prec<DBL>::T;
    const int n = s.n;
    auto right = [&](int t) -> int {
        if constexpr (QUAD) {
            const int y0 = ld_px<T>(s, 1, t, row, col1 - 1);
            const int y1 = ld_px<T>(s, 1, t, row, col1);
            const int y2 = ld_px<T>(s, 1, t, row, col1 + 1);
            const float a = 0.5f * (float)(y0 - 2 * y1 + y2), b = 0.5f * (float)(y2 - y0), c = (float)y1;
            return round_wrap<T>(__fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(a, x), x), __fmul_rn(b, x)), c));
        } else {
            return ld_px<T>(s, 1, t, row, col1);
        }
    };
    int sx = 0, sy = 0;
    for (int t = 0; t < n; ++t) {
        sx += ld_px<T>(s, 0, t, row, col);
        sy += right(t);
    }
    TP cov = 0, var0 = 0, var1 = 0;
    if constexpr (DBL) {
        const double m0 = __ddiv_rn((double)sx, (double)n), m1 = __ddiv_rn((double)sy, (double)n);
        for (int t = 0; t < n; ++t) {
            const double d0 = __dsub_rn((double)ld_px<T>(s, 0, t, row, col), m0);
            const double d1 = __dsub_rn((double)right(t), m1);
            var0 = __fma_rn(d0, d0, var0);
            cov = __fma_rn(d0, d1, cov);
            var1 = __fma_rn(d1, d1, var1);
        }
        if (mv && (var0 < (double)minvar || var1 < (double)minvar))
            return -1.0;
        return __ddiv_rn(cov, __dsqrt_rn(__dmul_rn(var0, var1)));
    } else {
        const float m0 = __fdiv_rn((float)sx, (float)n), m1 = __fdiv_rn((float)sy, (float)n);
        for (int t = 0; t < n; ++t) {
            const float d0 = __fsub_rn((float)ld_px<T>(s, 0, t, row, col), m0);
            const float d1 = __fsub_rn((float)right(t), m1);
            var0 = __fmaf_rn(d0, d0, var0);
            cov = __fmaf_rn(d0, d1, cov);
            var1 = __fmaf_rn(d1, d1, var1);
        }
        if (mv && (var0 < minvar || var1 < minvar))
            return -1.f;
        return __fdiv_rn(cov, __fsqrt_rn(__fmul_rn(var0, var1)));
    }
}

}  // namespace bicos_gb300
