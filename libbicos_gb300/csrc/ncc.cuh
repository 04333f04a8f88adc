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

// float(v) for |v| < 2^22 without a conversion instruction: v added into the
// mantissa of 1.5 * 2^23, the constant subtracted again (both exact)
__device__ __forceinline__ float small_int_to_float(int v) {
    return __fsub_rn(__int_as_float(0x4B400000 + v), 12582912.0f);
}

// (int)(T)__float2int_rn(q) for |q| < 2^22: q + 1.5 * 2^23 rounds to an
// integer half to even, whose low mantissa bits are the wrapped value
template<typename T>
__device__ __forceinline__ int round_wrap_bits(float q) {
    constexpr uint32_t kMask = sizeof(T) == 1 ? 0xFFu : 0xFFFFu;
    return (int)(__float_as_uint(__fadd_rn(q, 12582912.0f)) & kMask);
}

// the same as a float
template<typename T>
__device__ __forceinline__ float round_wrap_f(float q) {
    constexpr uint32_t kMask = sizeof(T) == 1 ? 0xFFu : 0xFFFFu;
    const float f = __fadd_rn(q, 12582912.0f);
    return __fsub_rn(__uint_as_float((__float_as_uint(f) & kMask) | 0x4B000000u), 8388608.0f);
}

// Row accessors: sample of frame t at column c of one image row, left or
// right side, from global memory or from a copy in shared memory.
template<typename T>
struct GlobalRow {
    const StackParams* s;
    int row;
    __device__ __forceinline__ int left(int t, int c) const { return ld_px<T>(*s, 0, t, row, c); }
    __device__ __forceinline__ int right(int t, int c) const { return ld_px<T>(*s, 1, t, row, c); }
};

// frame t of the left copy at L + t * lstride (elements) starting at column
// l0; the right copy likewise
template<typename T>
struct SharedRow {
    const T* L;
    const T* R;
    int lstride, rstride, l0, r0;
    __device__ __forceinline__ int left(int t, int c) const { return (int)L[t * lstride + (c - l0)]; }
    __device__ __forceinline__ int right(int t, int c) const { return (int)R[t * rstride + (c - r0)]; }
};

// The reference NCC of the left pixel against the right column col1 (QUAD
// false) or against the rounded interpolants of columns col1-1..col1+1 at
// x (QUAD true), streamed over the frames twice instead of held in
// registers: the same operations in the same order as nxc_full, so the same
// result (each accumulator still runs in frame order).
template<typename T, bool DBL, bool QUAD, typename Row>
__device__ __forceinline__ typename Prec<DBL>::T nxc_row(const Row& src, int n, int col, int col1, float x, bool mv,
                                                          float minvar) {
    using TP = typename Prec<DBL>::T;
    auto right = [&](int t) -> int {
        if constexpr (QUAD) {
            const int y0 = src.right(t, col1 - 1);
            const int y1 = src.right(t, col1);
            const int y2 = src.right(t, col1 + 1);
            const float a = 0.5f * (float)(y0 - 2 * y1 + y2), b = 0.5f * (float)(y2 - y0), c = (float)y1;
            return round_wrap<T>(__fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(a, x), x), __fmul_rn(b, x)), c));
        } else {
            return src.right(t, col1);
        }
    };
    int sx = 0, sy = 0;
    for (int t = 0; t < n; ++t) {
        sx += src.left(t, col);
        sy += right(t);
    }
    TP cov = 0, var0 = 0, var1 = 0;
    if constexpr (DBL) {
        const double m0 = __ddiv_rn((double)sx, (double)n), m1 = __ddiv_rn((double)sy, (double)n);
        for (int t = 0; t < n; ++t) {
            const double d0 = __dsub_rn((double)src.left(t, col), m0);
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
            const float d0 = __fsub_rn((float)src.left(t, col), m0);
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

template<typename T, bool DBL, bool QUAD>
__device__ __forceinline__ typename Prec<DBL>::T nxc_stream(const StackParams& s, int row, int col, int col1,
                                                             float x, bool mv, float minvar) {
    return nxc_row<T, DBL, QUAD>(GlobalRow<T>{&s, row}, s.n, col, col1, x, mv, minvar);
}

}  // namespace bicos_gb300
