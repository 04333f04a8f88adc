// Moment form of the NCC stage: the "precision form" (no counterpart in
// libBICOS; an alternative to the two-pass NCC of
// include/impl/cuda/agree.cuh:35-259).
//
// For a left pixel (col) matched to right column col1, with x_t the left
// and y_t(j) the right samples at col1+j, everything the agreement needs
// follows from exact integer moments:
//   Sx = sum x, Sxx = sum x^2, Sy[j] = sum y(j), Sxy[j] = sum x y(j),
//   Syy[j][k] = sum y(j) y(k),                              j, k in -2..2.
// The Sxy band of a row is formed on the tensor cores: one CTA stages its
// 128 left pixels and a 64-column right window as FP16 rows in shared
// memory and runs tcgen05.mma kind::f16 (FP32 accumulation) into TMEM;
// every product is an integer below 2^16 and every sum below 2^24, so the
// FP32 results are exact for 8-bit stacks (n <= 65).  12-bit data is split
// into 6-bit halves, x = 64 xh + xl: Sxy = 4096 (xh.yh) + 64 (xh.yl +
// xl.yh) + xl.yl from three accumulators, exact for samples below 4096;
// wider 16-bit samples give xh up to 1023, whose sums can pass 2^24, so a
// tile that stages such a sample uses SIMT dot products (the same
// integers), as do tiles whose disparities spread wider than the window.
//
// Leaving the sweep's quadratic interpolant unrounded, I(x) = a x^2 + b x + c
// (a, b, c from y at col1-1, col1, col1+1), the sweep correlation is
// rho(x) = P(x) / sqrt(V0 Q(x)) with
//   V0   = n Sxx - Sx^2,
//   P(x) = 2 n cov(x)  = P2 x^2 + P1 x + P0,
//   Q(x) = 4 n var1(x) = Q4 x^4 + Q3 x^3 + Q2 x^2 + Q1 x + Q0,
// all coefficients exact int64, so every cross term (the mu_x mu_y
// subtractions) is exact, and floating point (FP64 for precision double,
// else FP32) only evaluates the polynomials (Horner, fused multiply-add)
// and the ratio.  Sweep positions are the reference's float-accumulated
// x = -1, -1+step, ... <= 1; the best is the first strictly largest.  The
// results differ from the reference's, whose interpolants are rounded to
// integers: that difference is measured against the FP64 restatement of
// the reference in the test suite.
#include <cuda_fp16.h>
#include <math.h>

#include <type_traits>

#include "kernels.cuh"
#include "tcgen05.cuh"

namespace bicos_gb300 {

__device__ unsigned int g_mom_faults = 0;

namespace {

using namespace tc;

constexpr int kRowsM = 128;  // left pixels per CTA (MMA M)
constexpr int kWin = 64;     // right window (MMA N)
constexpr int kR = 2;        // offsets -kR..kR around col1
constexpr int kNOff = 2 * kR + 1;
constexpr int kNPair = kNOff * (kNOff + 1) / 2;
constexpr int kScratch = 65;  // padded row of the TMEM read-back scratch

__device__ __forceinline__ int pair_index(int j, int k) {  // j <= k, in 0..kNOff-1
    return j * kNOff - j * (j - 1) / 2 + (k - j);
}

template<typename T>
__device__ __forceinline__ int ld_px(const StackParams& p, int side, int t, int row, int col) {
    const T* r = reinterpret_cast<const T*>(p.frame[side][t] + (long long)row * p.pitch[side][t]);
    return (int)__ldg(r + col);
}

// frames t0..t0+7 of one pixel as FP16: the value (8-bit) or a 6-bit half
template<typename T, int PART>
__device__ __forceinline__ uint4 pack8(const StackParams& p, int side, int row, int col, int t0) {
    uint32_t w[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        float v[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int t = t0 + 2 * i + h;
            int x = (col >= 0 && t < p.n) ? ld_px<T>(p, side, t, row, col) : 0;
            if constexpr (sizeof(T) == 2)
                x = PART == 0 ? (x >> 6) : (x & 63);
            v[h] = (float)x;
        }
        const __half2 hv = __floats2half2_rn(v[0], v[1]);
        w[i] = *reinterpret_cast<const uint32_t*>(&hv);
    }
    return make_uint4(w[0], w[1], w[2], w[3]);
}

struct MomShared {
    uint64_t mbar;
    uint32_t tmem;
    int abort;
    int cmin, cmax;
    int big;  // 16-bit stacks: a staged sample of 4096 or more
};

template<bool DBL>
struct FT;
template<>
struct FT<false> {
    using T = float;
    __device__ static float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
    __device__ static float ratio(float p, float v0, float q) { return __fdiv_rn(p, __fsqrt_rn(__fmul_rn(v0, q))); }
};
template<>
struct FT<true> {
    using T = double;
    __device__ static double fma(double a, double b, double c) { return __fma_rn(a, b, c); }
    __device__ static double ratio(double p, double v0, double q) {
        return __ddiv_rn(p, __dsqrt_rn(__dmul_rn(v0, q)));
    }
};

// mode 0: agree at the integer disparity (int16 out, in place semantics)
// mode 1: subpixel sweep (float out)
// mode 2: learned-subpixel features (rho at col1-2..col1+2, variances)
template<typename T, int KSTEPS, bool DBL, int MODE>
__global__ void __launch_bounds__(kRowsM) k_moments(const __grid_constant__ MomentParams p) {
    using F = FT<DBL>;
    using R = typename F::T;
    constexpr int PARTS = sizeof(T) == 2 ? 2 : 1;
    constexpr int NACC = sizeof(T) == 2 ? 3 : 1;
    constexpr int KB = KSTEPS * 32;  // bytes per row: 16 FP16 values per K step
    constexpr int A_BYTES = kRowsM * KB, B_BYTES = kWin * KB;
    constexpr uint32_t kAChunk = kRowsM * 16, kBChunk = kWin * 16;
    constexpr uint32_t kTmemCols = NACC == 1 ? 64 : 256;
    extern __shared__ __align__(1024) uint8_t smem[];
    float* scratch = reinterpret_cast<float*>(smem + PARTS * (A_BYTES + B_BYTES));
    __shared__ MomShared sh;

    const int tid = threadIdx.x, warp = tid >> 5;
    const int row = blockIdx.y, col = blockIdx.x * kRowsM + tid;
    const int n = p.s.n, cols = p.s.cols;
    const bool in = col < cols;

    int16_t d = kInvalidDisp;
    if (in)
        d = reinterpret_cast<const int16_t*>(reinterpret_cast<const char*>(p.raw) + row * p.raw_pitch)[col];
    const int col1 = col - d;
    const bool valid = in && d != kInvalidDisp && col1 >= 0 && col1 < cols;

    if (warp == 0) {
        tmem_alloc(smem_u32(&sh.tmem), kTmemCols);
        tmem_relinquish();
    }
    if (tid == 0) {
        mbar_init(smem_u32(&sh.mbar), 1);
        sh.abort = 0;
        sh.cmin = 0x7fffffff;
        sh.cmax = -0x7fffffff;
        sh.big = 0;
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (valid) {
        atomicMin(&sh.cmin, col1);
        atomicMax(&sh.cmax, col1);
    }
    __syncthreads();
    const int wlo = sh.cmin - kR;
    bool use_tc = sh.cmax >= sh.cmin && sh.cmax + kR - wlo < kWin;
    if constexpr (sizeof(T) == 2) {
        // the 6+6-bit split is exact only for samples below 4096 (the high
        // parts' products summed over the frames stay below 2^24); a tile
        // that stages a larger one takes the exact SIMT sums instead
        if (use_tc) {
            bool big = false;
            for (int t = 0; t < n; ++t) {
                if (valid)
                    big |= ld_px<T>(p.s, 0, t, row, col) >= 4096;
                if (tid < kWin && wlo + tid >= 0 && wlo + tid < cols)
                    big |= ld_px<T>(p.s, 1, t, row, wlo + tid) >= 4096;
            }
            if (big)
                atomicOr(&sh.big, 1);
        }
        __syncthreads();
        use_tc = use_tc && !sh.big;
    }

    long long sxy[kNOff];
#pragma unroll
    for (int j = 0; j < kNOff; ++j)
        sxy[j] = 0;
    bool ok = true;
    if (use_tc) {
#pragma unroll
        for (int part = 0; part < PARTS; ++part) {
            uint8_t* A = smem + part * A_BYTES;
            uint8_t* B = smem + PARTS * A_BYTES + part * B_BYTES;
            for (int kc = 0; kc < 2 * KSTEPS; ++kc) {
                const int lc = valid ? col : -1;
                *reinterpret_cast<uint4*>(A + kc * kAChunk + (tid >> 3) * 128 + (tid & 7) * 16) =
                    part == 0 ? pack8<T, 0>(p.s, 0, row, lc, 8 * kc) : pack8<T, 1>(p.s, 0, row, lc, 8 * kc);
                if (tid < kWin) {
                    const int c = wlo + tid;
                    const int rc = (c >= 0 && c < cols) ? c : -1;
                    *reinterpret_cast<uint4*>(B + kc * kBChunk + (tid >> 3) * 128 + (tid & 7) * 16) =
                        part == 0 ? pack8<T, 0>(p.s, 1, row, rc, 8 * kc) : pack8<T, 1>(p.s, 1, row, rc, 8 * kc);
                }
            }
        }
        fence_async_smem();
        fence_before();
        __syncthreads();
        if (tid == 0) {
            fence_after();
            constexpr uint32_t idesc = idesc_f16(kRowsM, kWin);
            const uint32_t a0 = smem_u32(smem), b0 = smem_u32(smem + PARTS * A_BYTES);
            auto chain = [&](uint32_t acc, uint32_t abase, uint32_t bbase, bool first) {
#pragma unroll
                for (int s = 0; s < KSTEPS; ++s)
                    mma_f16(sh.tmem + acc, smem_desc(abase + s * 2 * kAChunk, kAChunk, 128),
                            smem_desc(bbase + s * 2 * kBChunk, kBChunk, 128), idesc,
                            (!first || s > 0) ? 1u : 0u);
            };
            chain(0, a0, b0, true);                        // x . y   (8-bit) / xh . yh
            if constexpr (PARTS == 2) {
                chain(kWin, a0, b0 + B_BYTES, true);       // xh . yl
                chain(kWin, a0 + A_BYTES, b0, false);      //   + xl . yh
                chain(2 * kWin, a0 + A_BYTES, b0 + B_BYTES, true);  // xl . yl
            }
            mma_commit(smem_u32(&sh.mbar));
        }
        ok = __syncthreads_and(wait_or_abort(smem_u32(&sh.mbar), 0, &sh.abort));
        if (ok) {
            fence_after();
            const int j0 = col1 - kR - wlo;  // this pixel's first window column
#pragma unroll
            for (int acc = 0; acc < NACC; ++acc) {
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    float v[32];
                    tmem_ld32(sh.tmem + ((uint32_t)(warp * 32) << 16) + acc * kWin + h * 32, v);
#pragma unroll
                    for (int k = 0; k < 32; ++k)
                        scratch[tid * kScratch + h * 32 + k] = v[k];
                }
                const long long w = NACC == 1 ? 1 : (acc == 0 ? 4096 : acc == 1 ? 64 : 1);
                if (valid)
#pragma unroll
                    for (int j = 0; j < kNOff; ++j)
                        sxy[j] += w * (long long)__float2ll_rn(scratch[tid * kScratch + j0 + j]);
            }
        }
    } else if (valid) {
        for (int t = 0; t < n; ++t) {
            const int x = ld_px<T>(p.s, 0, t, row, col);
#pragma unroll
            for (int j = 0; j < kNOff; ++j) {
                const int c = col1 + j - kR;
                if (c >= 0 && c < cols)
                    sxy[j] += (long long)x * ld_px<T>(p.s, 1, t, row, c);
            }
        }
    }

    // exact SIMT moments of the left pixel and the right columns: 8-bit
    // samples accumulate in 32 bits (n * 255^2 < 2^31 for n <= 65), 16-bit
    // ones in 64
    using Acc = typename std::conditional<sizeof(T) == 1, int, long long>::type;
    long long sx = 0, sxx = 0, sy[kNOff], syy[kNPair];
    {
        Acc ax = 0, axx = 0, ay[kNOff], ayy[kNPair];
#pragma unroll
        for (int j = 0; j < kNOff; ++j)
            ay[j] = 0;
#pragma unroll
        for (int j = 0; j < kNPair; ++j)
            ayy[j] = 0;
        if (valid && ok) {
            // unrolled by four: four frames' samples in flight at once
#pragma unroll 4
            for (int t = 0; t < n; ++t) {
                const Acc x = ld_px<T>(p.s, 0, t, row, col);
                ax += x;
                axx += x * x;
                Acc y[kNOff];
#pragma unroll
                for (int j = 0; j < kNOff; ++j) {
                    const int c = col1 + j - kR;
                    y[j] = (c >= 0 && c < cols) ? ld_px<T>(p.s, 1, t, row, c) : 0;
                    ay[j] += y[j];
                }
#pragma unroll
                for (int j = 0; j < kNOff; ++j)
#pragma unroll
                    for (int k = j; k < kNOff; ++k)
                        ayy[pair_index(j, k)] += y[j] * y[k];
            }
        }
        sx = ax;
        sxx = axx;
#pragma unroll
        for (int j = 0; j < kNOff; ++j)
            sy[j] = ay[j];
#pragma unroll
        for (int j = 0; j < kNPair; ++j)
            syy[j] = ayy[j];
    }

    const long long nn = n;
    const long long v0 = nn * sxx - sx * sx;
    const R mvn = (R)p.minvar * (R)n;  // the per-stack threshold times n
    const bool mv = p.has_minvar != 0;
    // rho from exact numerator and variance moments (num = n Sxy - Sx Sy)
    auto rho_int = [&](long long num, long long v1) -> R {
        if (mv && ((R)v0 < mvn || (R)v1 < mvn))
            return (R)-1;
        return F::ratio((R)num, (R)v0, (R)v1);
    };
    const int c0 = kR;  // index of offset 0

    if constexpr (MODE == 0) {
        if (in) {
            int16_t out = kInvalidDisp;
            R corr = (R)NAN;
            if (valid && ok) {
                corr = rho_int(nn * sxy[c0] - sx * sy[c0], nn * syy[pair_index(c0, c0)] - sy[c0] * sy[c0]);
                if (!(corr < (R)p.thr))
                    out = d;
            }
            reinterpret_cast<int16_t*>(reinterpret_cast<char*>(p.out) + row * p.out_pitch)[col] = out;
            if (p.corr)
                reinterpret_cast<R*>(reinterpret_cast<char*>(p.corr) + row * p.corr_pitch)[col] = corr;
            if (p.pts)
                reproject_store(p.q, reinterpret_cast<float*>(reinterpret_cast<char*>(p.pts) + row * p.pts_pitch),
                                col, row, (float)out);
        }
    } else if constexpr (MODE == 1) {
        if (in) {
            float result = NAN;
            R corr = (R)NAN;
            if (valid && ok) {
                if (col1 == 0 || col1 == cols - 1) {
                    corr = rho_int(nn * sxy[c0] - sx * sy[c0], nn * syy[pair_index(c0, c0)] - sy[c0] * sy[c0]);
                    if (!(corr < (R)p.thr))
                        result = (float)d;
                } else {
                    const int m = c0 - 1, z = c0, q = c0 + 1;  // offsets -1, 0, +1
                    const long long XA = sxy[m] - 2 * sxy[z] + sxy[q], XB = sxy[q] - sxy[m], XC = sxy[z];
                    const long long YA = sy[m] - 2 * sy[z] + sy[q], YB = sy[q] - sy[m], YC = sy[z];
                    const long long Smm = syy[pair_index(m, m)], Szz = syy[pair_index(z, z)],
                                    Sqq = syy[pair_index(q, q)], Smz = syy[pair_index(m, z)],
                                    Szq = syy[pair_index(z, q)], Smq = syy[pair_index(m, q)];
                    const long long AA = Smm + 4 * Szz + Sqq - 4 * Smz - 4 * Szq + 2 * Smq;
                    const long long AB = Sqq - Smm + 2 * Smz - 2 * Szq;
                    const long long BB = Sqq - 2 * Smq + Smm;
                    const long long AC2 = Smz - 2 * Szz + Szq;
                    const long long BC2 = Szq - Smz;
                    const long long CC = Szz;
                    const R P2 = (R)(nn * XA - sx * YA), P1 = (R)(nn * XB - sx * YB),
                            P0 = (R)(2 * (nn * XC - sx * YC));
                    const R Q4 = (R)(nn * AA - YA * YA), Q3 = (R)(2 * (nn * AB - YA * YB)),
                            Q2 = (R)(nn * BB + 4 * nn * AC2 - YB * YB - 4 * YA * YC),
                            Q1 = (R)(4 * (nn * BC2 - YB * YC)), Q0 = (R)(4 * (nn * CC - YC * YC));
                    const R V0 = (R)v0, mvq = (R)4 * mvn;
                    const bool low0 = mv && V0 < mvn;
                    R best = (R)-1;
                    float best_x = 0.f;
                    auto eval_all = [&]() {
                        for (float xs = -1.f; xs <= 1.f; xs = __fadd_rn(xs, p.step)) {
                            const R X = (R)xs;
                            const R Pv = F::fma(F::fma(P2, X, P1), X, P0);
                            const R Qv = F::fma(F::fma(F::fma(F::fma(Q4, X, Q3), X, Q2), X, Q1), X, Q0);
                            const R r = (low0 || (mv && Qv < mvq)) ? (R)-1 : F::ratio(Pv, V0, Qv);
                            if (best < r) {
                                best = r;
                                best_x = xs;
                            }
                        }
                    };
                    if constexpr (DBL) {
                        // Screening in single precision with a rigorous
                        // bound, FP64 (the Horner values and the ratio, as
                        // in eval_all) only for the points that can be the
                        // FP64 first maximum.  For |x| <= 1 the float Horner
                        // values Pf, Qf of the float-rounded coefficients
                        // lie within eP, eQ of the FP64 ones (three and five
                        // roundings of at most 2^-24 of the coefficients'
                        // magnitude sum, taken with a margin of 4); rho(x)
                        // is then bracketed by [lo, hi].  A point is a
                        // candidate while hi reaches the largest lo seen and
                        // -1 (which never wins); the min-variance test is
                        // decided in float when the bound allows, else the
                        // point is a candidate.  More than kMKeep
                        // candidates: every point in FP64.
                        constexpr int kMKeep = 6;
                        float kx[kMKeep], kh[kMKeep];
                        int nk = 0;
                        bool overflow = false;
                        const float p2 = (float)P2, p1 = (float)P1, p0 = (float)P0;
                        const float q4 = (float)Q4, q3 = (float)Q3, q2 = (float)Q2, q1 = (float)Q1, q0 = (float)Q0;
                        const float eP = ldexpf(fabsf(p2) + fabsf(p1) + fabsf(p0), -20);
                        const float eQ = ldexpf(fabsf(q4) + fabsf(q3) + fabsf(q2) + fabsf(q1) + fabsf(q0), -19);
                        const float v0f = (float)V0, mvqf = (float)mvq;
                        const float mv_lo = mvqf * (1.f - 0x1p-20f), mv_hi = mvqf * (1.f + 0x1p-20f);
                        float best_lo = -1.f;
                        if (!low0) {
                            for (float xs = -1.f; xs <= 1.f; xs = __fadd_rn(xs, p.step)) {
                                const float Pf = __fmaf_rn(__fmaf_rn(p2, xs, p1), xs, p0);
                                const float Qf =
                                    __fmaf_rn(__fmaf_rn(__fmaf_rn(__fmaf_rn(q4, xs, q3), xs, q2), xs, q1), xs, q0);
                                const float qlo = Qf - eQ, qhi = Qf + eQ;
                                bool unsure = false;
                                if (mv) {
                                    if (qhi < mv_lo)
                                        continue;  // rejected by the min-variance test: -1
                                    unsure = !(qlo >= mv_hi);
                                }
                                float lo = -INFINITY, hi = INFINITY;
                                if (!unsure && qlo > 0.f) {
                                    const float plo = Pf - eP, phi = Pf + eP;
                                    const float s_lo = rsqrtf(v0f * qhi), s_hi = rsqrtf(v0f * qlo);
                                    hi = phi >= 0.f ? phi * s_hi : phi * s_lo;
                                    lo = plo >= 0.f ? plo * s_lo : plo * s_hi;
                                    const float m = ldexpf(fmaxf(fabsf(hi), fabsf(lo)), -20);
                                    hi += m;
                                    lo -= m;
                                }
                                if (!(hi > -1.f) || hi < best_lo)
                                    continue;
                                if (lo > best_lo) {
                                    best_lo = lo;
                                    int w = 0;
                                    for (int i = 0; i < nk; ++i)
                                        if (!(kh[i] < best_lo)) {
                                            kx[w] = kx[i];
                                            kh[w] = kh[i];
                                            ++w;
                                        }
                                    nk = w;
                                }
                                if (nk < kMKeep) {
                                    kx[nk] = xs;
                                    kh[nk] = hi;
                                    ++nk;
                                } else {
                                    overflow = true;
                                }
                            }
                        }
                        if (!overflow) {
                            for (int i = 0; i < nk; ++i) {
                                if (kh[i] < best_lo)
                                    continue;
                                const R X = (R)kx[i];
                                const R Pv = F::fma(F::fma(P2, X, P1), X, P0);
                                const R Qv = F::fma(F::fma(F::fma(F::fma(Q4, X, Q3), X, Q2), X, Q1), X, Q0);
                                const R r = (mv && Qv < mvq) ? (R)-1 : F::ratio(Pv, V0, Qv);
                                if (best < r) {
                                    best = r;
                                    best_x = kx[i];
                                }
                            }
                        } else {
                            eval_all();
                        }
                    } else {
                        eval_all();
                    }
                    corr = best;
                    if (!(best < (R)p.thr))
                        result = __fsub_rn((float)d, best_x);
                }
            }
            reinterpret_cast<float*>(reinterpret_cast<char*>(p.out) + row * p.out_pitch)[col] = result;
            if (p.corr)
                reinterpret_cast<R*>(reinterpret_cast<char*>(p.corr) + row * p.corr_pitch)[col] = corr;
            if (p.pts)
                reproject_store(p.q, reinterpret_cast<float*>(reinterpret_cast<char*>(p.pts) + row * p.pts_pitch),
                                col, row, result);
        }
    } else {
        // features: rho at col1-2..col1+2 (NaN outside the image), the left
        // and right (col1) variances per frame, and a validity flag
        if (in) {
            float f[8];
#pragma unroll
            for (int j = 0; j < 8; ++j)
                f[j] = NAN;
            f[7] = 0.f;
            if (valid && ok) {
#pragma unroll
                for (int j = 0; j < kNOff; ++j) {
                    const int c = col1 + j - kR;
                    if (c >= 0 && c < cols) {
                        const long long v1 = nn * syy[pair_index(j, j)] - sy[j] * sy[j];
                        f[j] = (float)F::ratio((R)(nn * sxy[j] - sx * sy[j]), (R)v0, (R)v1);
                    }
                }
                const float n2 = (float)n * (float)n;
                f[5] = (float)v0 / n2;
                f[6] = (float)(nn * syy[pair_index(c0, c0)] - sy[c0] * sy[c0]) / n2;
                f[7] = 1.f;
            }
            float4* o = reinterpret_cast<float4*>(reinterpret_cast<char*>(p.out) + row * p.out_pitch) + 2 * col;
            o[0] = make_float4(f[0], f[1], f[2], f[3]);
            o[1] = make_float4(f[4], f[5], f[6], f[7]);
        }
    }

    if (tid == 0 && sh.abort)  // the MMAs land before the TMEM is freed
        wait_drain(smem_u32(&sh.mbar), 0);
    fence_before();
    __syncthreads();
    if (tid == 0 && sh.abort)
        atomicAdd(&g_mom_faults, 1u);
    if (warp == 0) {
        fence_after();
        tmem_dealloc(sh.tmem, kTmemCols);
    }
}

template<typename T, int KSTEPS, bool DBL, int MODE>
cudaError_t launch_k(const MomentParams& p, cudaStream_t st) {
    constexpr int PARTS = sizeof(T) == 2 ? 2 : 1;
    size_t smem = (size_t)PARTS * (kRowsM + kWin) * KSTEPS * 32 + (size_t)kRowsM * kScratch * 4;
    // 12-bit stacks hold 256 TMEM columns: at least 80 KB keeps it to two
    // CTAs (512 columns) per SM, so no allocation ever waits
    if (PARTS == 2 && smem < (size_t)80 * 1024)
        smem = (size_t)80 * 1024;
    auto k = k_moments<T, KSTEPS, DBL, MODE>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess)
        return e;
    const dim3 grid((p.s.cols + kRowsM - 1) / kRowsM, p.s.rows);
    k<<<grid, kRowsM, smem, st>>>(p);
    return cudaGetLastError();
}

template<typename T, bool DBL, int MODE>
cudaError_t launch_ks(const MomentParams& p, cudaStream_t st) {
    switch ((p.s.n + 15) / 16) {
        case 1: return launch_k<T, 1, DBL, MODE>(p, st);
        case 2: return launch_k<T, 2, DBL, MODE>(p, st);
        case 3: return launch_k<T, 3, DBL, MODE>(p, st);
        case 4: return launch_k<T, 4, DBL, MODE>(p, st);
        case 5: return launch_k<T, 5, DBL, MODE>(p, st);
        default: return cudaErrorInvalidValue;
    }
}

template<int MODE>
cudaError_t launch_mode(const MomentParams& p, bool dbl, cudaStream_t st) {
    if (p.s.elem_bytes == 1)
        return dbl ? launch_ks<uint8_t, true, MODE>(p, st) : launch_ks<uint8_t, false, MODE>(p, st);
    return dbl ? launch_ks<uint16_t, true, MODE>(p, st) : launch_ks<uint16_t, false, MODE>(p, st);
}

}  // namespace

cudaError_t launch_moments(const MomentParams& p, int mode, bool dbl, cudaStream_t st) {
    switch (mode) {
        case 0: return launch_mode<0>(p, dbl, st);
        case 1: return launch_mode<1>(p, dbl, st);
        case 2: return launch_mode<2>(p, false, st);
        default: return cudaErrorInvalidValue;
    }
}

unsigned int read_moment_faults() {
    unsigned int v = 0;
    cudaMemcpyFromSymbol(&v, g_mom_faults, sizeof v);
    return v;
}

}  // namespace bicos_gb300
