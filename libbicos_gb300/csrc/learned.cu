// Learned subpixel proposal (the library's extension; no counterpart in
// libBICOS).  A small MLP maps a match's integer-disparity correlation
// neighbourhood to a subpixel offset, in place of the reference's offset
// sweep (include/impl/cuda/agree.cuh:161-259); one NCC evaluation at the
// proposal then confirms it, and the reference sweep (agree.cu,
// k_subpixel_list) decides the pixels whose check fails.
//
// Network: 7 inputs -> 64 -> 64 -> 1, GELU (tanh form) hidden activations,
// output tanh(.) in (-1, 1): the disparity is d - x, as for the sweep.
// Inputs, from a feature row f[8] of the moment kernel (mode 2: rho at the
// right columns col1-2..col1+2, left and right per-frame variances, a
// validity flag):
//   rho0 = f[2], f[1] - rho0, f[3] - rho0, f[0] - rho0, f[4] - rho0,
//   log1p(var_left), log1p(var_right)
// (non-finite correlations count as -1), then (x - mean) * (1 / std).
//
// Model buffer (floats): W1[64][7], b1[64], W2[64][64], b2[64], w3[64], b3,
// mean[7], std[7].  Training keeps FP32 parameters; inference rounds every
// parameter to BF16 and runs the 64x64 layer on the tensor cores (tcgen05,
// BF16 operands, FP32 accumulation in TMEM).
//
// Kernels:
//   k_mlp_grad     forward + backward of 64 samples per CTA (register-tiled
//                  shared-memory products), gradients added to a global sum
//   k_mlp_adam     Adam step on the summed gradient, which it clears
//   k_mlp_propose  per feature row: layer 1 in FP32, layer 2 on the tensor
//                  cores (M = 128 rows, N = 64, K = 64), layer 3 and tanh in
//                  the epilogue
//   k_learned      the matcher's stage: features, network and NCC check
//                  per pixel in one persistent pass over 128-pixel tiles
#include <cuda_bf16.h>
#include <limits.h>
#include <math.h>
#include <string.h>

#include <map>
#include <mutex>
#include <type_traits>
#include <vector>

#include "../../include/bicos_c.h"
#include "kernels.cuh"
#include "ncc.cuh"
#include "tcgen05.cuh"

namespace bicos_gb300 {

// the model file compiled into the library (empty when none was present at
// build time); defined in a source generated by the build
extern const unsigned char kEmbeddedModel[];
extern const unsigned long long kEmbeddedModelSize;

namespace {

constexpr int kIn = 7, kH = 64;
constexpr int kW1 = 0, kB1 = kW1 + kH * kIn, kW2 = kB1 + kH, kB2 = kW2 + kH * kH, kW3 = kB2 + kH,
              kB3 = kW3 + kH, kParams = kB3 + 1;
constexpr int kNorm = kParams, kModelFloats = kParams + 2 * kIn;

constexpr float kGeluC = 0.7978845608028654f;  // sqrt(2 / pi)
constexpr float kGeluA = 0.044715f;

__device__ __forceinline__ float tanh_fast(float u) {
    float t;
    asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(u));
    return t;
}

__device__ __forceinline__ float gelu_arg(float z) { return kGeluC * fmaf(kGeluA * z, z * z, z); }
// inference form: 0.5 z + 0.5 z tanh(z (c + c a z^2)), hardware tanh
__device__ __forceinline__ float gelu_fast(float z) {
    const float hz = 0.5f * z;
    return fmaf(hz, tanh_fast(z * fmaf(kGeluC * kGeluA, z * z, kGeluC)), hz);
}
__device__ __forceinline__ float gelu_from(float z, float t) { return 0.5f * z * (1.f + t); }
__device__ __forceinline__ float gelu_grad_from(float z, float t) {
    return 0.5f * (1.f + t) + 0.5f * z * (1.f - t * t) * kGeluC * fmaf(3.f * kGeluA, z * z, 1.f);
}

// network inputs of a feature row (mean/std after the parameters)
__device__ __forceinline__ void net_inputs(const float (&f)[8], const float* norm, float (&x)[kIn]) {
    float r[5];
#pragma unroll
    for (int k = 0; k < 5; ++k)
        r[k] = isfinite(f[k]) ? f[k] : -1.f;
    x[0] = r[2];
    x[1] = r[1] - r[2];
    x[2] = r[3] - r[2];
    x[3] = r[0] - r[2];
    x[4] = r[4] - r[2];
    x[5] = log1pf(fmaxf(f[5], 0.f));
    x[6] = log1pf(fmaxf(f[6], 0.f));
#pragma unroll
    for (int i = 0; i < kIn; ++i)
        x[i] = (x[i] - norm[i]) * (1.f / norm[kIn + i]);
}

// ---------------------------------------------------------------- training

constexpr int kS = 64;             // samples per CTA
constexpr int kGradThreads = 256;  // 64 x 64 outputs as 4 x 4 tiles
constexpr int kP = kH + 1;         // padded row stride (conflict-free columns)

struct GradSmem {
    float w1[kH * kIn], b1[kH], w2[kH * kP], b2[kH], w3[kH], b3;
    float norm[2 * kIn];
    float x[kS][kIn + 2];
    float z1[kS][kP];  // z1, then dL/dz1
    float h1[kS][kP];
    float z2[kS][kP];  // z2, then dL/dz2
    float h2[kS][kP];
    float dz3[kS];
};

// samples: rows of 8 floats, the feature row with the target offset in
// place of the validity flag.  Loss: 0.5 (y - target)^2 summed.
__global__ void __launch_bounds__(kGradThreads) k_mlp_grad(const float* __restrict__ model,
                                                           const float* __restrict__ samples, int count,
                                                           float* __restrict__ grad, float* __restrict__ loss) {
    extern __shared__ float4 smem_raw[];
    GradSmem& S = *reinterpret_cast<GradSmem*>(smem_raw);
    const int tid = threadIdx.x;
    for (int i = tid; i < kH * kIn; i += kGradThreads)
        S.w1[i] = model[kW1 + i];
    for (int i = tid; i < kH * kH; i += kGradThreads)
        S.w2[(i / kH) * kP + i % kH] = model[kW2 + i];
    for (int i = tid; i < kH; i += kGradThreads) {
        S.b1[i] = model[kB1 + i];
        S.b2[i] = model[kB2 + i];
        S.w3[i] = model[kW3 + i];
    }
    if (tid == 0)
        S.b3 = model[kB3];
    if (tid < 2 * kIn)
        S.norm[tid] = model[kNorm + tid];
    __syncthreads();

    const int base = blockIdx.x * kS;
    bool live = false;
    float target = 0.f;
    if (tid < kS) {
        live = base + tid < count;
        float f[8], x[kIn];
#pragma unroll
        for (int j = 0; j < 8; ++j)
            f[j] = live ? samples[(size_t)(base + tid) * 8 + j] : 0.f;
        target = f[7];
        net_inputs(f, S.norm, x);
#pragma unroll
        for (int i = 0; i < kIn; ++i)
            S.x[tid][i] = live ? x[i] : 0.f;
    }
    __syncthreads();

    // layer 1
    for (int e = tid; e < kS * kH; e += kGradThreads) {
        const int s = e % kS, j = e / kS;
        float a = S.b1[j];
#pragma unroll
        for (int i = 0; i < kIn; ++i)
            a = fmaf(S.w1[j * kIn + i], S.x[s][i], a);
        S.z1[s][j] = a;
        S.h1[s][j] = gelu_from(a, tanhf(gelu_arg(a)));
    }
    __syncthreads();

    // layer 2: thread tile rows s = sg + 16 r, columns j = 4 jg + c
    const int sg = tid & 15, jg = tid >> 4;
    {
        float acc[4][4];
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int c = 0; c < 4; ++c)
                acc[r][c] = S.b2[jg * 4 + c];
        for (int i = 0; i < kH; ++i) {
            float a[4], b[4];
#pragma unroll
            for (int r = 0; r < 4; ++r)
                a[r] = S.h1[sg + 16 * r][i];
#pragma unroll
            for (int c = 0; c < 4; ++c)
                b[c] = S.w2[(jg * 4 + c) * kP + i];
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    acc[r][c] = fmaf(a[r], b[c], acc[r][c]);
        }
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const float z = acc[r][c];
                S.z2[sg + 16 * r][jg * 4 + c] = z;
                S.h2[sg + 16 * r][jg * 4 + c] = gelu_from(z, tanhf(gelu_arg(z)));
            }
    }
    __syncthreads();

    // output, loss, dL/dz3
    if (tid < kS) {
        float a = S.b3;
        for (int j = 0; j < kH; ++j)
            a = fmaf(S.w3[j], S.h2[tid][j], a);
        const float y = tanhf(a);
        const float dy = live ? y - target : 0.f;
        S.dz3[tid] = dy * (1.f - y * y);
        float l = 0.5f * dy * dy;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            l += __shfl_xor_sync(0xffffffffu, l, o);
        if ((tid & 31) == 0)
            atomicAdd(loss, l);
    }
    __syncthreads();

    // dL/dz2 in place of z2
    for (int e = tid; e < kS * kH; e += kGradThreads) {
        const int s = e % kS, j = e / kS;
        const float z = S.z2[s][j];
        S.z2[s][j] = S.dz3[s] * S.w3[j] * gelu_grad_from(z, tanhf(gelu_arg(z)));
    }
    __syncthreads();

    // dL/dz1 = (dz2 W2) * gelu'(z1), in place of z1 (each element is read
    // and written by its own thread only)
    {
        float acc[4][4] = {};
        for (int j = 0; j < kH; ++j) {
            float a[4], b[4];
#pragma unroll
            for (int r = 0; r < 4; ++r)
                a[r] = S.z2[sg + 16 * r][j];
#pragma unroll
            for (int c = 0; c < 4; ++c)
                b[c] = S.w2[j * kP + jg * 4 + c];
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    acc[r][c] = fmaf(a[r], b[c], acc[r][c]);
        }
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const float z = S.z1[sg + 16 * r][jg * 4 + c];
                S.z1[sg + 16 * r][jg * 4 + c] = acc[r][c] * gelu_grad_from(z, tanhf(gelu_arg(z)));
            }
    }
    __syncthreads();

    // dW2[j][i] = sum_s dz2[s][j] h1[s][i]: thread tile rows j = sg + 16 r,
    // columns i = 4 jg + c
    {
        float acc[4][4] = {};
        for (int s = 0; s < kS; ++s) {
            float a[4], b[4];
#pragma unroll
            for (int r = 0; r < 4; ++r)
                a[r] = S.z2[s][sg + 16 * r];
#pragma unroll
            for (int c = 0; c < 4; ++c)
                b[c] = S.h1[s][jg * 4 + c];
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    acc[r][c] = fmaf(a[r], b[c], acc[r][c]);
        }
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int c = 0; c < 4; ++c)
                atomicAdd(&grad[kW2 + (sg + 16 * r) * kH + jg * 4 + c], acc[r][c]);
    }
    // dW1, db1, db2, dw3, db3
    for (int e = tid; e < kH * kIn + 3 * kH + 1; e += kGradThreads) {
        float a = 0.f;
        if (e < kH * kIn) {
            const int j = e / kIn, i = e % kIn;
            for (int s = 0; s < kS; ++s)
                a = fmaf(S.z1[s][j], S.x[s][i], a);
            atomicAdd(&grad[kW1 + e], a);
        } else if (e < kH * kIn + kH) {
            const int j = e - kH * kIn;
            for (int s = 0; s < kS; ++s)
                a += S.z1[s][j];
            atomicAdd(&grad[kB1 + j], a);
        } else if (e < kH * kIn + 2 * kH) {
            const int j = e - kH * kIn - kH;
            for (int s = 0; s < kS; ++s)
                a += S.z2[s][j];
            atomicAdd(&grad[kB2 + j], a);
        } else if (e < kH * kIn + 3 * kH) {
            const int j = e - kH * kIn - 2 * kH;
            for (int s = 0; s < kS; ++s)
                a = fmaf(S.dz3[s], S.h2[s][j], a);
            atomicAdd(&grad[kW3 + j], a);
        } else {
            for (int s = 0; s < kS; ++s)
                a += S.dz3[s];
            atomicAdd(&grad[kB3], a);
        }
    }
}

// Adam (Kingma & Ba 2015) with bias correction; grad is scaled by `scale`
// (1 / batch) and cleared for the next batch
__global__ void k_mlp_adam(float* __restrict__ params, float* __restrict__ grad, float* __restrict__ m,
                           float* __restrict__ v, int step, float lr, float scale) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParams)
        return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float g = grad[i] * scale;
    const float mi = b1 * m[i] + (1.f - b1) * g;
    const float vi = b2 * v[i] + (1.f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / (1.f - powf(b1, (float)step));
    const float vh = vi / (1.f - powf(b2, (float)step));
    params[i] -= lr * mh / (sqrtf(vh) + eps);
    grad[i] = 0.f;
}

// --------------------------------------------------------------- inference

constexpr int kRowsPT = 128;      // rows (pixels) per tile = MMA M = threads per CTA
constexpr int kInferCtas = 8;     // resident CTAs per SM (TMEM: 8 x 64 columns)
constexpr uint32_t kAChunk = kRowsPT * 16;  // bytes of one 8-wide K chunk of A
constexpr uint32_t kBChunk = kH * 16;       // same for B
constexpr uint32_t kTmemCols = 64;

__device__ unsigned int g_mlp_faults = 0;

struct InferSmem {
    // A: hidden layer 1 as BF16, 128 rows x 64, canonical K-major without
    // swizzle, K-chunk-major: chunk c (units 8c..8c+7) of row r at
    // c * kAChunk + r * 16.  B: W2 as 64 (units out) x 64 (units in), same
    // layout with kBChunk.
    alignas(128) uint8_t a[kRowsPT * kH * 2];
    alignas(128) uint8_t b[kH * kH * 2];
    float4 w1[kH / 2][4];  // units 2p, 2p+1: (w[2p][i], w[2p+1][i], w[2p][i+1], w[2p+1][i+1]) ..., biases
    float4 bw[kH / 2];     // units 2p, 2p+1 of layer 2: biases, then output weights
    float norm[2 * kIn];
    float b3;
    alignas(8) uint64_t mbar;
    uint32_t tmem;
    int abort;
};

__device__ __forceinline__ float bf16r(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

// two floats to BF16 (round to nearest even), lo in the low half
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}

// packed FP32 pairs (f32x2): two hidden units per instruction
typedef unsigned long long f2;
__device__ __forceinline__ f2 pk(float lo, float hi) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void upk(f2 v, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f2 add2(f2 a, f2 b) {
    f2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 mul2(f2 a, f2 b) {
    f2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
    f2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
// gelu_fast on both lanes
__device__ __forceinline__ f2 gelu2(f2 z) {
    const f2 hz = mul2(z, pk(0.5f, 0.5f));
    const f2 u = mul2(z, fma2(mul2(z, z), pk(kGeluC * kGeluA, kGeluC * kGeluA), pk(kGeluC, kGeluC)));
    float u0, u1;
    upk(u, u0, u1);
    return fma2(hz, pk(tanh_fast(u0), tanh_fast(u1)), hz);
}

// parameters (rounded to BF16) into shared memory, mbarrier, TMEM
__device__ void infer_setup(InferSmem& S, const float* __restrict__ model) {
    using namespace tc;
    const int tid = threadIdx.x;
    for (int p = tid; p < kH / 2; p += kRowsPT) {
        const float* w0 = model + kW1 + (2 * p) * kIn;
        const float* w1 = model + kW1 + (2 * p + 1) * kIn;
        float v[16];
        for (int i = 0; i < kIn; ++i) {
            v[2 * i] = bf16r(w0[i]);
            v[2 * i + 1] = bf16r(w1[i]);
        }
        v[14] = bf16r(model[kB1 + 2 * p]);
        v[15] = bf16r(model[kB1 + 2 * p + 1]);
        for (int q = 0; q < 4; ++q)
            S.w1[p][q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
        S.bw[p] = make_float4(bf16r(model[kB2 + 2 * p]), bf16r(model[kB2 + 2 * p + 1]), bf16r(model[kW3 + 2 * p]),
                              bf16r(model[kW3 + 2 * p + 1]));
    }
    if (tid < 2 * kIn)
        S.norm[tid] = model[kNorm + tid];
    if (tid == 0) {
        S.b3 = bf16r(model[kB3]);
        S.abort = 0;
        mbar_init(smem_u32(&S.mbar), 1);
    }
    // W2 into the B tile: 8 consecutive inputs of one unit per 16-byte store
    for (int e = tid; e < kH * (kH / 8); e += kRowsPT) {
        const int j = e / (kH / 8), c = e % (kH / 8);
        const float* w = model + kW2 + j * kH + c * 8;
        *reinterpret_cast<uint4*>(S.b + c * kBChunk + j * 16) =
            make_uint4(pack_bf16(w[0], w[1]), pack_bf16(w[2], w[3]), pack_bf16(w[4], w[5]), pack_bf16(w[6], w[7]));
    }
    if ((tid >> 5) == 0) {
        tmem_alloc(smem_u32(&S.tmem), kTmemCols);
        tmem_relinquish();
    }
    fence_before();
    __syncthreads();
    fence_after();
}

__device__ void infer_teardown(InferSmem& S) {
    using namespace tc;
    fence_before();
    __syncthreads();
    if (threadIdx.x == 0 && S.abort)
        atomicAdd(&g_mlp_faults, 1u);
    if ((threadIdx.x >> 5) == 0) {
        fence_after();
        tmem_dealloc(S.tmem, kTmemCols);
    }
}

// The network on one tile of 128 rows, one row per thread (every thread of
// the CTA calls it): layer 1 in FP32 with GELU into row threadIdx.x of A as
// BF16, layer 2 by four tcgen05 MMAs (K = 16 each) into TMEM, then bias,
// GELU, the output unit and tanh from this thread's TMEM lane.  False when
// the MMA's completion was not seen in time (the CTA then stops).
__device__ bool infer_tile(InferSmem& S, const float (&x)[kIn], uint32_t phase, float* y) {
    using namespace tc;
    const int tid = threadIdx.x, warp = tid >> 5;
    f2 X[kIn];
#pragma unroll
    for (int i = 0; i < kIn; ++i)
        X[i] = pk(x[i], x[i]);
    // layer 1: two units per packed FMA chain
#pragma unroll 1
    for (int c = 0; c < kH / 8; ++c) {
        uint32_t h[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int p = c * 4 + q;
            const float4 w01 = S.w1[p][0], w23 = S.w1[p][1], w45 = S.w1[p][2], w6b = S.w1[p][3];
            f2 z = pk(w6b.z, w6b.w);
            z = fma2(pk(w01.x, w01.y), X[0], z);
            z = fma2(pk(w01.z, w01.w), X[1], z);
            z = fma2(pk(w23.x, w23.y), X[2], z);
            z = fma2(pk(w23.z, w23.w), X[3], z);
            z = fma2(pk(w45.x, w45.y), X[4], z);
            z = fma2(pk(w45.z, w45.w), X[5], z);
            z = fma2(pk(w6b.x, w6b.y), X[6], z);
            float g0, g1;
            upk(gelu2(z), g0, g1);
            h[q] = pack_bf16(g0, g1);
        }
        *reinterpret_cast<uint4*>(S.a + c * kAChunk + tid * 16) = make_uint4(h[0], h[1], h[2], h[3]);
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    const uint32_t mbar = smem_u32(&S.mbar);
    if (tid == 0) {
        fence_after();
        constexpr uint32_t idesc = idesc_bf16(kRowsPT, kH);
        const uint32_t a_base = smem_u32(S.a), b_base = smem_u32(S.b);
#pragma unroll
        for (int ks = 0; ks < kH / 16; ++ks)
            mma_f16(S.tmem, smem_desc(a_base + 2 * ks * kAChunk, kAChunk, 128),
                    smem_desc(b_base + 2 * ks * kBChunk, kBChunk, 128), idesc, ks > 0 ? 1u : 0u);
        mma_commit(mbar);
    }
    const bool ok = wait_or_abort(mbar, phase, &S.abort);
    if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0)  // the MMAs land before the TMEM is freed
            wait_drain(mbar, phase);
        return false;
    }
    fence_after();
    // layer 2 epilogue, two units per packed step; even and odd units
    // accumulate in the two lanes
    f2 acc = 0ull;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        float v[32];
        tmem_ld32(S.tmem + ((uint32_t)(warp * 32) << 16) + half * 32, v);
#pragma unroll
        for (int k = 0; k < 32; k += 2) {
            const float4 bw = S.bw[(half * 32 + k) / 2];
            const f2 z = add2(pk(v[k], v[k + 1]), pk(bw.x, bw.y));
            acc = fma2(pk(bw.z, bw.w), gelu2(z), acc);
        }
    }
    float a0, a1;
    upk(acc, a0, a1);
    *y = tanhf(S.b3 + (a0 + a1));
    return true;
}

// proposals of feature rows (training validation, bicos_mlp_propose_v1)
__global__ void __launch_bounds__(kRowsPT) k_mlp_propose(const float* __restrict__ model,
                                                          const float* __restrict__ features, int count,
                                                          float* __restrict__ out) {
    __shared__ InferSmem S;
    infer_setup(S, model);
    const int tiles = (count + kRowsPT - 1) / kRowsPT;
    uint32_t phase = 0;
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x, phase ^= 1u) {
        const int row = tile * kRowsPT + threadIdx.x;
        const bool live = row < count;
        float f[8], x[kIn];
        if (live) {
            const float4* fr = reinterpret_cast<const float4*>(features + (size_t)row * 8);
            const float4 u = __ldg(fr), w = __ldg(fr + 1);
            f[0] = u.x, f[1] = u.y, f[2] = u.z, f[3] = u.w, f[4] = w.x, f[5] = w.y, f[6] = w.z, f[7] = w.w;
        } else {
#pragma unroll
            for (int j = 0; j < 8; ++j)
                f[j] = 0.f;
        }
        net_inputs(f, S.norm, x);
        float y;
        if (!infer_tile(S, x, phase, &y))
            break;
        if (live)
            out[row] = y;
    }
    infer_teardown(S);
}

// Feature row of one interior match, the same values as the moment
// kernel's mode 2 (moments.cu): exact integer sums over the frames of the
// left pixel and of the right columns col1-2..col1+2, then FP32 ratios.
template<typename T, typename Row>
__device__ __forceinline__ void pixel_features(const Row& src, int n, int cols, int col, int col1, float (&f)[8]) {
    using Acc = typename std::conditional<sizeof(T) == 1, int, long long>::type;
    Acc sx = 0, sxx = 0, sy[5] = {}, syy[5] = {}, sxy[5] = {};
    for (int t = 0; t < n; ++t) {
        const Acc x = (Acc)src.left(t, col);
        sx += x;
        sxx += x * x;
#pragma unroll
        for (int j = 0; j < 5; ++j) {
            const int c = col1 + j - 2;
            const Acc y = (c >= 0 && c < cols) ? (Acc)src.right(t, c) : (Acc)0;
            sy[j] += y;
            syy[j] += y * y;
            sxy[j] += x * y;
        }
    }
    const long long nn = n;
    const long long v0 = nn * (long long)sxx - (long long)sx * (long long)sx;
    const float fv0 = __ll2float_rn(v0);
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        const int c = col1 + j - 2;
        if (c >= 0 && c < cols) {
            const long long v1 = nn * (long long)syy[j] - (long long)sy[j] * (long long)sy[j];
            const long long num = nn * (long long)sxy[j] - (long long)sx * (long long)sy[j];
            f[j] = __fdiv_rn(__ll2float_rn(num), __fsqrt_rn(__fmul_rn(fv0, __ll2float_rn(v1))));
        } else {
            f[j] = NAN;
        }
    }
    const float n2 = __fmul_rn((float)n, (float)n);
    f[5] = __fdiv_rn(fv0, n2);
    f[6] = __fdiv_rn(__ll2float_rn(nn * (long long)syy[2] - (long long)sy[2] * (long long)sy[2]), n2);
    f[7] = 1.f;
}

// The same features from the tile's shared-memory copy: lp points at the
// left sample of frame 0 (frames kRowsPT apart), rp at the right column col1
// of frame 0 (frames rstride apart); bit j of okm: column col1-2+j is inside
// the image (outside ones read column col1 and count as 0).  Also returns
// the left sum.
template<typename T>
__device__ __forceinline__ int features_staged(const T* __restrict__ lp, const T* __restrict__ rp, int n,
                                               int rstride, int okm, float (&f)[8]) {
    using Acc = typename std::conditional<sizeof(T) == 1, int, long long>::type;
    int off[5];
    Acc m[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        const bool ok = (okm >> j) & 1;
        off[j] = ok ? j - 2 : 0;
        m[j] = ok ? 1 : 0;
    }
    Acc sx = 0, sxx = 0, sy[5] = {}, syy[5] = {}, sxy[5] = {};
    if (okm == 31) {  // all five columns inside the image
#pragma unroll 2
        for (int t = 0; t < n; ++t, lp += kRowsPT, rp += rstride) {
            const Acc x = (Acc)lp[0];
            sx += x;
            sxx += x * x;
#pragma unroll
            for (int j = 0; j < 5; ++j) {
                const Acc y = (Acc)rp[j - 2];
                sy[j] += y;
                syy[j] += y * y;
                sxy[j] += x * y;
            }
        }
    } else {
        for (int t = 0; t < n; ++t, lp += kRowsPT, rp += rstride) {
            const Acc x = (Acc)lp[0];
            sx += x;
            sxx += x * x;
#pragma unroll
            for (int j = 0; j < 5; ++j) {
                const Acc y = (Acc)rp[off[j]] * m[j];
                sy[j] += y;
                syy[j] += y * y;
                sxy[j] += x * y;
            }
        }
    }
    const long long nn = n;
    const long long v0 = nn * (long long)sxx - (long long)sx * (long long)sx;
    const float fv0 = __ll2float_rn(v0);
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        if ((okm >> j) & 1) {
            const long long v1 = nn * (long long)syy[j] - (long long)sy[j] * (long long)sy[j];
            const long long num = nn * (long long)sxy[j] - (long long)sx * (long long)sy[j];
            f[j] = __fdiv_rn(__ll2float_rn(num), __fsqrt_rn(__fmul_rn(fv0, __ll2float_rn(v1))));
        } else {
            f[j] = NAN;
        }
    }
    const float n2 = __fmul_rn((float)n, (float)n);
    f[5] = __fdiv_rn(fv0, n2);
    f[6] = __fdiv_rn(__ll2float_rn(nn * (long long)syy[2] - (long long)sy[2] * (long long)sy[2]), n2);
    f[7] = 1.f;
    return (int)sx;
}

// The reference NCC at offset x (nxc_row<T, DBL, true>, same operations in
// the same order) from the tile's shared-memory copy, with the left sum sx
// known and the rounded interpolants of the first pass kept in iv (this
// thread's column, frames kRowsPT apart) for the second.
template<typename T, bool DBL>
__device__ __forceinline__ typename Prec<DBL>::T check_staged(const T* __restrict__ lp, const T* __restrict__ rp,
                                                               T* __restrict__ iv, int n, int rstride, int sx,
                                                               float x, bool mv, float minvar) {
    int sy = 0;
    {
        const T* r = rp;
        T* v = iv;
#pragma unroll 2
        for (int t = 0; t < n; ++t, r += rstride, v += kRowsPT) {
            const int y0 = r[-1], y1 = r[0], y2 = r[1];
            const float a = 0.5f * small_int_to_float(y0 - 2 * y1 + y2), b = 0.5f * small_int_to_float(y2 - y0),
                        c = small_int_to_float(y1);
            const int q = round_wrap_bits<T>(__fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(a, x), x), __fmul_rn(b, x)), c));
            *v = (T)q;
            sy += q;
        }
    }
    if constexpr (DBL) {
        double cov = 0, var0 = 0, var1 = 0;
        const double m0 = __ddiv_rn((double)sx, (double)n), m1 = __ddiv_rn((double)sy, (double)n);
        for (int t = 0; t < n; ++t, lp += kRowsPT, iv += kRowsPT) {
            const double d0 = __dsub_rn((double)(int)lp[0], m0);
            const double d1 = __dsub_rn((double)(int)iv[0], m1);
            var0 = __fma_rn(d0, d0, var0);
            cov = __fma_rn(d0, d1, cov);
            var1 = __fma_rn(d1, d1, var1);
        }
        if (mv && (var0 < (double)minvar || var1 < (double)minvar))
            return -1.0;
        return __ddiv_rn(cov, __dsqrt_rn(__dmul_rn(var0, var1)));
    } else {
        float cov = 0, var0 = 0, var1 = 0;
        const float m0 = __fdiv_rn((float)sx, (float)n), m1 = __fdiv_rn((float)sy, (float)n);
#pragma unroll 2
        for (int t = 0; t < n; ++t, lp += kRowsPT, iv += kRowsPT) {
            const float d0 = __fsub_rn(small_int_to_float(lp[0]), m0);
            const float d1 = __fsub_rn(small_int_to_float(iv[0]), m1);
            var0 = __fmaf_rn(d0, d0, var0);
            cov = __fmaf_rn(d0, d1, cov);
            var1 = __fmaf_rn(d1, d1, var1);
        }
        if (mv && (var0 < minvar || var1 < minvar))
            return -1.f;
        return __fdiv_rn(cov, __fsqrt_rn(__fmul_rn(var0, var1)));
    }
}

constexpr int kWin = 256;  // right-window columns one tile may stage

// shared-memory copy of frames' columns [c0, c1) of one row, row stride
// `stride` elements; 16-byte loads when the frames allow them
template<typename T>
__device__ __forceinline__ void stage_rows(const StackParams& s, int side, int row, int c0, int c1, T* dst,
                                           int stride, bool vec16) {
    const int n = s.n;
    if (vec16) {
        const int chunks = (c1 - c0) * (int)sizeof(T) / 16;
        for (int e = threadIdx.x; e < n * chunks; e += blockDim.x) {
            const int t = e / chunks, k = e - t * chunks;
            const uint8_t* src = s.frame[side][t] + (long long)row * s.pitch[side][t] + (long long)c0 * sizeof(T);
            *reinterpret_cast<uint4*>(reinterpret_cast<uint8_t*>(dst + t * stride) + k * 16) =
                __ldg(reinterpret_cast<const uint4*>(src) + k);
        }
    } else {
        const int w = c1 - c0;
        for (int e = threadIdx.x; e < n * w; e += blockDim.x) {
            const int t = e / w, k = e - t * w;
            dst[t * stride + k] = __ldg(reinterpret_cast<const T*>(s.frame[side][t] + (long long)row * s.pitch[side][t]) + c0 + k);
        }
    }
}

template<typename T>
constexpr int stage_rstride() { return kWin + 32 / (int)sizeof(T); }

template<typename T>
size_t stage_bytes(int n) { return (size_t)n * sizeof(T) * (kRowsPT + stage_rstride<T>()); }

// The learned agreement stage in one pass over 128-pixel row tiles: per
// pixel the features, the network's offset x (tensor cores for the 64x64
// layer), and one NCC evaluation in the reference's arithmetic at x; the
// proposal is accepted when rho(x) >= rho(0) - drop (rho(0) = feature 2)
// and written as the sweep would write offset x (d - x, corrmap rho(x),
// NaN below the threshold); otherwise the pixel joins the list for the
// reference sweep.  Border pixels (col1 = 0 or cols - 1) take the plain
// correlation at col1, as in the sweep (agree.hpp:110-118).
//
// Each tile first copies its left columns and the right columns its
// matches need (at most kWin wide) of every frame into shared memory, so
// the three passes over the frames read shared memory; a tile whose
// matches spread wider reads the frames from global memory instead.
template<typename T, bool DBL>
__global__ void __launch_bounds__(kRowsPT) k_learned(const __grid_constant__ LearnedParams lp) {
    using TP = typename Prec<DBL>::T;
    __shared__ InferSmem S;
    __shared__ int red[2][kRowsPT / 32];
    extern __shared__ __align__(16) uint8_t stage[];
    constexpr int rstride = stage_rstride<T>();
    infer_setup(S, lp.model);
    const AgreeParams& p = lp.a;
    const StackParams& s = p.s;
    const int cols = s.cols, n = s.n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool mv = p.has_minvar != 0;
    T* Ls = reinterpret_cast<T*>(stage);
    T* Rs = Ls + n * kRowsPT;
    const int per_row = (cols + kRowsPT - 1) / kRowsPT;
    const int tiles = s.rows * per_row;
    __shared__ int next_tile;
    uint32_t phase = 0;
    for (;; phase ^= 1u) {
        // tiles are claimed from a global counter, so every resident CTA
        // keeps working however many the SMs hold
        __syncthreads();  // the previous tile is done with the staged rows and next_tile
        if (threadIdx.x == 0)
            next_tile = atomicAdd(lp.tile_counter, 1);
        __syncthreads();
        const int tile = next_tile;
        if (tile >= tiles)
            break;
        const int row = tile / per_row;
        const int c0 = (tile - row * per_row) * kRowsPT, col = c0 + (int)threadIdx.x;
        int kind = 0;  // 0: no match, 1: border, 2: interior
        int d = 0, col1 = 0;
        if (col < cols) {
            d = reinterpret_cast<const int16_t*>(reinterpret_cast<const char*>(p.raw) + row * p.raw_pitch)[col];
            col1 = col - d;
            if (d != kInvalidDisp && col1 >= 0 && col1 < cols)
                kind = (col1 == 0 || col1 == cols - 1) ? 1 : 2;
        }
        // the right columns this tile's matches read
        int need_lo = INT_MAX, need_hi = INT_MIN;
        if (kind == 2) {
            need_lo = max(col1 - 2, 0);
            need_hi = min(col1 + 2, cols - 1);
        } else if (kind == 1) {
            need_lo = need_hi = col1;
        }
        need_lo = __reduce_min_sync(0xffffffffu, need_lo);
        need_hi = __reduce_max_sync(0xffffffffu, need_hi);
        if (lane == 0) {
            red[0][warp] = need_lo;
            red[1][warp] = need_hi;
        }
        __syncthreads();
        int lo = red[0][0], hi = red[1][0];
#pragma unroll
        for (int w = 1; w < kRowsPT / 32; ++w) {
            lo = min(lo, red[0][w]);
            hi = max(hi, red[1][w]);
        }
        int r0 = lo, r1 = hi + 1;
        if (lp.vec16 && lo <= hi) {
            r0 = ((lo * (int)sizeof(T)) & ~15) / (int)sizeof(T);
            r1 = min((((r1 * (int)sizeof(T)) + 15) & ~15) / (int)sizeof(T), cols);
        }
        const bool staged = lo > hi || r1 - r0 <= rstride;
        if (staged && lo <= hi) {
            stage_rows<T>(s, 0, row, c0, min(c0 + kRowsPT, cols), Ls, kRowsPT, lp.vec16);
            stage_rows<T>(s, 1, row, r0, r1, Rs, rstride, lp.vec16);
        }
        __syncthreads();
        const SharedRow<T> sh{Ls, Rs, kRowsPT, rstride, c0, r0};
        const GlobalRow<T> gl{&s, row};

        const T* lcol = Ls + (col - c0);
        const T* rcol = Rs + (col1 - r0);
        float x[kIn] = {};
        float r0f = NAN;
        int sx = 0;
        if (kind == 2) {
            float f[8];
            if (staged) {
                const int okm = (col1 >= 2 ? 1 : 0) | 2 | 4 | 8 | (col1 + 2 < cols ? 16 : 0);
                sx = features_staged<T>(lcol, rcol, n, rstride, okm, f);
            } else {
                pixel_features<T>(gl, n, cols, col, col1, f);
            }
            net_inputs(f, S.norm, x);
            r0f = f[2];
        }
        float xo;
        if (!infer_tile(S, x, phase, &xo))
            break;
        if (col >= cols)
            continue;
        float result = NAN;
        TP corr = (TP)NAN;
        bool fallback = false;
        if (kind == 1) {
            corr = staged ? nxc_row<T, DBL, false>(sh, n, col, col1, 0.f, mv, p.minvar)
                          : nxc_row<T, DBL, false>(gl, n, col, col1, 0.f, mv, p.minvar);
            if (!(corr < (TP)p.thr))
                result = (float)d;
        } else if (kind == 2) {
            // the A tile is free once the MMA has completed: it holds the
            // rounded interpolants between the check's two passes
            const bool iv_fits = n * (int)sizeof(T) * kRowsPT <= (int)sizeof(S.a);
            const TP nxc = staged && iv_fits
                               ? check_staged<T, DBL>(lcol, rcol, reinterpret_cast<T*>(S.a) + threadIdx.x, n, rstride,
                                                      sx, xo, mv, p.minvar)
                           : staged ? nxc_row<T, DBL, true>(sh, n, col, col1, xo, mv, p.minvar)
                                    : nxc_row<T, DBL, true>(gl, n, col, col1, xo, mv, p.minvar);
            TP floor_rho;
            if constexpr (DBL)
                floor_rho = __dsub_rn((double)r0f, (double)lp.drop);
            else
                floor_rho = __fsub_rn(r0f, lp.drop);
            if (nxc >= floor_rho) {
                corr = nxc;
                if (!(nxc < (TP)p.thr))
                    result = __fsub_rn((float)d, xo);
            } else {
                fallback = true;
            }
        }
        if (lp.proposal)
            reinterpret_cast<float*>(reinterpret_cast<char*>(lp.proposal) + row * lp.proposal_pitch)[col] =
                kind == 2 ? xo : NAN;
        if (fallback) {
            lp.list[atomicAdd(lp.count, 1)] = row * cols + col;
        } else {
            reinterpret_cast<float*>(reinterpret_cast<char*>(p.out) + row * p.out_pitch)[col] = result;
            if (p.corr)
                reinterpret_cast<TP*>(reinterpret_cast<char*>(p.corr) + row * p.corr_pitch)[col] = corr;
            agree_point(p, row, col, result);
        }
    }
    infer_teardown(S);
}

int sm_count(cudaError_t* e) {
    int dev = 0, sms = 0;
    *e = cudaGetDevice(&dev);
    if (*e == cudaSuccess)
        *e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

// ------------------------------------------------------------ model store

// file layout (little endian): "BICOSMLP", u32 version (1), u32 inputs (7),
// u32 hidden (64), u32 parameter count, f32 mean[7], f32 std[7], then the
// parameters as BF16 in model-buffer order
constexpr char kMagic[8] = {'B', 'I', 'C', 'O', 'S', 'M', 'L', 'P'};
constexpr size_t kHeaderBytes = 8 + 4 * 4 + 2 * kIn * 4;

struct DeviceModel {
    float* ptr = nullptr;
    unsigned long long version = 0;
};

std::mutex g_model_mu;
std::vector<float> g_model;  // installed model, empty = none
unsigned long long g_model_version = 0;
bool g_model_init = false;
std::map<int, DeviceModel> g_device_models;

uint32_t rd_u32(const unsigned char* p) {
    return (uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 | (uint32_t)p[3] << 24;
}

bool parse_model(const unsigned char* p, size_t n, std::vector<float>* out, std::string* err) {
    if (n < kHeaderBytes || memcmp(p, kMagic, 8) != 0) {
        *err = "learned subpixel model: not a BICOSMLP file";
        return false;
    }
    const uint32_t version = rd_u32(p + 8), nin = rd_u32(p + 12), hidden = rd_u32(p + 16), np = rd_u32(p + 20);
    if (version != 1) {
        *err = "learned subpixel model: unsupported version " + std::to_string(version);
        return false;
    }
    if (nin != (uint32_t)kIn || hidden != (uint32_t)kH || np != (uint32_t)kParams) {
        *err = "learned subpixel model: shape " + std::to_string(nin) + "/" + std::to_string(hidden) + "/" +
               std::to_string(np) + " does not match the network (7/64/" + std::to_string(kParams) + ")";
        return false;
    }
    if (n != kHeaderBytes + 2 * (size_t)kParams) {
        *err = "learned subpixel model: size " + std::to_string(n) + " bytes, expected " +
               std::to_string(kHeaderBytes + 2 * (size_t)kParams);
        return false;
    }
    std::vector<float> m(kModelFloats);
    for (int i = 0; i < kParams; ++i) {
        const unsigned char* q = p + kHeaderBytes + 2 * i;
        const uint32_t bits = ((uint32_t)q[0] | (uint32_t)q[1] << 8) << 16;
        memcpy(&m[i], &bits, 4);
    }
    for (int i = 0; i < 2 * kIn; ++i) {
        const uint32_t bits = rd_u32(p + 24 + 4 * i);
        memcpy(&m[kNorm + i], &bits, 4);
    }
    for (int i = 0; i < kIn; ++i)
        if (!(m[kNorm + kIn + i] > 0.f) || !isfinite(m[kNorm + kIn + i]) || !isfinite(m[kNorm + i])) {
            *err = "learned subpixel model: bad normalisation statistics";
            return false;
        }
    for (int i = 0; i < kParams; ++i)
        if (!isfinite(m[i])) {
            *err = "learned subpixel model: non-finite parameter";
            return false;
        }
    *out = std::move(m);
    return true;
}

void init_default_locked() {
    if (g_model_init)
        return;
    g_model_init = true;
    if (kEmbeddedModelSize == 0)
        return;
    std::string err;
    std::vector<float> m;
    if (parse_model(kEmbeddedModel, (size_t)kEmbeddedModelSize, &m, &err)) {
        g_model = std::move(m);
        g_model_version = 1;
    }
}

}  // namespace

int mlp_param_count() { return kParams; }
int mlp_model_floats() { return kModelFloats; }

cudaError_t launch_mlp_grad(const float* model, const float* samples, int count, float* grad, float* loss,
                            cudaStream_t st) {
    if (count <= 0)
        return cudaSuccess;
    const size_t smem = sizeof(GradSmem);
    cudaError_t e = cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess)
        return e;
    k_mlp_grad<<<(count + kS - 1) / kS, kGradThreads, smem, st>>>(model, samples, count, grad, loss);
    return cudaGetLastError();
}

cudaError_t launch_mlp_adam(float* params, float* grad, float* m, float* v, int step, float lr, float scale,
                            cudaStream_t st) {
    k_mlp_adam<<<(kParams + 255) / 256, 256, 0, st>>>(params, grad, m, v, step, lr, scale);
    return cudaGetLastError();
}

cudaError_t launch_mlp_propose(const float* model, const float* features, int count, float* out,
                               cudaStream_t st) {
    if (count <= 0)
        return cudaSuccess;
    cudaError_t e;
    const int sms = sm_count(&e);
    if (e != cudaSuccess)
        return e;
    const int tiles = (count + kRowsPT - 1) / kRowsPT;
    const int grid = tiles < sms * kInferCtas ? tiles : sms * kInferCtas;
    k_mlp_propose<<<grid, kRowsPT, 0, st>>>(model, features, count, out);
    return cudaGetLastError();
}

template<typename T, bool DBL>
cudaError_t launch_learned_t(const LearnedParams& p, int sms, cudaStream_t st) {
    auto k = k_learned<T, DBL>;
    const size_t smem = stage_bytes<T>(p.a.s.n);
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess)
        return e;
    // at most kInferCtas CTAs fit an SM (TMEM); CTAs beyond what the SM
    // holds start when others finish and find the tile counter exhausted
    const int tiles = p.a.s.rows * ((p.a.s.cols + kRowsPT - 1) / kRowsPT);
    const int grid = tiles < sms * kInferCtas ? tiles : sms * kInferCtas;
    k<<<grid, kRowsPT, smem, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_learned(const LearnedParams& p, bool dbl, cudaStream_t st) {
    cudaError_t e;
    const int sms = sm_count(&e);
    if (e != cudaSuccess)
        return e;
    if (p.a.s.elem_bytes == 1)
        return dbl ? launch_learned_t<uint8_t, true>(p, sms, st) : launch_learned_t<uint8_t, false>(p, sms, st);
    return dbl ? launch_learned_t<uint16_t, true>(p, sms, st) : launch_learned_t<uint16_t, false>(p, sms, st);
}

unsigned int read_mlp_faults() {
    unsigned int v = 0;
    cudaMemcpyFromSymbol(&v, g_mlp_faults, sizeof v);
    return v;
}

const float* learned_model_device(cudaStream_t st, std::string* err) {
    std::lock_guard<std::mutex> lock(g_model_mu);
    init_default_locked();
    if (g_model.empty()) {
        *err = "no learned subpixel model is installed (bicos_learned_model_v1)";
        return nullptr;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    DeviceModel& dm = g_device_models[dev];
    if (e == cudaSuccess && !dm.ptr)
        e = cudaMalloc(&dm.ptr, kModelFloats * sizeof(float));
    if (e == cudaSuccess && dm.version != g_model_version) {
        // a model install replaced the one this buffer holds: kernels (or a
        // cached batch graph) still running on other streams may read it,
        // so the device finishes its work before the buffer is rewritten
        // (installs are rare)
        if (dm.version != 0)
            e = cudaDeviceSynchronize();
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(dm.ptr, g_model.data(), kModelFloats * sizeof(float), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(st);
        if (e == cudaSuccess)
            dm.version = g_model_version;
    }
    if (e != cudaSuccess) {
        *err = std::string("learned subpixel model upload: ") + cudaGetErrorString(e);
        return nullptr;
    }
    return dm.ptr;
}

}  // namespace bicos_gb300

using namespace bicos_gb300;

extern "C" {

bicos_status bicos_learned_model_v1(const void* data, size_t nbytes) {
    std::lock_guard<std::mutex> lock(g_model_mu);
    g_model_init = true;  // an explicit install replaces the built-in model
    if (!data) {
        g_model.clear();
        ++g_model_version;
        return BICOS_OK;
    }
    std::vector<float> m;
    std::string err;
    if (!parse_model(static_cast<const unsigned char*>(data), nbytes, &m, &err)) {
        set_last_error(err);
        return BICOS_ERR_INVALID_ARGUMENT;
    }
    g_model = std::move(m);
    ++g_model_version;
    return BICOS_OK;
}

int bicos_learned_model_installed(void) {
    std::lock_guard<std::mutex> lock(g_model_mu);
    init_default_locked();
    return g_model.empty() ? 0 : 1;
}

bicos_status bicos_learned_model_floats_v1(float* out, int capacity) {
    std::lock_guard<std::mutex> lock(g_model_mu);
    init_default_locked();
    if (g_model.empty()) {
        set_last_error("no learned subpixel model is installed (bicos_learned_model_v1)");
        return BICOS_ERR_INVALID_ARGUMENT;
    }
    if (!out || capacity < kModelFloats) {
        set_last_error("bicos_learned_model_floats_v1: need room for " + std::to_string(kModelFloats) + " floats");
        return BICOS_ERR_INVALID_ARGUMENT;
    }
    memcpy(out, g_model.data(), kModelFloats * sizeof(float));
    return BICOS_OK;
}

void bicos_mlp_sizes(int* n_params, int* n_model_floats) {
    if (n_params)
        *n_params = kParams;
    if (n_model_floats)
        *n_model_floats = kModelFloats;
}

static bicos_status mlp_status(cudaError_t e, const char* what) {
    if (e == cudaSuccess)
        return BICOS_OK;
    set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
    return BICOS_ERR_CUDA;
}

bicos_status bicos_mlp_grad_v1(const float* model, const float* samples, int count, float* grad, float* loss,
                               void* stream) {
    if (!model || !grad || !loss || count < 0 || (count > 0 && !samples)) {
        set_last_error("bicos_mlp_grad_v1: null buffer or negative count");
        return BICOS_ERR_INVALID_ARGUMENT;
    }
    return mlp_status(launch_mlp_grad(model, samples, count, grad, loss, static_cast<cudaStream_t>(stream)),
                      "bicos_mlp_grad_v1");
}

bicos_status bicos_mlp_adam_v1(float* params, float* grad, float* m, float* v, int step, float lr, float scale,
                               void* stream) {
    if (!params || !grad || !m || !v || step < 1) {
        set_last_error("bicos_mlp_adam_v1: null buffer or step < 1");
        return BICOS_ERR_INVALID_ARGUMENT;
    }
    return mlp_status(launch_mlp_adam(params, grad, m, v, step, lr, scale, static_cast<cudaStream_t>(stream)),
                      "bicos_mlp_adam_v1");
}

bicos_status bicos_mlp_propose_v1(const float* model, const float* features, int count, float* out,
                                  void* stream) {
    if (!model || count < 0 || (count > 0 && (!features || !out))) {
        set_last_error("bicos_mlp_propose_v1: null buffer or negative count");
        return BICOS_ERR_INVALID_ARGUMENT;
    }
    return mlp_status(launch_mlp_propose(model, features, count, out, static_cast<cudaStream_t>(stream)),
                      "bicos_mlp_propose_v1");
}

}  // extern "C"
