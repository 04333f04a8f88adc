// Binary temporal descriptor transform (stage a).
//
// Semantics follow libBICOS include/impl/cpu/descriptor_transform.hpp:31-123
// (and the CUDA kernels include/impl/cuda/descriptor_transform.cuh:30-149):
// bit i of the descriptor is set LSB-first, word i/32.  Design: one thread
// per pixel, both sides in one launch (blockIdx.z), the n samples held in
// registers, every bit position a compile-time constant (loops fully
// unrolled over the bucket maximum), so the descriptor words never leave
// registers.  The temporal mean is the reference's float RN(sum / n); the
// sum is exact in int, and `a < mean` is evaluated as `a < ceil(mean)`,
// which is the same predicate for integer a.
#include "batch.cuh"
#include "fp8_tiles.cuh"
#include "kernels.cuh"

namespace bicos_gb300 {
namespace {

// Bit assembly: each comparison x < y is the sign bit of x - y (the
// operands are small non-negative integers), shifted into a 32-bit
// accumulator with one funnel shift, most recent bit lowest; every 32 bits
// the accumulator, bit-reversed, is one descriptor word (LSB-first).  No
// predicates and no per-bit masks: a subtraction and a shift per bit.
template<int NW>
struct BitSink {
    uint32_t w[NW];
    uint32_t acc = 0;
    __device__ __forceinline__ BitSink() {
#pragma unroll
        for (int j = 0; j < NW; ++j)
            w[j] = 0u;
    }
    // bit number k (0-based, known at compile time after unrolling) = 1
    // when d < 0
    __device__ __forceinline__ void push(int d, int k) {
        acc = __funnelshift_l((uint32_t)d, acc, 1);
        if ((k & 31) == 31)
            w[k >> 5] = __brev(acc);
    }
    // the bits pushed since the last full word (count = total pushed, not a
    // multiple of 32 and possibly known only at run time) into their word
    __device__ __forceinline__ void flush_partial(int count) {
        const int r = count & 31;
        if (r == 0)
            return;
        const uint32_t v = __brev(acc) >> (32 - r);
        const int k = count >> 5;
#pragma unroll
        for (int j = 0; j < NW; ++j)
            if (j == k)
                w[j] |= v;
    }
};

// position known only at run time: select the word without local memory
template<int NW>
__device__ __forceinline__ void set_bit_dyn(uint32_t (&w)[NW], int pos, bool v) {
    const uint32_t m = (uint32_t)v << (pos & 31);
    const int k = pos >> 5;
#pragma unroll
    for (int j = 0; j < NW; ++j)
        if (j == k)
            w[j] |= m;
}

template<typename T>
__device__ __forceinline__ int ld_px(const StackParams& p, int side, int t, int row, int col) {
    const T* r = reinterpret_cast<const T*>(p.frame[side][t] + (long long)row * p.pitch[side][t]);
    return (int)__ldg(r + col);
}

constexpr int kTfBlock = 256;  // pixels (threads) per CTA of the grid launches

template<int NW>
__device__ __forceinline__ void store_desc(uint32_t* out, const uint32_t (&w)[NW]) {
    if constexpr (NW % 4 == 0) {
        uint4* o = reinterpret_cast<uint4*>(out);
#pragma unroll
        for (int j = 0; j < NW / 4; ++j)
            o[j] = make_uint4(w[4 * j], w[4 * j + 1], w[4 * j + 2], w[4 * j + 3]);
    } else if constexpr (NW == 2) {
        *reinterpret_cast<uint2*>(out) = make_uint2(w[0], w[1]);
    } else {
        out[0] = w[0];
    }
}

// The candidate side's FP8 search tiles, written with the descriptors
// (fp8_tiles.cuh; what k_expand_tiles makes from them otherwise): x the
// side's tiles or null, enc the column-coded form.  Columns past the last
// (up to the tile boundary) repeat the last column's descriptor, as there.
template<int NW>
__device__ __forceinline__ void store_tiles(uint8_t* x, int row, int col, int ntiles, int enc,
                                            const uint32_t (&w)[NW]) {
    if constexpr (NW <= 8) {
        fp8t::Desc<NW> d;
#pragma unroll
        for (int j = 0; j < NW; ++j)
            d.w[j] = w[j];
        if (enc)
            fp8t::expand_candidate<NW, true>(x, row, col, ntiles, d);
        else
            fp8t::expand_candidate<NW, false>(x, row, col, ntiles, d);
    }
}

// extra arguments of the grid kernels for the fused tile output
struct TileOut {
    uint8_t* x0 = nullptr;  // side 0's tiles (searched in direction 1), or null
    uint8_t* x1 = nullptr;  // side 1's tiles (searched in direction 0), or null
    int ntiles = 0;
    int enc = 0;
};

__host__ __device__ constexpr int words_for_bits(int bits) {
    return bits <= 32 ? 1 : bits <= 64 ? 2 : bits <= 128 ? 4 : bits <= 256 ? 8 : ((bits + 127) / 128) * 4;
}

// limited mode: 3 bits per t < n-2 plus a pair-sum bit from t >= 2, 4 tail bits
// block bodies take the block coordinates as arguments, so the same code
// runs as a grid over one stack and inside a persistent multi-stack launch
// (batch.cuh): bx = column block, row, side
// EXACT: the stack has exactly NMAX frames (the top of its word width's
// range, e.g. n = 33 for 128-bit words), so every frame loop has a constant
// trip count and the tail's bit positions are constants too
template<typename T, int NW, int NMAX, bool EXACT = false>
__device__ __forceinline__ void transform_limited(const StackParams& p, uint32_t* __restrict__ d0,
                                                  uint32_t* __restrict__ d1, int bx, int row, int side,
                                                  const TileOut& to = TileOut {}) {
    const int cx = bx * blockDim.x + threadIdx.x;
    uint8_t* const xt = side ? to.x1 : to.x0;
    const bool pad = cx >= p.cols;  // a tile row past the last column
    if (pad && (!xt || cx >= to.ntiles * fp8t::kRows))
        return;
    const int col = pad ? p.cols - 1 : cx;
    const int n = EXACT ? NMAX : p.n;
    // the launchers pick the word width from the bit count 4n - 7, so a
    // stack of this instance has more frames than the next narrower width
    // holds and the frame checks below that count fold away
    constexpr int kNMin = NMAX == 9 ? 2 : NMAX == 17 ? 10 : NMAX == 33 ? 18 : 34;

    int v[NMAX];
    int sum = 0;
#pragma unroll
    for (int t = 0; t < NMAX; ++t) {
        v[t] = (t < kNMin || t < n) ? ld_px<T>(p, side, t, row, col) : 0;
        sum += v[t];
    }
    const float av = __fdiv_rn((float)sum, (float)n);
    const int iav = (int)ceilf(av);  // a < av  <=>  a < ceil(av) for integer a

    BitSink<NW> bs;
    int a = v[0], b = v[1];
    int pp = -1, p1 = -1;  // pair sums of steps t-2 and t-1 (reference's prev_pair_sums ring)
#pragma unroll
    for (int t = 0; t < NMAX - 2; ++t) {
        if (t < kNMin - 2 || t < n - 2) {
            const int c = v[t + 2];
            const int pos = 3 * t + (t >= 2 ? t - 2 : 0);
            bs.push(a - b, pos);
            bs.push(a - c, pos + 1);
            bs.push(a - iav, pos + 2);
            const int cur = a + b;
            if (t >= 2)
                bs.push(pp - cur, pos + 3);
            pp = p1;
            p1 = cur;
            a = b;
            b = c;
        }
    }
    const int pos = 3 * (n - 2) + max(0, n - 4);
    bs.flush_partial(pos);
    set_bit_dyn(bs.w, pos, a < b);
    set_bit_dyn(bs.w, pos + 1, a < iav);
    set_bit_dyn(bs.w, pos + 2, b < iav);
    set_bit_dyn(bs.w, pos + 3, pp < a + b);

    if (!pad)
        store_desc(((side ? d1 : d0) + ((size_t)row * p.cols + col) * NW), bs.w);
    if (xt)
        store_tiles<NW>(xt, row, cx, to.ntiles, to.enc, bs.w);
}

template<typename T, int NW, int NMAX, bool EXACT>
__global__ void __launch_bounds__(kTfBlock) k_transform_limited(const __grid_constant__ StackParams p,
                                                                uint32_t* __restrict__ d0,
                                                                uint32_t* __restrict__ d1, const TileOut to) {
    transform_limited<T, NW, NMAX, EXACT>(p, d0, d1, blockIdx.x, blockIdx.y, blockIdx.z, to);
}

// full mode: 3 bits per t < n-2, 3 tail bits, then every ordered pair of
// non-adjacent pair sums; n is a template parameter so every position is
// a constant
template<typename T, int N>
__device__ __forceinline__ void transform_full(const StackParams& p, uint32_t* __restrict__ d0,
                                               uint32_t* __restrict__ d1, int bx, int row, int side,
                                               const TileOut& to = TileOut {}) {
    constexpr int NW = words_for_bits(N * N - 2 * N + 3);
    const int cx = bx * blockDim.x + threadIdx.x;
    uint8_t* const xt = side ? to.x1 : to.x0;
    const bool pad = cx >= p.cols;  // a tile row past the last column
    if (pad && (!xt || cx >= to.ntiles * fp8t::kRows))
        return;
    const int col = pad ? p.cols - 1 : cx;

    int v[N];
    int sum = 0;
#pragma unroll
    for (int t = 0; t < N; ++t) {
        v[t] = ld_px<T>(p, side, t, row, col);
        sum += v[t];
    }
    const float av = __fdiv_rn((float)sum, (float)N);
    const int iav = (int)ceilf(av);

    BitSink<NW> bs;
    int ps[N - 1];
    int pos = 0;
#pragma unroll
    for (int t = 0; t < N - 2; ++t) {
        bs.push(v[t] - v[t + 1], pos++);
        bs.push(v[t] - v[t + 2], pos++);
        bs.push(v[t] - iav, pos++);
    }
#pragma unroll
    for (int t = 0; t < N - 1; ++t)
        ps[t] = v[t] + v[t + 1];
    bs.push(v[N - 2] - v[N - 1], pos++);
    bs.push(v[N - 2] - iav, pos++);
    bs.push(v[N - 1] - iav, pos++);
#pragma unroll
    for (int t = 0; t < N - 1; ++t)
#pragma unroll
        for (int i = 0; i < N - 1; ++i) {
            if (i == t || i == t - 1 || i == t + 1)
                continue;
            bs.push(ps[t] - ps[i], pos++);
        }
    bs.flush_partial(pos);

    if (!pad)
        store_desc(((side ? d1 : d0) + ((size_t)row * p.cols + col) * NW), bs.w);
    if (xt)
        store_tiles<NW>(xt, row, cx, to.ntiles, to.enc, bs.w);
}

template<typename T, int N>
__global__ void __launch_bounds__(kTfBlock) k_transform_full(const __grid_constant__ StackParams p,
                                                             uint32_t* __restrict__ d0,
                                                             uint32_t* __restrict__ d1, const TileOut to) {
    transform_full<T, N>(p, d0, d1, blockIdx.x, blockIdx.y, blockIdx.z, to);
}

// persistent multi-stack forms (batch.cuh)
template<typename T, int NW, int NMAX>
struct TfLimitedOp {
    using P = TransformJob;
    static constexpr int kMaxThreads = 256;
    static constexpr int kMinBlocks = NW <= 2 ? 8 : NW == 4 ? 4 : 2;
    static __device__ __forceinline__ void run(const P& q, int bx, int row, int side) {
        transform_limited<T, NW, NMAX>(q.s, q.d0, q.d1, bx, row, side);
    }
};
template<typename T, int N>
struct TfFullOp {
    using P = TransformJob;
    static constexpr int kMaxThreads = 256;
    static constexpr int kMinBlocks = 4;
    static __device__ __forceinline__ void run(const P& q, int bx, int row, int side) {
        transform_full<T, N>(q.s, q.d0, q.d1, bx, row, side);
    }
};

template<typename T>
using tf_kernel_t = void (*)(StackParams, uint32_t*, uint32_t*, TileOut);

template<typename T>
tf_kernel_t<T> pick_full(int n) {
    switch (n) {
#define BICOS_FULL_CASE(N) \
    case N: return k_transform_full<T, N>;
        BICOS_FULL_CASE(2) BICOS_FULL_CASE(3) BICOS_FULL_CASE(4) BICOS_FULL_CASE(5)
        BICOS_FULL_CASE(6) BICOS_FULL_CASE(7) BICOS_FULL_CASE(8) BICOS_FULL_CASE(9)
        BICOS_FULL_CASE(10) BICOS_FULL_CASE(11) BICOS_FULL_CASE(12) BICOS_FULL_CASE(13)
        BICOS_FULL_CASE(14) BICOS_FULL_CASE(15) BICOS_FULL_CASE(16) BICOS_FULL_CASE(17)
        BICOS_FULL_CASE(18) BICOS_FULL_CASE(19) BICOS_FULL_CASE(20) BICOS_FULL_CASE(21)
        BICOS_FULL_CASE(22) BICOS_FULL_CASE(23)
#undef BICOS_FULL_CASE
        default: return nullptr;
    }
}

template<typename T>
tf_kernel_t<T> pick_limited(int nwords, int n) {
    switch (nwords) {
        case 1: return n == 9 ? k_transform_limited<T, 1, 9, true> : k_transform_limited<T, 1, 9, false>;
        case 2: return n == 17 ? k_transform_limited<T, 2, 17, true> : k_transform_limited<T, 2, 17, false>;
        case 4: return n == 33 ? k_transform_limited<T, 4, 33, true> : k_transform_limited<T, 4, 33, false>;
        case 8: return n == 65 ? k_transform_limited<T, 8, 65, true> : k_transform_limited<T, 8, 65, false>;
        default: return nullptr;
    }
}

}  // namespace

cudaError_t launch_transform(const StackParams& p, int sides, bool full, int nwords, uint32_t* desc0,
                             uint32_t* desc1, cudaStream_t st, uint8_t* tiles0, uint8_t* tiles1, int bits) {
    void (*k)(StackParams, uint32_t*, uint32_t*, TileOut) = nullptr;
    if (full) {
        if (words_for_bits(p.n * p.n - 2 * p.n + 3) != nwords)
            return cudaErrorInvalidValue;
        k = p.elem_bytes == 1 ? pick_full<uint8_t>(p.n) : pick_full<uint16_t>(p.n);
    } else {
        if (words_for_bits(4 * p.n - 7) != nwords)
            return cudaErrorInvalidValue;
        k = p.elem_bytes == 1 ? pick_limited<uint8_t>(nwords, p.n) : pick_limited<uint16_t>(nwords, p.n);
    }
    if (!k)
        return cudaErrorInvalidValue;
    TileOut to;
    if ((tiles0 || tiles1) && nwords <= 8) {
        to.x0 = tiles0;
        to.x1 = sides > 1 ? tiles1 : nullptr;
        to.ntiles = (p.cols + fp8t::kRows - 1) / fp8t::kRows;
        to.enc = bits >= 1 && bits <= 32 * nwords - 2;  // the search's column-coded form
    }
    const dim3 block(kTfBlock);
    const dim3 grid((p.cols + kTfBlock - 1) / kTfBlock, p.rows, sides);
    k<<<grid, block, 0, st>>>(p, desc0, desc1, to);
    return cudaGetLastError();
}

namespace {
template<typename T>
cudaError_t transform_batch_t(bool full, int key, const BatchArgs<TransformJob>& a, const BatchLaunch& l,
                              cudaStream_t st) {
    if (full) {
        switch (key) {
#define BICOS_FULL_CASE(N) \
    case N: return launch_batch_op<TfFullOp<T, N>>(a, l, 0, st);
            BICOS_FULL_CASE(2) BICOS_FULL_CASE(3) BICOS_FULL_CASE(4) BICOS_FULL_CASE(5)
            BICOS_FULL_CASE(6) BICOS_FULL_CASE(7) BICOS_FULL_CASE(8) BICOS_FULL_CASE(9)
            BICOS_FULL_CASE(10) BICOS_FULL_CASE(11) BICOS_FULL_CASE(12) BICOS_FULL_CASE(13)
            BICOS_FULL_CASE(14) BICOS_FULL_CASE(15) BICOS_FULL_CASE(16) BICOS_FULL_CASE(17)
            BICOS_FULL_CASE(18) BICOS_FULL_CASE(19) BICOS_FULL_CASE(20) BICOS_FULL_CASE(21)
            BICOS_FULL_CASE(22) BICOS_FULL_CASE(23)
#undef BICOS_FULL_CASE
            default: return cudaErrorInvalidValue;
        }
    }
    switch (key) {
        case 1: return launch_batch_op<TfLimitedOp<T, 1, 9>>(a, l, 0, st);
        case 2: return launch_batch_op<TfLimitedOp<T, 2, 17>>(a, l, 0, st);
        case 4: return launch_batch_op<TfLimitedOp<T, 4, 33>>(a, l, 0, st);
        case 8: return launch_batch_op<TfLimitedOp<T, 8, 65>>(a, l, 0, st);
        default: return cudaErrorInvalidValue;
    }
}
}  // namespace

cudaError_t launch_transform_batch(int elem_bytes, bool full, int key, const BatchArgs<TransformJob>& a,
                                   const BatchLaunch& l, cudaStream_t st) {
    return elem_bytes == 1 ? transform_batch_t<uint8_t>(full, key, a, l, st)
                           : transform_batch_t<uint16_t>(full, key, a, l, st);
}

}  // namespace bicos_gb300
