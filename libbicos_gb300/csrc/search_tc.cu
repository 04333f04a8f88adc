// Row-wise Hamming arg-min on the 5th-generation tensor cores (stage b).
//
// Hamming distance as a dot product: with every descriptor bit mapped to
// +1 (set) or -1 (clear), dot(a, b) = K - 2 * ham(a, b) for K-bit words, so
// the minimum Hamming distance is the maximum dot product.  Per CTA:
//   A = 128 query descriptors of one row (TMEM lanes), B = 128 candidate
//   descriptors per tile, both expanded to FP8 e4m3 (+1 = 0x38, -1 = 0xB8)
//   in shared memory in the canonical no-swizzle K-major layout;
//   tcgen05.mma kind::f8f6f4 (M=128, N=128, K=32 per instruction) writes
//   D = A * B^T to TMEM with FP32 accumulation (exact: |D| <= K <= 512);
//   the epilogue reads D back with tcgen05.ld (thread = query pixel) and
//   keeps the two largest keys  key = dot - col * 2^-12  (exact in FP32 for
//   cols <= 4096), which carry the first arg-max and the tie test of
//   libBICOS's bicos_search (include/impl/cpu/bicos.hpp:50-76).
// Column-coded form (descriptors using at most 32*NW-2 bit positions, the
// match path's): the two top K slots of every row are padding, so they
// carry the candidate's column within its pair of tiles (c = 0..255)
// instead, and the MMA itself yields
//   D = 128 * dot' - c   (dot' = the sum over the other 32*NW-2 slots,
//   even; descriptor slots +-16 (queries) x +-8 (candidates), code slots
//   -1, -16 in the query row against c's two nibbles in the candidate row)
// -- the first-arg-max key within a tile pair with no per-candidate
// arithmetic (integers below 2^17, exact in the FP32 accumulator).  The
// epilogue decodes each tile's maxima into global keys (8192 e -/+ column)
// once per tile.  The candidate tiles arrive pre-expanded in global memory
// (written by the transform, or by k_expand_tiles) for words up to 256
// bits, else producer warps expand them in every CTA.
// Outputs and semantics are those of k_search (search.cu).  All waits are
// bounded: a wait that runs out records a fault, and the CTA frees its TMEM
// and exits.
#include <climits>
#include <type_traits>

#include "fp8_tiles.cuh"
#include "kernels.cuh"
#include "tcgen05.cuh"

namespace bicos_gb300 {

__device__ unsigned int g_tc_faults = 0;

namespace {

using namespace tc;
using namespace fp8t;

constexpr float kColScale = 1.0f / 4096.0f;
constexpr int kMaxCols = 4096;      // key exactness bound

constexpr uint32_t kIdesc = tc::idesc_f8_e4m3(kRows, kRows);

// three-input max (sm_100+): one ALU instruction
__device__ __forceinline__ float fmax3(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Row reduction over the candidates' dot products (dot = bits - 2 *
// Hamming, integer-valued).  Chain A keeps max(dot - col/4096): the largest
// dot at its first column, the reference's first minimum.  Chain B (only
// with no-duplicates) keeps max(dot + col/4096): the same dot at its last
// column; the minimum cost is duplicated exactly when the two columns
// differ, which is the reference's no-duplicates rule (a later column with
// the same cost).  All keys are exact in FP32 (|dot| <= 512, offsets
// multiples of 2^-12 below 1).  Per pair of candidates: 2 (or 4) FADDs with
// immediate offsets on the FMA pipe and 1 (or 2) three-input maxima on the
// ALU pipe.
template<bool NODUP, bool MASKED>
__device__ __forceinline__ void reduce_chunk(const float (&v)[32], int j0, int lim, float& mA, float& mB) {
    float ca[4], cb[4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
        ca[i] = cb[i] = -INFINITY;
#pragma unroll
    for (int k = 0; k < 32; k += 2) {
        const float va = v[k], vb = v[k + 1];
        float a = va - (float)k * kColScale;
        float b = vb - (float)(k + 1) * kColScale;
        float a2 = va + (float)k * kColScale;
        float b2 = vb + (float)(k + 1) * kColScale;
        if constexpr (MASKED) {
            a = k < lim ? a : -INFINITY;
            b = k + 1 < lim ? b : -INFINITY;
            a2 = k < lim ? a2 : -INFINITY;
            b2 = k + 1 < lim ? b2 : -INFINITY;
        }
        const int i = (k >> 1) & 3;
        ca[i] = fmax3(ca[i], a, b);
        if constexpr (NODUP)
            cb[i] = fmax3(cb[i], a2, b2);
    }
    const float off = (float)j0 * kColScale;
    mA = fmax3(mA, fmax3(ca[0], ca[1], ca[2]) - off, ca[3] - off);
    if constexpr (NODUP)
        mB = fmax3(mB, fmax3(cb[0], cb[1], cb[2]) + off, cb[3] + off);
}

// The same reduction over column-coded keys (D = 128 * dot' - c, c the
// column within the tile pair, v[j] at c = c0 + j): chain A is the plain
// maximum of D; chain B (with no-duplicates) keeps max(D + 2c) =
// 128 * dot' + c.  Per pair of candidates: 1 three-input maximum, plus
// (no-duplicates) 2 FADDs and 1 more maximum.
template<bool NODUP, bool MASKED>
__device__ __forceinline__ void reduce_chunk_coded(const float (&v)[32], int c0, int lim, float& kA, float& kB) {
    float ca[4], cb[4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
        ca[i] = cb[i] = -INFINITY;
#pragma unroll
    for (int k = 0; k < 32; k += 2) {
        float a = v[k], b = v[k + 1];
        float a2 = a + (float)(2 * k);
        float b2 = b + (float)(2 * k + 2);
        if constexpr (MASKED) {
            a = k < lim ? a : -INFINITY;
            b = k + 1 < lim ? b : -INFINITY;
            a2 = k < lim ? a2 : -INFINITY;
            b2 = k + 1 < lim ? b2 : -INFINITY;
        }
        const int i = (k >> 1) & 3;
        ca[i] = fmax3(ca[i], a, b);
        if constexpr (NODUP)
            cb[i] = fmax3(cb[i], a2, b2);
    }
    kA = fmax3(kA, fmax3(ca[0], ca[1], ca[2]), ca[3]);
    if constexpr (NODUP) {
        const float off = (float)(2 * c0);
        kB = fmax3(kB, fmax3(cb[0], cb[1], cb[2]) + off, cb[3] + off);
    }
}

// one tile pair's chain-A maximum (D = 256 e - c) -> global key
// 8192 e - (256 * pair + c), merged into gA; chain B (D + 2c = 256 e + c)
// -> 8192 e + (256 * pair + c) into gB
__device__ __forceinline__ void decode_a(float& kA, int pair, int& gA) {
    if (kA > -INFINITY) {
        const int a = (int)kA;
        const int c = (-a) & 255;
        gA = max(gA, ((a + c) >> 8) * 8192 - (pair * 256 + c));
    }
    kA = -INFINITY;
}
__device__ __forceinline__ void decode_b(float& kB, int pair, int& gB) {
    if (kB > -INFINITY) {
        const int b = (int)kB;
        const int c = b & 255;
        gB = max(gB, ((b - c) >> 8) * 8192 + (pair * 256 + c));
    }
    kB = -INFINITY;
}

// Warp roles of the pipelined CTA (one CTA = one row x 128 query pixels;
// the MMA and producer waits back off between polls, the epilogue's do not):
//   warps 0..7   epilogue: warp w reads TMEM lane quarter w%4; column-coded
//                form: warps 0..3 the even tiles, 4..7 the odd ones, all
//                128 columns; plain form: columns [64*(w/4), 64*(w/4)+64)
//                of every tile; in the pre-expanded form warps 0..3 first
//                expand the A tile (query row = thread), idle as they are
//                until the first accumulator is full
//   producers    in-kernel form (4 warps): thread p expands candidate row p
//                of each tile into the FP8 ring (and query row p into the
//                A tile); pre-expanded form (1 warp): one lane moves each
//                candidate tile, already in FP8 in global memory
//                (k_expand_tiles), into the ring with one bulk copy
//   last warp    MMA issue (one lane)
// A ring of smem B buffers and two TMEM accumulators (2 x 128 columns) let
// the producers run ahead of the tensor core, which runs one tile ahead of
// the epilogue.
constexpr int kEpiWarps = 8;
template<bool PRE>
__host__ __device__ constexpr int prod_warps() { return PRE ? 1 : 4; }
template<bool PRE>
__host__ __device__ constexpr int threads_tc() { return 32 * (kEpiWarps + prod_warps<PRE>() + 1); }
constexpr int kAccCols = kRows;

constexpr int kMaxStages = 5;

// B ring depth: in-kernel expansion 4 (words up to 128 bits) or 2; bulk
// copies from L2 have a longer latency to cover, so 5 tiles of 16 KB (two
// CTAs per SM within the 228 KB) or, for wider words, as many as fit
template<int NW, bool PRE>
__host__ __device__ constexpr int b_stages() {
    return PRE ? (NW <= 4 ? 5 : NW <= 8 ? 2 : 1) : (NW <= 4 ? 4 : 2);
}

struct TcShared {
    uint64_t full_b[kMaxStages];   // producers -> MMA (128 arrivals, or 1 + transaction bytes)
    uint64_t b_empty[kMaxStages];  // MMA commit -> producers (slot read)
    uint64_t a_full;               // A tile written (128 arrivals)
    uint64_t acc_full[2];   // MMA commit -> epilogue / producers
    uint64_t acc_empty[2];  // epilogue -> MMA, 256 arrivals
    uint32_t tmem;
    int abort;
    float2 red[kRows];      // second column half's (chain A, chain B) maxima per query
};

// Candidate descriptors -> FP8 tiles in global memory, in the B ring's
// shared-memory layout (tile t of row r at xt + (r * ntiles + t) * TILE),
// with the candidate clear pattern and, in the column-coded form, the
// column code; rows past the last column repeat it (the epilogue masks
// them).  One CTA of 128 threads per tile; each warp stores 512
// contiguous bytes per 16-byte K chunk.
template<int NW, bool ENC>
__global__ void __launch_bounds__(kRows) k_expand_tiles(const uint32_t* __restrict__ d, int cols, int ntiles,
                                                         uint8_t* __restrict__ xt) {
    constexpr int TILE = kRows * NW * 32;
    const int t = blockIdx.x, row = blockIdx.y, p = threadIdx.x;
    const int c = min(t * kRows + p, cols - 1);
    const Desc<NW> v = load_desc<NW>(d + ((size_t)row * cols + c) * NW);
    expand_desc<NW, ENC>(xt + ((size_t)row * ntiles + t) * TILE, p, v, ENC ? kClearCand : kClearPlain,
                         ENC ? column_code((t & 1) * kRows + p) : 0u);
}

template<int NW, bool NODUP, bool ENC, bool PRE>
__global__ void __launch_bounds__(threads_tc<PRE>(), 2) k_search_tc(const uint32_t* __restrict__ d0,
                                                                   const uint32_t* __restrict__ d1, int rows, int cols,
                                                                   int16_t* __restrict__ disp, long long disp_pitch,
                                                                   int32_t* __restrict__ best0,
                                                                   int32_t* __restrict__ best1,
                                                                   const uint8_t* __restrict__ x0,
                                                                   const uint8_t* __restrict__ x1) {
    constexpr int KB = NW * 32;       // FP8 elements (bytes) per descriptor
    constexpr int TILE = kRows * KB;  // bytes of one 128-row tile
    constexpr int KSTEPS = KB / 32;   // MMA K = 32 bytes per instruction
    constexpr int STAGES = b_stages<NW, PRE>();
    constexpr int PROD = prod_warps<PRE>();
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* sA = smem;
    uint8_t* sB = smem + TILE;  // STAGES buffers
    __shared__ TcShared sh;
    volatile int* abort = &sh.abort;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int row = blockIdx.y, dir = blockIdx.z;
    const int m0 = blockIdx.x * kRows;
    const size_t row_off = (size_t)row * cols * NW;
    const uint32_t* qrow = (dir ? d1 : d0) + row_off;
    const uint32_t* crow = (dir ? d0 : d1) + row_off;
    const int ntiles = (cols + kRows - 1) / kRows;

    if (warp == 0) {
        tmem_alloc(smem_u32(&sh.tmem), 2 * kAccCols);
        tmem_relinquish();
    }
    if (tid == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(smem_u32(&sh.full_b[s]), PRE ? 1 : 32 * PROD);
            mbar_init(smem_u32(&sh.b_empty[s]), 1);
        }
        mbar_init(smem_u32(&sh.a_full), kRows);
        for (int b = 0; b < 2; ++b) {
            mbar_init(smem_u32(&sh.acc_full[b]), 1);
            // column-coded form: one group of four epilogue warps per
            // accumulator; plain form: all eight warps on every tile
            mbar_init(smem_u32(&sh.acc_empty[b]), ENC ? 16 * kEpiWarps : 32 * kEpiWarps);
        }
        sh.abort = 0;
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = sh.tmem;

    if (warp >= kEpiWarps + PROD) {
        // ---- MMA issue ----
        if (lane == 0) {
            const uint32_t a_addr = smem_u32(sA);
            int issued = -1;
            const bool a_ok = !PRE || wait_or_abort<32>(smem_u32(&sh.a_full), 0, abort);
            for (int t = 0; t < ntiles && a_ok; ++t) {
                const int b = t & 1, slot = t % STAGES;
                if (!wait_or_abort<32>(smem_u32(&sh.full_b[slot]), (t / STAGES) & 1, abort))
                    break;
                if (t >= 2 && !wait_or_abort<32>(smem_u32(&sh.acc_empty[b]), ((t >> 1) - 1) & 1, abort))
                    break;
                fence_after();
                const uint32_t b_addr = smem_u32(sB + slot * TILE);
#pragma unroll
                for (int s = 0; s < KSTEPS; ++s)
                    mma_f8f6f4(tmem + b * kAccCols, smem_desc(a_addr + s * 2 * kChunkBytes, kChunkBytes, 128),
                               smem_desc(b_addr + s * 2 * kChunkBytes, kChunkBytes, 128), kIdesc,
                               s > 0 ? 1u : 0u);
                mma_commit(smem_u32(&sh.acc_full[b]));
                mma_commit(smem_u32(&sh.b_empty[slot]));
                issued = t;
            }
            if (issued >= 0 && *abort)  // let the last MMA land before TMEM is freed
                wait_drain(smem_u32(&sh.acc_full[issued & 1]), (issued >> 1) & 1);
        }
    } else if (warp >= kEpiWarps) {
        // ---- producers ----
        const int p = tid - 32 * kEpiWarps;
        if constexpr (PRE) {
            // the A tile comes from the epilogue warps (idle until the first
            // accumulator is full); this warp starts the copies at once
            if (lane == 0) {
                const uint8_t* src = (dir ? x0 : x1) + (size_t)row * ntiles * TILE;
                int issued = -1;
                for (int t = 0; t < ntiles; ++t) {
                    const int slot = t % STAGES;
                    if (t >= STAGES &&
                        !wait_or_abort<64>(smem_u32(&sh.b_empty[slot]), (t / STAGES - 1) & 1, abort))
                        break;
                    mbar_arrive_expect_tx(smem_u32(&sh.full_b[slot]), TILE);
                    bulk_g2s(smem_u32(sB + slot * TILE), src + (size_t)t * TILE, TILE, smem_u32(&sh.full_b[slot]));
                    issued = t;
                }
                if (*abort)  // copies still in flight land before the CTA leaves
                    for (int t = max(0, issued - STAGES + 1); t <= issued; ++t)
                        wait_drain(smem_u32(&sh.full_b[t % STAGES]), (t / STAGES) & 1);
            }
        } else {
            // a register ring keeps the descriptors of the next PF tiles in flight
            constexpr int PF = NW <= 4 ? 4 : 2;
            auto cand = [&](int t) {
                return load_desc<NW>(crow + (size_t)min(min(t, ntiles - 1) * kRows + p, cols - 1) * NW);
            };
            Desc<NW> ring[PF];
#pragma unroll
            for (int i = 0; i < PF; ++i)
                ring[i] = cand(i);
            expand_desc<NW, ENC>(sA, p, load_desc<NW>(qrow + (size_t)min(m0 + p, cols - 1) * NW),
                                 ENC ? kClearQuery : kClearPlain, kQueryCode);
            bool live = true;
            for (int t0 = 0; t0 < ntiles && live; t0 += PF) {
#pragma unroll
                for (int i = 0; i < PF; ++i) {
                    const int t = t0 + i;
                    if (t >= ntiles)
                        break;
                    const Desc<NW> cur = ring[i];
                    ring[i] = cand(t + PF);
                    const int slot = t % STAGES;
                    if (t >= STAGES &&
                        !wait_or_abort<64>(smem_u32(&sh.b_empty[slot]), (t / STAGES - 1) & 1, abort)) {
                        live = false;
                        break;
                    }
                    expand_desc<NW, ENC>(sB + slot * TILE, p, cur, ENC ? kClearCand : kClearPlain,
                                         ENC ? column_code((t & 1) * kRows + p) : 0u);
                    fence_async_smem();
                    mbar_arrive(smem_u32(&sh.full_b[slot]));
                }
            }
        }
    } else {
        // ---- epilogue ----
        if constexpr (PRE) {
            // pre-expanded form: the first four epilogue warps expand the
            // A tile (one query row per thread) before the first result
            if (tid < kRows) {
                expand_desc<NW, ENC>(sA, tid, load_desc<NW>(qrow + (size_t)min(m0 + tid, cols - 1) * NW),
                                     ENC ? kClearQuery : kClearPlain, kQueryCode);
                fence_async_smem();
                mbar_arrive(smem_u32(&sh.a_full));
            }
        }
        // column-coded form: warps 0..3 take the even tiles, warps 4..7 the
        // odd ones, each warp all 128 columns of its lane quarter (so the
        // per-tile waits, loads and decodes are paid once per 128
        // columns); plain form: warp w reads lane quarter w%4, columns
        // [64*(w/4), 64*(w/4)+64) of every tile
        const int q = warp & 3, half = warp >> 2;
        const uint32_t lane_addr = tmem + ((uint32_t)(q * 32) << 16) + (ENC ? 0 : half * 64);
        float mA = -INFINITY, mB = -INFINITY;
        int gA = INT_MIN, gB = INT_MIN;  // column-coded form: global keys
        bool ok = true;
        // column-coded maxima of 64 columns [j0, j0 + 64) of tile u: both
        // 32-column loads in flight before one wait
        auto coded_max64 = [&](int u, int r, uint32_t acc) {
            const int j0 = u * kRows + r * 64, c0 = (u & 1) * kRows + r * 64;
            if (cols - j0 >= 64) {
                uint32_t r0[32], r1[32];
                tmem_ld32_async(acc, r0);
                tmem_ld32_async(acc + 32, r1);
                tmem_wait_ld();
                tmem_hold(r0);
                tmem_hold(r1);
                float v[32];
#pragma unroll
                for (int j = 0; j < 32; ++j)
                    v[j] = __uint_as_float(r0[j]);
                reduce_chunk_coded<NODUP, false>(v, c0, 32, mA, mB);
#pragma unroll
                for (int j = 0; j < 32; ++j)
                    v[j] = __uint_as_float(r1[j]);
                reduce_chunk_coded<NODUP, false>(v, c0 + 32, 32, mA, mB);
            } else {
#pragma unroll
                for (int ch = 0; ch < 2; ++ch) {
                    if (j0 + ch * 32 < cols) {
                        float v[32];
                        tmem_ld32(acc + ch * 32, v);
                        reduce_chunk_coded<NODUP, true>(v, c0 + ch * 32, cols - j0 - ch * 32, mA, mB);
                    }
                }
            }
        };
        if constexpr (ENC && NODUP) {
            // column-coded, no-duplicates: one instance per group (tile
            // parity P), so every candidate's column code c = 128 P + j is a
            // constant and chain B's D + 2c an addition of an immediate; the
            // partial maxima run across the whole tile
            auto run_group = [&](auto par) {
                constexpr int P = decltype(par)::value;
                const uint32_t acc = lane_addr + P * kAccCols;
                for (int t = P; t < ntiles && ok; t += 2) {
                    ok = wait_or_abort(smem_u32(&sh.acc_full[P]), (t >> 1) & 1, abort);
                    ok = __all_sync(0xffffffffu, ok);
                    if (!ok)
                        break;
                    fence_after();
                    if (t * kRows + kRows <= cols) {
                        float ca[4], cb[4];
#pragma unroll
                        for (int i = 0; i < 4; ++i)
                            ca[i] = cb[i] = -INFINITY;
#pragma unroll
                        for (int r = 0; r < 2; ++r) {
                            uint32_t r0[32], r1[32];
                            tmem_ld32_async(acc + r * 64, r0);
                            tmem_ld32_async(acc + r * 64 + 32, r1);
                            tmem_wait_ld();
                            tmem_hold(r0);
                            tmem_hold(r1);
                            auto chunk = [&](const uint32_t (&rv)[32], int c0) {
#pragma unroll
                                for (int k = 0; k < 32; k += 2) {
                                    const float a = __uint_as_float(rv[k]), bb = __uint_as_float(rv[k + 1]);
                                    const int c = c0 + k;  // a constant after unrolling
                                    const int i = (k >> 1) & 3;
                                    ca[i] = fmax3(ca[i], a, bb);
                                    cb[i] = fmax3(cb[i], a + (float)(2 * c), bb + (float)(2 * c + 2));
                                }
                            };
                            chunk(r0, P * kRows + r * 64);
                            chunk(r1, P * kRows + r * 64 + 32);
                        }
                        mA = fmax3(mA, fmax3(ca[0], ca[1], ca[2]), ca[3]);
                        mB = fmax3(mB, fmax3(cb[0], cb[1], cb[2]), cb[3]);
                    } else {
                        coded_max64(t, 0, acc);
                        if (t * kRows + 64 < cols)
                            coded_max64(t, 1, acc + 64);
                    }
                    fence_before();
                    mbar_arrive(smem_u32(&sh.acc_empty[P]));
                    decode_a(mA, t >> 1, gA);
                    decode_b(mB, t >> 1, gB);
                }
            };
            if (half == 0)
                run_group(std::integral_constant<int, 0> {});
            else
                run_group(std::integral_constant<int, 1> {});
        } else if constexpr (ENC) {
            for (int t = half; t < ntiles && ok; t += 2) {
                const int b = t & 1;
                ok = wait_or_abort(smem_u32(&sh.acc_full[b]), (t >> 1) & 1, abort);
                ok = __all_sync(0xffffffffu, ok);
                if (!ok)
                    break;
                fence_after();
                coded_max64(t, 0, lane_addr + b * kAccCols);
                if (t * kRows + 64 < cols)
                    coded_max64(t, 1, lane_addr + b * kAccCols + 64);
                fence_before();
                mbar_arrive(smem_u32(&sh.acc_empty[b]));
                decode_a(mA, t >> 1, gA);
                if constexpr (NODUP)
                    decode_b(mB, t >> 1, gB);
            }
        } else {
            for (int t = 0; t < ntiles && ok; ++t) {
                const int b = t & 1;
                ok = wait_or_abort(smem_u32(&sh.acc_full[b]), (t >> 1) & 1, abort);
                ok = __all_sync(0xffffffffu, ok);
                if (!ok)
                    break;
                fence_after();
#pragma unroll
                for (int ch = 0; ch < 2; ++ch) {
                    const int j0 = t * kRows + half * 64 + ch * 32;
                    if (j0 < cols) {
                        float v[32];
                        tmem_ld32(lane_addr + b * kAccCols + ch * 32, v);
                        if (cols - j0 >= 32)
                            reduce_chunk<NODUP, false>(v, j0, 32, mA, mB);
                        else
                            reduce_chunk<NODUP, true>(v, j0, cols - j0, mA, mB);
                    }
                }
                fence_before();
                mbar_arrive(smem_u32(&sh.acc_empty[b]));
            }
        }
        if (half == 1) {
            if constexpr (ENC)
                sh.red[q * 32 + lane] = make_float2(__int_as_float(gA), __int_as_float(gB));
            else
                sh.red[q * 32 + lane] = make_float2(mA, mB);
        }
        asm volatile("bar.sync 1, %0;" ::"r"(32 * kEpiWarps) : "memory");
        const int c = m0 + q * 32 + lane;
        if (half == 0 && *abort && c < cols) {
            // the CTA gave up: no match rather than stale outputs
            if (disp) {
                int16_t* o = reinterpret_cast<int16_t*>(reinterpret_cast<char*>(disp) + row * disp_pitch);
                o[c] = kInvalidDisp;
            } else {
                (dir ? best1 : best0)[(size_t)row * cols + c] = -1;
            }
        } else if (half == 0 && c < cols) {
            const float2 r = sh.red[q * 32 + lane];
            int best;
            bool valid;
            if constexpr (ENC) {
                gA = max(gA, __float_as_int(r.x));
                gB = max(gB, __float_as_int(r.y));
                best = (-gA) & 8191;
                valid = !NODUP || (gB & 8191) == best;
            } else {
                mA = fmaxf(mA, r.x);
                mB = fmaxf(mB, r.y);
                best = (int)((ceilf(mA) - mA) * 4096.0f);
                valid = !NODUP || (int)((mB - floorf(mB)) * 4096.0f) == best;
            }
            if (disp) {
                int16_t* o = reinterpret_cast<int16_t*>(reinterpret_cast<char*>(disp) + row * disp_pitch);
                o[c] = valid ? (int16_t)(c - best) : kInvalidDisp;
            } else {
                (dir ? best1 : best0)[(size_t)row * cols + c] = valid ? best : -1;
            }
        }
    }

    fence_before();
    __syncthreads();
    if (tid == 0 && *abort)
        atomicAdd(&g_tc_faults, 1u);
    if (warp == 0) {
        fence_after();
        tmem_dealloc(tmem, 2 * kAccCols);
    }
}

template<int NW, bool PRE>
constexpr size_t tc_smem() {
    // A tile and B ring; at least 80 KB per CTA: at most 2 CTAs (2 x 256
    // TMEM columns) per SM
    return (size_t)(1 + b_stages<NW, PRE>()) * kRows * NW * 32 > (size_t)80 * 1024
               ? (size_t)(1 + b_stages<NW, PRE>()) * kRows * NW * 32
               : (size_t)80 * 1024;
}

template<int NW, bool NODUP>
cudaError_t launch_tc_nw(const uint32_t* d0, const uint32_t* d1, int rows, int cols, int bits, int dirs,
                         int16_t* disp, long long disp_pitch, int32_t* b0, int32_t* b1, uint8_t* xbuf,
                         cudaStream_t st, bool ready) {
    constexpr int TILE = kRows * NW * 32;
    // column-coded when the two top K slots are padding
    const bool enc = bits >= 1 && bits <= 32 * NW - 2;
    const dim3 grid((cols + kRows - 1) / kRows, rows, dirs);
    cudaError_t e;
    if (xbuf && NW <= 8) {
        // candidate sides expanded once: direction 0 searches d1, direction 1 d0
        const int ntiles = (cols + kRows - 1) / kRows;
        const size_t side = (size_t)rows * ntiles * TILE;
        uint8_t* x1 = xbuf;
        uint8_t* x0 = dirs > 1 ? xbuf + side : nullptr;
        const dim3 xg(ntiles, rows);
        if (!ready) {
            auto xk = enc ? k_expand_tiles<NW, true> : k_expand_tiles<NW, false>;
            xk<<<xg, kRows, 0, st>>>(d1, cols, ntiles, x1);
            if (dirs > 1)
                xk<<<xg, kRows, 0, st>>>(d0, cols, ntiles, x0);
        }
        auto k = enc ? k_search_tc<NW, NODUP, true, true> : k_search_tc<NW, NODUP, false, true>;
        constexpr size_t smem = tc_smem<NW, true>();
        if ((e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
            return e;
        k<<<grid, threads_tc<true>(), smem, st>>>(d0, d1, rows, cols, disp, disp_pitch, b0, b1, x0, x1);
    } else {
        auto k = enc ? k_search_tc<NW, NODUP, true, false> : k_search_tc<NW, NODUP, false, false>;
        constexpr size_t smem = tc_smem<NW, false>();
        if ((e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
            return e;
        k<<<grid, threads_tc<false>(), smem, st>>>(d0, d1, rows, cols, disp, disp_pitch, b0, b1, nullptr, nullptr);
    }
    return cudaGetLastError();
}

template<bool NODUP>
cudaError_t launch_tc_dup(const uint32_t* d0, const uint32_t* d1, int rows, int cols, int nwords, int bits,
                          int dirs, int16_t* disp, long long disp_pitch, int32_t* b0, int32_t* b1, uint8_t* xbuf,
                          cudaStream_t st, bool ready) {
    switch (nwords) {
        case 1:
            return launch_tc_nw<1, NODUP>(d0, d1, rows, cols, bits, dirs, disp, disp_pitch, b0, b1, xbuf, st,
                                             ready);
        case 2:
            return launch_tc_nw<2, NODUP>(d0, d1, rows, cols, bits, dirs, disp, disp_pitch, b0, b1, xbuf, st,
                                             ready);
        case 4:
            return launch_tc_nw<4, NODUP>(d0, d1, rows, cols, bits, dirs, disp, disp_pitch, b0, b1, xbuf, st,
                                             ready);
        case 8:
            return launch_tc_nw<8, NODUP>(d0, d1, rows, cols, bits, dirs, disp, disp_pitch, b0, b1, xbuf, st,
                                             ready);
        case 12:
            return launch_tc_nw<12, NODUP>(d0, d1, rows, cols, bits, dirs, disp, disp_pitch, b0, b1, xbuf, st,
                                             ready);
        case 16:
            return launch_tc_nw<16, NODUP>(d0, d1, rows, cols, bits, dirs, disp, disp_pitch, b0, b1, xbuf, st,
                                             ready);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace

bool search_tc_supported(int cols) { return cols >= 1 && cols <= kMaxCols; }

size_t search_expand_bytes(int rows, int cols, int nwords, int directions) {
    // wider words take the in-kernel expansion: their tiles leave room for
    // too few ring slots to hide a bulk copy's latency
    if (!search_tc_supported(cols) || rows < 1 || nwords > 8)
        return 0;
    const size_t ntiles = (size_t)(cols + kRows - 1) / kRows;
    return (size_t)directions * rows * ntiles * kRows * nwords * 32;
}

cudaError_t launch_search_tc(const uint32_t* desc0, const uint32_t* desc1, int rows, int cols, int nwords,
                             int bits, bool nodupes, int directions, int16_t* disp, long long disp_pitch,
                             int32_t* best0, int32_t* best1, cudaStream_t st, uint8_t* xbuf, bool xbuf_ready) {
    if (!search_tc_supported(cols) || rows < 1)
        return cudaErrorInvalidValue;
    return nodupes ? launch_tc_dup<true>(desc0, desc1, rows, cols, nwords, bits, directions, disp, disp_pitch,
                                         best0, best1, xbuf, st, xbuf_ready)
                   : launch_tc_dup<false>(desc0, desc1, rows, cols, nwords, bits, directions, disp, disp_pitch,
                                          best0, best1, xbuf, st, xbuf_ready);
}

unsigned int read_tc_faults() {
    unsigned int v = 0;
    cudaMemcpyFromSymbol(&v, g_tc_faults, sizeof v);
    return v;
}

}  // namespace bicos_gb300
