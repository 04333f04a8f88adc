// FP8 candidate and query tiles of the tensor-core Hamming search (stage b):
// descriptor bits as +-1 (+-16 / +-8 in the column-coded form) e4m3 values
// in the canonical no-swizzle K-major layout that tcgen05.mma reads from
// shared memory.  Shared by the search (search_tc.cu) and the descriptor
// transform, which can write the candidate side's tiles as it makes the
// descriptors (transform.cu).
#pragma once

#include <stdint.h>

namespace bicos_gb300 {
namespace fp8t {

constexpr int kRows = 128;  // rows (candidates or queries) per tile: MMA M = N = 128

// K-chunk major tiles: the 16 core matrices of one 16-byte K chunk (all 128
// rows) are contiguous (SBO = 128 B, LBO = 2 KB), so an MMA's operand fetch
// of one K step walks contiguous shared memory.
constexpr uint32_t kChunkBytes = 128 * 16;  // one 16-byte K chunk of 128 rows

__host__ __device__ constexpr size_t tile_bytes(int nw) { return (size_t)kRows * nw * 32; }

// FP8 patterns of a clear bit (a set bit flips bit 7, the sign): +-1, and
// in the column-coded form +-16 (query rows) and +-8 (candidate rows)
constexpr uint32_t kClearPlain = 0xB8B8B8B8u;
constexpr uint32_t kClearQuery = 0xD8D8D8D8u;
constexpr uint32_t kClearCand = 0xD0D0D0D0u;

// bits 0..3 (lo) or 4..7 (hi) of x -> 4 FP8 bytes: the product puts nibble
// bit i at bit 8i+7 (the four shifted copies of the nibble do not overlap,
// so nothing carries), the mask keeps those bits, the XOR applies them to
// the clear pattern's sign bits
__device__ __forceinline__ uint32_t fp8_lo(uint32_t x, uint32_t clear4) {
    return (((x & 0xFu) * 0x10204080u) & 0x80808080u) ^ clear4;
}
__device__ __forceinline__ uint32_t fp8_hi(uint32_t x, uint32_t clear4) {
    return (((x & 0xF0u) * 0x01020408u) & 0x80808080u) ^ clear4;
}

// e4m3 encoding of the integers 0..15 (exact: at most 4 significant bits)
__device__ __forceinline__ uint32_t e4m3_small(uint32_t v) {
    const uint32_t e = 31u - __clz(v | 1u);
    return v ? ((e + 7u) << 3) | ((v << (3u - e)) & 7u) : 0u;
}

// byte lanes 2..3 of a row's last 4 K slots: the query row's code factors
// -1, -16 and a candidate's column nibbles (c < 256)
constexpr uint32_t kQueryCode = 0xD8B80000u;
__device__ __forceinline__ uint32_t column_code(uint32_t c) {
    return (e4m3_small(c & 15u) << 16) | (e4m3_small(c >> 4) << 24);
}

// one descriptor's words, loaded ahead of its expansion
template<int NW>
struct Desc {
    uint32_t w[NW];
};

template<int NW>
__device__ __forceinline__ Desc<NW> load_desc(const uint32_t* p) {
    Desc<NW> d;
    if constexpr (NW % 4 == 0) {
#pragma unroll
        for (int j = 0; j < NW / 4; ++j) {
            const uint4 q = __ldg(reinterpret_cast<const uint4*>(p) + j);
            d.w[4 * j] = q.x;
            d.w[4 * j + 1] = q.y;
            d.w[4 * j + 2] = q.z;
            d.w[4 * j + 3] = q.w;
        }
    } else if constexpr (NW == 2) {
        const uint2 q = __ldg(reinterpret_cast<const uint2*>(p));
        d.w[0] = q.x;
        d.w[1] = q.y;
    } else {
        d.w[0] = __ldg(p);
    }
    return d;
}

// one descriptor into row rr of a 128-row FP8 tile (canonical layout).
// code (column-coded form): bytes 2..3 of the row's last 4 K slots,
// replacing the padding bits there.
template<int NW, bool ENC>
__device__ __forceinline__ void expand_desc(uint8_t* tile, int rr, const Desc<NW>& d, uint32_t clear4,
                                            uint32_t code = 0) {
    uint8_t* base = tile + (rr >> 3) * 128 + (rr & 7) * 16;
#pragma unroll
    for (int w = 0; w < NW; ++w) {
        const uint32_t x = d.w[w];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const uint32_t y = x >> (16 * h), z = y >> 8;
            uint32_t top = fp8_hi(z, clear4);
            if (ENC && w == NW - 1 && h == 1)
                top = (top & 0xFFFFu) | code;
            *reinterpret_cast<uint4*>(base + (2 * w + h) * kChunkBytes) =
                make_uint4(fp8_lo(y, clear4), fp8_hi(y, clear4), fp8_lo(z, clear4), top);
        }
    }
}

// candidate row of column `col` in its tile pair's column code, written
// into the candidate tiles of one row: tile col / 128, row col % 128
template<int NW, bool ENC>
__device__ __forceinline__ void expand_candidate(uint8_t* xt, int row, int col, int ntiles, const Desc<NW>& d) {
    const int t = col / kRows, p = col - t * kRows;
    expand_desc<NW, ENC>(xt + ((size_t)row * ntiles + t) * tile_bytes(NW), p, d, ENC ? kClearCand : kClearPlain,
                         ENC ? column_code((t & 1) * kRows + p) : 0u);
}

}  // namespace fp8t
}  // namespace bicos_gb300
