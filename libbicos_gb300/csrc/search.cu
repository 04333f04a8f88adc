// Row-wise Hamming arg-min over the whole rectified row (stage b) and the
// left-right consistency postfilter.
//
// Semantics: libBICOS include/impl/cpu/bicos.hpp:50-113 (bicos_search /
// bicos).  The reference scans the row in order, keeps the first strict
// minimum and, under NODUPES, rejects a pixel when any later column ties
// the final minimum.  That is order-free once written as a reduction:
// with key = cost << 16 | column, the first minimum is the smallest key,
// and "a tie exists" means the second-smallest key has the same cost.  So
// each thread keeps (m1, m2), the two smallest keys, updated with three
// integer min/max operations per candidate.
//
// Design: a CTA owns one row and 128*QPT query pixels; the candidate row is
// staged through shared memory in chunks and read back as broadcast
// 128-bit loads; each thread keeps QPT query descriptors in registers so
// one shared-memory read feeds QPT Hamming distances.  The consistency
// variant runs both directions in one launch (blockIdx.z) and a small
// elementwise kernel combines them.
#include "kernels.cuh"

namespace bicos_gb300 {
namespace {

constexpr int kThreads = 128;
constexpr int kSmemBytes = 48 * 1024;

template<int NW>
struct Vec {
    using type = uint4;
    static constexpr int per = 4;
};
template<>
struct Vec<2> {
    using type = uint2;
    static constexpr int per = 2;
};
template<>
struct Vec<1> {
    using type = uint32_t;
    static constexpr int per = 1;
};

template<int NW, bool NODUP, int QPT>
__global__ void __launch_bounds__(kThreads) k_search(const uint32_t* __restrict__ d0,
                                                     const uint32_t* __restrict__ d1, int rows,
                                                     int cols, int chunk, int16_t* __restrict__ disp,
                                                     long long disp_pitch, int32_t* __restrict__ best0,
                                                     int32_t* __restrict__ best1) {
    using V = typename Vec<NW>::type;
    constexpr int VPD = NW / Vec<NW>::per;  // vectors per descriptor
    extern __shared__ __align__(16) unsigned char smem_raw[];
    V* cand = reinterpret_cast<V*>(smem_raw);

    const int row = blockIdx.y, dir = blockIdx.z;
    const size_t row_off = (size_t)row * cols * NW;
    const uint32_t* qrow = (dir ? d1 : d0) + row_off;
    const V* crow = reinterpret_cast<const V*>((dir ? d0 : d1) + row_off);

    uint32_t q[QPT][NW];
    unsigned m1[QPT], m2[QPT];
    const int qbase = blockIdx.x * (kThreads * QPT) + threadIdx.x;
#pragma unroll
    for (int j = 0; j < QPT; ++j) {
        const int c = qbase + j * kThreads;
        const V* src = reinterpret_cast<const V*>(qrow + (size_t)min(c, cols - 1) * NW);
#pragma unroll
        for (int v = 0; v < VPD; ++v) {
            const V x = __ldg(src + v);
            if constexpr (Vec<NW>::per == 4) {
                q[j][4 * v] = x.x;
                q[j][4 * v + 1] = x.y;
                q[j][4 * v + 2] = x.z;
                q[j][4 * v + 3] = x.w;
            } else if constexpr (Vec<NW>::per == 2) {
                q[j][2 * v] = x.x;
                q[j][2 * v + 1] = x.y;
            } else {
                q[j][v] = x;
            }
        }
        m1[j] = 0xFFFFFFFFu;
        m2[j] = 0xFFFFFFFFu;
    }

    for (int cs = 0; cs < cols; cs += chunk) {
        const int cn = min(chunk, cols - cs);
        __syncthreads();
        for (int i = threadIdx.x; i < cn * VPD; i += kThreads)
            cand[i] = __ldg(crow + (size_t)cs * VPD + i);
        __syncthreads();

#pragma unroll 2
        for (int k = 0; k < cn; ++k) {
            uint32_t c[NW];
#pragma unroll
            for (int v = 0; v < VPD; ++v) {
                const V x = cand[k * VPD + v];
                if constexpr (Vec<NW>::per == 4) {
                    c[4 * v] = x.x;
                    c[4 * v + 1] = x.y;
                    c[4 * v + 2] = x.z;
                    c[4 * v + 3] = x.w;
                } else if constexpr (Vec<NW>::per == 2) {
                    c[2 * v] = x.x;
                    c[2 * v + 1] = x.y;
                } else {
                    c[v] = x;
                }
            }
            const unsigned colk = (unsigned)(cs + k);
#pragma unroll
            for (int j = 0; j < QPT; ++j) {
                unsigned cost = 0;
#pragma unroll
                for (int w = 0; w < NW; ++w)
                    cost += __popc(q[j][w] ^ c[w]);
                const unsigned key = (cost << 16) | colk;
                if constexpr (NODUP)
                    m2[j] = min(m2[j], max(m1[j], key));
                m1[j] = min(m1[j], key);
            }
        }
    }

#pragma unroll
    for (int j = 0; j < QPT; ++j) {
        const int c = qbase + j * kThreads;
        if (c >= cols)
            continue;
        const int best = (int)(m1[j] & 0xFFFFu);
        const bool valid = !NODUP || (m2[j] >> 16) != (m1[j] >> 16);
        if (disp) {
            int16_t* o = reinterpret_cast<int16_t*>(reinterpret_cast<char*>(disp) + row * disp_pitch);
            o[c] = valid ? (int16_t)(c - best) : kInvalidDisp;
        } else {
            (dir ? best1 : best0)[(size_t)row * cols + c] = valid ? best : -1;
        }
    }
}

// include/impl/cpu/bicos.hpp:96-105: reverse search of desc1[best] over
// row0 is the column-wise arg-min rev[best]; valid iff |col0 - rev| <= m
__global__ void k_consistency(const int32_t* __restrict__ fwd, const int32_t* __restrict__ rev,
                              int rows, int cols, int max_lr_diff, int16_t* __restrict__ disp,
                              long long disp_pitch) {
    const int c0 = blockIdx.x * blockDim.x + threadIdx.x;
    const int row = blockIdx.y;
    if (c0 >= cols)
        return;
    int16_t out = kInvalidDisp;
    const int b = fwd[(size_t)row * cols + c0];
    if (b >= 0) {
        const int r = rev[(size_t)row * cols + b];
        if (r >= 0 && abs(c0 - r) <= max_lr_diff)
            out = (int16_t)((c0 + r) / 2 - b);
    }
    reinterpret_cast<int16_t*>(reinterpret_cast<char*>(disp) + row * disp_pitch)[c0] = out;
}

template<int NW, bool NODUP>
cudaError_t launch_nw(const uint32_t* d0, const uint32_t* d1, int rows, int cols, int dirs,
                      int16_t* disp, long long disp_pitch, int32_t* b0, int32_t* b1, cudaStream_t st) {
    constexpr int QPT = NW >= 8 ? 1 : 2;
    const int chunk = min(cols, kSmemBytes / (NW * 4));
    const dim3 grid((cols + kThreads * QPT - 1) / (kThreads * QPT), rows, dirs);
    k_search<NW, NODUP, QPT><<<grid, kThreads, (size_t)chunk * NW * 4, st>>>(d0, d1, rows, cols, chunk,
                                                                             disp, disp_pitch, b0, b1);
    return cudaGetLastError();
}

template<bool NODUP>
cudaError_t launch_dup(const uint32_t* d0, const uint32_t* d1, int rows, int cols, int nwords, int dirs,
                       int16_t* disp, long long disp_pitch, int32_t* b0, int32_t* b1, cudaStream_t st) {
    switch (nwords) {
        case 1: return launch_nw<1, NODUP>(d0, d1, rows, cols, dirs, disp, disp_pitch, b0, b1, st);
        case 2: return launch_nw<2, NODUP>(d0, d1, rows, cols, dirs, disp, disp_pitch, b0, b1, st);
        case 4: return launch_nw<4, NODUP>(d0, d1, rows, cols, dirs, disp, disp_pitch, b0, b1, st);
        case 8: return launch_nw<8, NODUP>(d0, d1, rows, cols, dirs, disp, disp_pitch, b0, b1, st);
        case 12: return launch_nw<12, NODUP>(d0, d1, rows, cols, dirs, disp, disp_pitch, b0, b1, st);
        case 16: return launch_nw<16, NODUP>(d0, d1, rows, cols, dirs, disp, disp_pitch, b0, b1, st);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace

cudaError_t launch_search(const uint32_t* desc0, const uint32_t* desc1, int rows, int cols, int nwords,
                          int bits, bool nodupes, int directions, int16_t* disp, long long disp_pitch,
                          int32_t* best0, int32_t* best1, cudaStream_t st, uint8_t* xbuf, bool xbuf_ready) {
    if (cols > 32767 || cols < 1 || rows < 1)
        return cudaErrorInvalidValue;
    if (search_tc_supported(cols))
        return launch_search_tc(desc0, desc1, rows, cols, nwords, bits, nodupes, directions, disp, disp_pitch,
                                best0, best1, st, xbuf, xbuf_ready);
    return nodupes ? launch_dup<true>(desc0, desc1, rows, cols, nwords, directions, disp, disp_pitch,
                                      best0, best1, st)
                   : launch_dup<false>(desc0, desc1, rows, cols, nwords, directions, disp, disp_pitch,
                                       best0, best1, st);
}

cudaError_t launch_consistency(const int32_t* fwd, const int32_t* rev, int rows, int cols, int max_lr_diff,
                               int16_t* disp, long long disp_pitch, cudaStream_t st) {
    const dim3 grid((cols + 255) / 256, rows);
    k_consistency<<<grid, 256, 0, st>>>(fwd, rev, rows, cols, max_lr_diff, disp, disp_pitch);
    return cudaGetLastError();
}

}  // namespace bicos_gb300
