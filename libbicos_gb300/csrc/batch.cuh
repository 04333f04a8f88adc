// Persistent multi-stack launches (the batch API, batch.cu).
//
// A kernel that normally runs as a grid over one stack is written as a
// block body taking virtual block coordinates (bx, by, bz).  k_batch runs
// such a body for every block of every stack of a batch in one persistent
// launch: CTAs claim runs of `claim` virtual blocks from a global counter
// and map each to (stack, bx, by, bz) through the per-stack work table.
// The bodies contain no barriers, so a CTA can move from a block of one
// stack to a block of another freely.
#pragma once

#include <cuda_runtime.h>

#include "kernels.cuh"

namespace bicos_gb300 {

// one stack's virtual grid: its blocks are start .. start + gx*gy*gz - 1
struct BatchTile {
    int start;
    int gx, gy, gz;
};

struct BatchWork {
    const BatchTile* tiles;  // device, one per stack, ascending start
    int nstacks;
    int total;               // virtual blocks over all stacks
    int* counter;            // device, zeroed before the launch
    int claim;               // virtual blocks per claim
};

// Op: struct with `using P = ...;`, `static constexpr int kMaxThreads` and
// `static __device__ void run(const P&, int bx, int by, int bz)`
template<typename Op>
__global__ void __launch_bounds__(Op::kMaxThreads) k_batch(const typename Op::P* __restrict__ params,
                                                           const BatchWork w) {
    __shared__ int base;
    for (;;) {
        if (threadIdx.x == 0)
            base = atomicAdd(w.counter, w.claim);
        __syncthreads();
        const int b0 = base;
        __syncthreads();  // every thread has read base before it is claimed again
        if (b0 >= w.total)
            break;
        const int b1 = min(b0 + w.claim, w.total);
        int s = 0;
        for (int v = b0; v < b1; ++v) {
            while (s + 1 < w.nstacks && w.tiles[s + 1].start <= v)
                ++s;
            const BatchTile t = w.tiles[s];
            const int local = v - t.start;
            const int bx = local % t.gx, rest = local / t.gx;
            Op::run(params[s], bx, rest % t.gy, rest / t.gy);
        }
    }
}

// launch shape of one persistent launch
struct BatchLaunch {
    int grid;   // CTAs
    int block;  // threads per CTA (transform: the column block width)
};

template<typename Op>
cudaError_t launch_batch_op(const typename Op::P* params, const BatchWork& w, const BatchLaunch& l, size_t smem,
                            cudaStream_t st) {
    if (l.block > Op::kMaxThreads)
        return cudaErrorInvalidValue;
    auto k = k_batch<Op>;
    if (smem > 0) {  // k_batch's own shared variable counts against the default 48 KB
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess)
            return e;
    }
    k<<<l.grid, l.block, smem, st>>>(params, w);
    return cudaGetLastError();
}

}  // namespace bicos_gb300
