// Persistent multi-stack launches (the batch API, batch_api.cu).
//
// A kernel that normally runs as a grid over one stack is written as a
// block body taking virtual block coordinates (bx, by, bz).  k_batch runs
// such a body for every block of up to kBatchJobs stacks in one persistent
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

// Stacks per persistent launch: their parameters travel by value in the
// kernel's parameter space (the constant bank, as for a one-stack launch;
// kernel parameters may take up to 32764 bytes), a class with more stacks
// takes several launches.
constexpr int kBatchJobs = 12;

template<typename P>
struct BatchArgs {
    P jobs[kBatchJobs];
    BatchTile tiles[kBatchJobs];
    int nstacks;
    int total;    // virtual blocks over the launch's stacks
    int claim;    // virtual blocks per claim
    int* counter;  // device, zeroed before the launch
};

// Op: struct with `using P = ...;`, `static constexpr int kMaxThreads`,
// `static constexpr int kMinBlocks` (resident CTAs of kMaxThreads the
// register budget keeps, matching the one-stack kernel's occupancy) and
// `static __device__ void run(const P&, int bx, int by, int bz)`
template<typename Op>
__global__ void __launch_bounds__(Op::kMaxThreads, Op::kMinBlocks)
    k_batch(const __grid_constant__ BatchArgs<typename Op::P> a) {
    using P = typename Op::P;
    static_assert(sizeof(BatchArgs<P>) <= 32000, "kernel parameters exceed 32 KB");
    static_assert(sizeof(P) % 4 == 0, "parameters copied as 32-bit words");
    // the current stack's parameters: the bodies read them at fixed shared
    // addresses, as a one-stack grid reads its own from the constant bank
    __shared__ __align__(16) P cur;
    __shared__ int base;
    int cur_s = -1;
    for (;;) {
        if (threadIdx.x == 0)
            base = atomicAdd(a.counter, a.claim);
        __syncthreads();
        const int b0 = base;
        __syncthreads();  // every thread has read base before it is claimed again
        if (b0 >= a.total)
            break;
        const int b1 = min(b0 + a.claim, a.total);
        int s = 0;
        for (int v = b0; v < b1; ++v) {
            while (s + 1 < a.nstacks && a.tiles[s + 1].start <= v)
                ++s;
            if (s != cur_s) {  // uniform over the CTA
                __syncthreads();
                const int* src = reinterpret_cast<const int*>(&a.jobs[s]);
                int* dst = reinterpret_cast<int*>(&cur);
                for (int i = threadIdx.x; i < (int)(sizeof(P) / 4); i += blockDim.x)
                    dst[i] = src[i];
                __syncthreads();
                cur_s = s;
            }
            const BatchTile& t = a.tiles[s];
            const int local = v - t.start;
            const int bx = local % t.gx, rest = local / t.gx;
            Op::run(cur, bx, rest % t.gy, rest / t.gy);
        }
    }
}

// launch shape of one persistent launch
struct BatchLaunch {
    int grid;   // CTAs
    int block;  // threads per CTA (transform: the column block width)
};

template<typename Op>
cudaError_t launch_batch_op(const BatchArgs<typename Op::P>& args, const BatchLaunch& l, size_t smem,
                            cudaStream_t st) {
    if (l.block > Op::kMaxThreads || args.nstacks < 1 || args.nstacks > kBatchJobs)
        return cudaErrorInvalidValue;
    auto k = k_batch<Op>;
    if (smem > 0) {  // k_batch's own shared variable counts against the default 48 KB
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess)
            return e;
    }
    k<<<l.grid, l.block, smem, st>>>(args);
    return cudaGetLastError();
}

}  // namespace bicos_gb300
