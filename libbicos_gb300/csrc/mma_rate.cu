// FP8 tensor-core rate of this GPU for the Hamming search's MMA shape
// (bicos_tc_fp8_rate_v1), a measurement tool: the denominator of the
// search's roofline.  The search's +-1 dot products run as tcgen05.mma
// kind::f8f6f4 (e4m3 x e4m3 -> FP32 in TMEM), M = 128, N = 128, K = 32 per
// instruction, four instructions per 128-bit descriptor tile; this kernel
// issues that instruction stream alone -- one 128-row A tile and one N-row
// B tile of +-1 values staged once in shared memory, `rounds` x 4
// back-to-back MMAs from one thread, no copies and no epilogue -- so its
// rate is what the tensor cores give the search's shape when nothing else
// limits them.  N = 256 (the largest single-CTA shape) gives the device's
// FP8 rate for comparison.
//
// Two CTAs per SM at most (their dynamic shared memory), each holding 256
// TMEM columns: N = 128 alternates two 128-column accumulators as the
// search does, N = 256 accumulates into one.  The completion wait is
// bounded; a CTA whose wait runs out counts itself in g_rate_faults, which
// the entry point turns into an error (and bicos_kernel_faults counts).
#include <cuda_runtime.h>

#include <string>

#include "../../include/bicos_c.h"
#include "kernels.cuh"
#include "tcgen05.cuh"

namespace bicos_gb300 {

__device__ unsigned int g_rate_faults = 0;

unsigned int read_rate_faults() {
    unsigned int v = 0;
    cudaMemcpyFromSymbol(&v, g_rate_faults, sizeof v);
    return v;
}

namespace {

using namespace tc;

constexpr int kRateThreads = 128;
constexpr int kRateK = 128;  // bytes of K per round: the search's 128-bit descriptors, four MMAs of 32
// dynamic shared memory per CTA: more than a third of an SM's, so no third
// CTA (and no third TMEM allocation) lands on an SM
constexpr int kRateSmem = 100 * 1024;
constexpr int kRateLaunches = 3;

template<int N>
__global__ void __launch_bounds__(kRateThreads, 2) k_fp8_mma_rate(int rounds) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint32_t tmem_slot;
    __shared__ __align__(8) uint64_t done;
    constexpr int kBytes = (128 + N) * kRateK;
    static_assert(kBytes <= kRateSmem, "tiles exceed the shared memory");
    const int tid = threadIdx.x, warp = tid >> 5;

    // +1 / -1 in e4m3 (0x38 / 0xB8), drawn from a hash of the byte index
    for (int i = tid; i < kBytes; i += kRateThreads) {
        const uint32_t h = ((uint32_t)i ^ (blockIdx.x << 20)) * 2654435761u;
        smem[i] = ((h >> 16) & 1u) ? 0xB8 : 0x38;
    }
    fence_async_smem();
    if (warp == 0) {
        tmem_alloc(smem_u32(&tmem_slot), 256);
        tmem_relinquish();
    }
    if (tid == 0)
        mbar_init(smem_u32(&done), 1);
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_slot;

    if (tid == 0) {
        constexpr uint32_t kIdescRate = idesc_f8_e4m3(128, N);
        // a 16-byte K slice of all rows: the canonical K-major layout
        // without swizzle (8-row core matrices 128 bytes apart)
        constexpr uint32_t a_chunk = 128 * 16, b_chunk = N * 16;
        constexpr int fresh = N == 128 ? 2 : 1;  // rounds that start an accumulator
        const uint32_t a = smem_u32(smem), b = a + 128 * kRateK;
        for (int r = 0; r < rounds; ++r) {
            const uint32_t d = tmem + (N == 128 ? (uint32_t)(r & 1) * 128u : 0u);
#pragma unroll
            for (int s = 0; s < kRateK / 32; ++s)
                mma_f8f6f4(d, smem_desc(a + s * 2 * a_chunk, a_chunk, 128),
                           smem_desc(b + s * 2 * b_chunk, b_chunk, 128), kIdescRate,
                           (r >= fresh || s > 0) ? 1u : 0u);
        }
        mma_commit(smem_u32(&done));
        const long long start = clock64();
        bool ok = mbar_try_wait(smem_u32(&done), 0);
        while (!ok && clock64() - start < kWaitCycles)
            ok = mbar_try_wait(smem_u32(&done), 0);
        if (!ok)
            atomicAdd(&g_rate_faults, 1u);
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0)
        tmem_dealloc(tmem, 256);
}

template<int N>
cudaError_t time_rate(int rounds, int grid, cudaStream_t st, cudaEvent_t t0, cudaEvent_t t1, float* ms) {
    auto k = k_fp8_mma_rate<N>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, kRateSmem);
    if (e != cudaSuccess)
        return e;
    k<<<grid, kRateThreads, kRateSmem, st>>>(rounds);  // warm-up
    e = cudaEventRecord(t0, st);
    for (int i = 0; i < kRateLaunches && e == cudaSuccess; ++i) {
        k<<<grid, kRateThreads, kRateSmem, st>>>(rounds);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaEventRecord(t1, st);
    if (e == cudaSuccess)
        e = cudaEventSynchronize(t1);
    if (e == cudaSuccess)
        e = cudaEventElapsedTime(ms, t0, t1);
    return e;
}

bicos_status rate_fail(bicos_status s, const std::string& msg) {
    set_last_error(msg);
    return s;
}

}  // namespace
}  // namespace bicos_gb300

using namespace bicos_gb300;

extern "C" bicos_status bicos_tc_fp8_rate_v1(int32_t n, double* tflops) {
    if (!tflops || (n != 128 && n != 256))
        return rate_fail(BICOS_ERR_INVALID_ARGUMENT, "bicos_tc_fp8_rate_v1: n must be 128 or 256, tflops non-null");
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess)
        return rate_fail(BICOS_ERR_CUDA, std::string("tensor-core rate: ") + cudaGetErrorString(e));
    const unsigned int faults0 = read_rate_faults();
    // about a millisecond per launch at the nominal FP8 rate
    const int rounds = n == 128 ? 4096 : 2048;
    const int grid = 2 * sms;
    cudaStream_t st = nullptr;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaEventCreate(&t0);
    if (e == cudaSuccess)
        e = cudaEventCreate(&t1);
    float ms = 0.f;
    if (e == cudaSuccess)
        e = n == 128 ? time_rate<128>(rounds, grid, st, t0, t1, &ms) : time_rate<256>(rounds, grid, st, t0, t1, &ms);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    if (t0)
        cudaEventDestroy(t0);
    if (t1)
        cudaEventDestroy(t1);
    if (st)
        cudaStreamDestroy(st);
    if (e != cudaSuccess)
        return rate_fail(BICOS_ERR_CUDA, std::string("tensor-core rate: ") + cudaGetErrorString(e));
    if (read_rate_faults() != faults0)
        return rate_fail(BICOS_ERR_CUDA, "tensor-core rate: an MMA completion wait ran out");
    // 2 x M x N x K per instruction, four instructions per round
    const double flop = 2.0 * 128 * n * 32 * 4 * (double)rounds * grid * kRateLaunches;
    *tflops = flop / (ms * 1e-3) / 1e12;
    return BICOS_OK;
}
