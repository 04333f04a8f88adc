// Allocation-free variant of the search stage (bicos_search_noalloc_v1).
//
// Who needs it: callers that must not allocate device memory while they
// run -- a real-time capture loop with a fixed memory plan, a host
// framework or plugin sandbox that owns every device allocation and
// forbids cudaMalloc inside its callbacks, or code that must not risk an
// allocation failure (or the implicit synchronisation cudaMalloc/cudaFree
// can cause) in the middle of a pipeline.  bicos_search_v1 takes its
// consistency scratch from the library's growable cache, which may call
// cudaMalloc; this entry point takes it from a fixed array instead.
//
// The scratch is the forward and backward best-column buffers of the
// consistency search (2 x int32 per pixel), in a file-scope __device__
// array sized for kNoAllocMaxPixels pixels: 2 x 4 Mi x 4 B = 32 MiB.  Every
// GPU that loads this part of the library holds the array until the
// process exits.  No element needs clearing between calls: the search
// kernel writes every best column of the image before the combine kernel
// reads any of them (a search CTA whose bounded waits run out writes -1,
// "no match", for its pixels instead of leaving the previous call's
// columns).  All calls share the one array, so calls whose work overlaps
// on the GPU (different streams, or threads without ordering) race on it;
// serialise them.  The first consistency call on a device looks the
// array's address up, which also loads the module holding it where modules
// load lazily: make one such call at initialisation, outside any stream
// capture, so that later calls only launch kernels.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/bicos_c.h"
#include "kernels.cuh"

namespace {

constexpr long long kNoAllocMaxPixels = 4LL << 20;  // rows * cols limit

static __device__ __align__(256) int32_t g_noalloc_best[2 * kNoAllocMaxPixels];

constexpr int kMaxDevices = 64;

std::mutex g_scratch_mu;
int32_t* g_scratch_ptr[kMaxDevices] = {};

// Device address of the array on the current device (in host code the
// array's name is only a host-side stand-in).  Only a successful lookup is
// kept: a lookup that failed (for instance one attempted inside a stream
// capture, where loading the module holding the array is not allowed) is
// tried again on the next call.
cudaError_t scratch_address(int32_t** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    if (dev < 0 || dev >= kMaxDevices)
        return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_best);
        if (e != cudaSuccess)
            return e;
        g_scratch_ptr[dev] = static_cast<int32_t*>(p);
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

bicos_status noalloc_fail(bicos_status s, const std::string& msg) {
    bicos_gb300::set_last_error(msg);
    return s;
}

}  // namespace

extern "C" bicos_status bicos_search_noalloc_v1(const uint32_t* desc0, const uint32_t* desc1, int32_t rows,
                                                int32_t cols, uint32_t nwords, int32_t flags,
                                                int32_t max_lr_diff, bicos_image* disparity,
                                                bicos_stream_t stream) {
    using namespace bicos_gb300;
    if (!desc0 || !desc1 || rows < 1 || cols < 1 || cols > 32767)
        return noalloc_fail(BICOS_ERR_INVALID_ARGUMENT, "bad descriptor arguments");
    if (nwords != 1 && nwords != 2 && nwords != 4 && nwords != 8 && nwords != 12 && nwords != 16)
        return noalloc_fail(BICOS_ERR_INVALID_ARGUMENT, "unsupported descriptor width");
    if (!disparity || !disparity->data || disparity->rows != rows || disparity->cols != cols ||
        disparity->type != BICOS_16S || disparity->step < (size_t)cols * 2)
        return noalloc_fail(BICOS_ERR_EXCEPTION, "disparity must be an int16 image of the descriptor size");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const bool nodup = (flags & BICOS_FLAG_NODUPES) != 0;
    cudaError_t e;
    if (flags & BICOS_FLAG_CONSISTENCY) {
        const long long px = (long long)rows * cols;
        if (px > kNoAllocMaxPixels)
            return noalloc_fail(BICOS_ERR_INVALID_ARGUMENT,
                                "bicos_search_noalloc_v1: " + std::to_string(px) +
                                    " pixels exceed the fixed scratch of " + std::to_string(kNoAllocMaxPixels) +
                                    " pixels (rows * cols); use bicos_search_v1");
        int32_t* base = nullptr;
        e = scratch_address(&base);
        if (e != cudaSuccess)
            return noalloc_fail(BICOS_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        int32_t* fwd = base;
        int32_t* rev = base + kNoAllocMaxPixels;
        e = launch_search(desc0, desc1, rows, cols, (int)nwords, 0, nodup, 2, nullptr, 0, fwd, rev, st);
        if (e == cudaSuccess)
            e = launch_consistency(fwd, rev, rows, cols, max_lr_diff, static_cast<int16_t*>(disparity->data),
                                   (long long)disparity->step, st);
    } else {
        // no scratch in this form: the kernel writes the disparity directly
        e = launch_search(desc0, desc1, rows, cols, (int)nwords, 0, nodup, 1, static_cast<int16_t*>(disparity->data),
                          (long long)disparity->step, nullptr, nullptr, st);
    }
    if (e != cudaSuccess)
        return noalloc_fail(BICOS_ERR_CUDA, std::string("search launch: ") + cudaGetErrorString(e));
    return BICOS_OK;
}
