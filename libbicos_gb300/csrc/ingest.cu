// Frame-by-frame ingest of a stereo stack: the upstream side of the match
// (frames arrive one pattern at a time from the cameras; libBICOS's CLI
// uploads the finished stacks first and times that separately,
// src/cli.cpp:177-183).  A handle owns device frames for one stack shape;
// each push uploads one frame of both sides on the caller's stream, so the
// uploads overlap the capture of the next patterns, and the match then runs
// bicos_match_v1 on the resident frames.  Only the upload is streamed: the
// descriptor transform compares every frame with the stack's temporal mean
// and the search needs whole descriptors, so no stage can finish before
// the last frame arrives.
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/bicos_c.h"
#include "kernels.cuh"

using namespace bicos_gb300;

struct bicos_ingest {
    int rows = 0, cols = 0, type = 0, eb = 0;
    uint32_t n = 0;
    size_t row_bytes = 0, plane = 0;  // device frames packed, side 0 then side 1
    void* frames = nullptr;
    std::vector<cudaEvent_t> done;  // frame t of both sides uploaded
    std::vector<char> pushed;
    // recorded after the last match's kernels on the match's stream: a push
    // waits for it before overwriting a frame that match may still read
    cudaEvent_t consumed = nullptr;
    bool matched = false;
};

namespace {

bicos_status ingest_fail(bicos_status s, const std::string& msg) {
    set_last_error(msg);
    return s;
}

bicos_status ingest_cuda_fail(cudaError_t e, const char* where) {
    return ingest_fail(BICOS_ERR_CUDA, std::string("libBICOS CUDA error in ") + where + ": " + cudaGetErrorString(e));
}

}  // namespace

extern "C" {

bicos_status bicos_ingest_create(bicos_ingest** out, int32_t rows, int32_t cols, uint32_t n, int32_t type) {
    if (!out)
        return ingest_fail(BICOS_ERR_INVALID_ARGUMENT, "null handle pointer");
    *out = nullptr;
    if (n < 2)
        return ingest_fail(BICOS_ERR_EXCEPTION, "need at least two images");
    if (n > (uint32_t)kMaxFrames)
        return ingest_fail(BICOS_ERR_EXCEPTION, "Bad number of images");
    if (type != BICOS_8U && type != BICOS_16U)
        return ingest_fail(BICOS_ERR_EXCEPTION, "bad input depths, only CV_8UC1 and CV_16UC1 are supported");
    if (rows < 1 || cols < 1)
        return ingest_fail(BICOS_ERR_EXCEPTION, "empty images");
    if (cols > 32767)
        return ingest_fail(BICOS_ERR_EXCEPTION, "image width exceeds the int16 disparity range");
    bicos_ingest* h = new bicos_ingest();
    h->rows = rows;
    h->cols = cols;
    h->type = type;
    h->eb = type == BICOS_8U ? 1 : 2;
    h->n = n;
    h->row_bytes = (size_t)cols * h->eb;
    h->plane = h->row_bytes * rows;
    h->done.assign(n, nullptr);
    h->pushed.assign(n, 0);
    cudaError_t e = cudaMalloc(&h->frames, 2 * (size_t)n * h->plane);
    for (uint32_t t = 0; t < n && e == cudaSuccess; ++t)
        e = cudaEventCreateWithFlags(&h->done[t], cudaEventDisableTiming);
    if (e == cudaSuccess)
        e = cudaEventCreateWithFlags(&h->consumed, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        bicos_ingest_destroy(h);
        return ingest_cuda_fail(e, "bicos_ingest_create");
    }
    *out = h;
    return BICOS_OK;
}

bicos_status bicos_ingest_destroy(bicos_ingest* h) {
    if (!h)
        return BICOS_OK;
    for (cudaEvent_t ev : h->done)
        if (ev)
            cudaEventDestroy(ev);
    if (h->consumed)
        cudaEventDestroy(h->consumed);
    if (h->frames)
        cudaFree(h->frames);
    delete h;
    return BICOS_OK;
}

bicos_status bicos_ingest_push_v1(bicos_ingest* h, uint32_t t, const void* frame0, const void* frame1,
                                  size_t host_step, bicos_stream_t stream) {
    if (!h || !frame0 || !frame1)
        return ingest_fail(BICOS_ERR_INVALID_ARGUMENT, "null argument");
    if (t >= h->n)
        return ingest_fail(BICOS_ERR_INVALID_ARGUMENT,
                           "frame index " + std::to_string(t) + " outside the stack of " + std::to_string(h->n));
    if (host_step < h->row_bytes)
        return ingest_fail(BICOS_ERR_INVALID_ARGUMENT, "host row step smaller than a row");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    char* base = static_cast<char*>(h->frames);
    // write-after-read: the previous match (possibly on another stream) may
    // still be reading this frame
    cudaError_t e = h->matched ? cudaStreamWaitEvent(st, h->consumed, 0) : cudaSuccess;
    for (int side = 0; side < 2 && e == cudaSuccess; ++side) {
        char* dst = base + ((size_t)side * h->n + t) * h->plane;
        const void* src = side ? frame1 : frame0;
        e = host_step == h->row_bytes
                ? cudaMemcpyAsync(dst, src, h->plane, cudaMemcpyHostToDevice, st)
                : cudaMemcpy2DAsync(dst, h->row_bytes, src, host_step, h->row_bytes, h->rows, cudaMemcpyHostToDevice,
                                    st);
    }
    if (e == cudaSuccess)
        e = cudaEventRecord(h->done[t], st);
    if (e != cudaSuccess)
        return ingest_cuda_fail(e, "bicos_ingest_push_v1");
    h->pushed[t] = 1;
    return BICOS_OK;
}

bicos_status bicos_ingest_match_v1(bicos_ingest* h, bicos_image* disparity, bicos_image* corrmap,
                                   const bicos_config* cfg, bicos_stream_t stream) {
    if (!h)
        return ingest_fail(BICOS_ERR_INVALID_ARGUMENT, "null handle");
    for (uint32_t t = 0; t < h->n; ++t)
        if (!h->pushed[t])
            return ingest_fail(BICOS_ERR_EXCEPTION, "frame " + std::to_string(t) + " of the stack was not pushed");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    for (uint32_t t = 0; t < h->n; ++t)  // pushes may have used other streams
        if (cudaError_t e = cudaStreamWaitEvent(st, h->done[t], 0))
            return ingest_cuda_fail(e, "bicos_ingest_match_v1");
    // matches of one handle run in call order, so the event recorded after
    // this one also covers every earlier match (whatever its stream)
    if (h->matched)
        if (cudaError_t e = cudaStreamWaitEvent(st, h->consumed, 0))
            return ingest_cuda_fail(e, "bicos_ingest_match_v1");
    bicos_image im0[kMaxFrames], im1[kMaxFrames];
    char* base = static_cast<char*>(h->frames);
    for (uint32_t t = 0; t < h->n; ++t) {
        im0[t] = bicos_image{base + (size_t)t * h->plane, h->row_bytes, h->rows, h->cols, h->type, 0};
        im1[t] = bicos_image{base + ((size_t)h->n + t) * h->plane, h->row_bytes, h->rows, h->cols, h->type, 0};
    }
    const bicos_status s = bicos_match_v1(im0, im1, h->n, disparity, corrmap, cfg, stream);
    if (s != BICOS_OK)
        return s;
    if (cudaError_t e = cudaEventRecord(h->consumed, st))
        return ingest_cuda_fail(e, "bicos_ingest_match_v1");
    h->matched = true;
    return BICOS_OK;
}

}  // extern "C"
