// Internal interface between the host orchestration (capi.cu, batch_api.cu)
// and the sm_103a kernels (transform.cu, search_tc.cu, search.cu, agree.cu,
// moments.cu, learned.cu, reproject.cu, mma_rate.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

namespace bicos_gb300 {

constexpr int kMaxFrames = 65;      // limited mode, 256-bit descriptors (4*65-7 = 253)
constexpr int kMaxFullFrames = 23;  // full mode, 512-bit extension (23^2-2*23+3 = 486)
constexpr int16_t kInvalidDisp = INT16_MIN;

// Frame pointers and row pitches of both sides, passed by value
// (__grid_constant__) so kernels read them from the constant bank.
struct StackParams {
    const uint8_t* frame[2][kMaxFrames];
    long long pitch[2][kMaxFrames];
    int n;
    int rows;
    int cols;
    int elem_bytes;
};

struct AgreeParams {
    StackParams s;
    const int16_t* raw;   // int16 disparity in (subpixel) / in-out (agree)
    long long raw_pitch;
    int16_t* raw_io;
    void* out;            // float disparity (subpixel)
    long long out_pitch;
    void* corr;           // float or double corrmap, may be null
    long long corr_pitch;
    float thr;
    float step;
    int has_minvar;
    float minvar;
    // 1.0, read at run time: the sweep's packed sums fma(t, one, u) must not
    // be folded with the product that made t, which a literal 1 would allow
    float one = 1.0f;
    // optional point cloud written in the same pass (bicos_match_points_v1):
    // BICOS_32FC3 rows, Q row-major as floats
    float* pts = nullptr;
    long long pts_pitch = 0;
    float q[16] = {};
};

// Point of pixel (x, y) with disparity d: [X Y Z W]^T = Q [x y d 1]^T
// written as (X/W, Y/W, Z/W), W = 0 giving (0, 0, 0) (cv::reprojectImageTo3D
// as bicos-cli runs it, src/cli.cpp:228-250); FP32, each row of Q a fused
// sum.  Shared by the reprojection pass and the agreement kernels' fused
// output, so both give the same bits.
__device__ __forceinline__ void reproject_store(const float* q, float* pts_row, int x, int y, float d) {
    const float fx = (float)x, fy = (float)y;
    float h[4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
        h[i] = fmaf(q[4 * i], fx, fmaf(q[4 * i + 1], fy, fmaf(q[4 * i + 2], d, q[4 * i + 3])));
    const float iw = h[3] != 0.0f ? 1.0f / h[3] : 0.0f;
    float* out = pts_row + 3 * x;
    out[0] = h[0] * iw;
    out[1] = h[1] * iw;
    out[2] = h[2] * iw;
}
__device__ __forceinline__ void agree_point(const AgreeParams& p, int row, int col, float d) {
    if (p.pts)
        reproject_store(p.q, reinterpret_cast<float*>(reinterpret_cast<char*>(p.pts) + (long long)row * p.pts_pitch),
                        col, row, d);
}

// moment form of the NCC stage (moments.cu)
struct MomentParams {
    StackParams s;
    const int16_t* raw;  // int16 disparity in
    long long raw_pitch;
    void* out;           // mode 0: int16 disparity (may alias raw), 1: float, 2: float[8] features
    long long out_pitch;
    void* corr;          // float / double corrmap (modes 0, 1), may be null
    long long corr_pitch;
    float thr;
    float step;
    int has_minvar;
    float minvar;
    // optional point cloud written in the same pass (modes 0 and 1), as in
    // AgreeParams; null when unused
    float* pts;
    long long pts_pitch;
    float q[16];
};

// mode 0: agree at the integer disparity, 1: subpixel sweep, 2: features
cudaError_t launch_moments(const MomentParams& p, int mode, bool dbl, cudaStream_t st);
unsigned int read_moment_faults();

// tiles0 / tiles1: when set (words up to 256 bits), the transform also
// writes side 0's / side 1's FP8 candidate tiles for the tensor-core search
// (the layout k_expand_tiles writes; bits decides the column-coded form),
// and the search is then told they are there
cudaError_t launch_transform(const StackParams& p, int sides, bool full, int nwords,
                             uint32_t* desc0, uint32_t* desc1, cudaStream_t st, uint8_t* tiles0 = nullptr,
                             uint8_t* tiles1 = nullptr, int bits = 0);

// Row-wise arg-min.  When disp != nullptr (one direction, NODUPES or plain)
// the kernel writes int16 disparities col0 - best directly; otherwise it
// writes int32 best columns (-1 = invalid) of each direction to best0/best1.
// bits: the descriptors' bit count when known (the transform's), else 0
// (every bit of the nwords words may be set).
// xbuf (optional, search_expand_bytes(rows, cols, nwords, directions)
// bytes): scratch for the candidate sides expanded to FP8 tiles once per
// call, which the tensor-core search then moves into shared memory with
// bulk copies; without it the search expands them in every CTA.
cudaError_t launch_search(const uint32_t* desc0, const uint32_t* desc1, int rows, int cols,
                          int nwords, int bits, bool nodupes, int directions, int16_t* disp,
                          long long disp_pitch, int32_t* best0, int32_t* best1,
                          cudaStream_t st, uint8_t* xbuf = nullptr, bool xbuf_ready = false);
// bytes of the optional expansion scratch (0: the search cannot use one);
// xbuf_ready: the transform already wrote the candidate tiles there
size_t search_expand_bytes(int rows, int cols, int nwords, int directions);

// point-cloud reprojection (reproject.cu): q = Q row-major, as floats
struct ReprojectParams {
    const void* disp;
    long long disp_pitch;
    float* pts;
    long long pts_pitch;
    int rows, cols;
    float q[16];
};
cudaError_t launch_reproject(const ReprojectParams& p, bool float_disp, cudaStream_t st);

// tensor-core search (search_tc.cu): same contract as launch_search, for
// rows of at most 4096 columns
bool search_tc_supported(int cols);
cudaError_t launch_search_tc(const uint32_t* desc0, const uint32_t* desc1, int rows, int cols, int nwords,
                             int bits, bool nodupes, int directions, int16_t* disp, long long disp_pitch,
                             int32_t* best0, int32_t* best1, cudaStream_t st, uint8_t* xbuf = nullptr,
                             bool xbuf_ready = false);
// number of tensor-core search CTAs whose bounded waits ran out (synchronous)
unsigned int read_tc_faults();
// the same for the FP8 rate probe (mma_rate.cu)
unsigned int read_rate_faults();

cudaError_t launch_consistency(const int32_t* fwd, const int32_t* rev, int rows, int cols,
                               int max_lr_diff, int16_t* disp, long long disp_pitch,
                               cudaStream_t st);

cudaError_t launch_agree(const AgreeParams& p, bool dbl, cudaStream_t st);
cudaError_t launch_agree_subpixel(const AgreeParams& p, bool dbl, cudaStream_t st);

// learned subpixel form (learned.cu): per pixel features -> network
// proposal -> one reference NCC check; pixels whose check fails are
// appended to `list` for the reference sweep (launch_subpixel_list)
struct LearnedParams {
    AgreeParams a;             // raw in, float disparity out, corrmap, threshold, min_var
    const float* model;        // device model buffer (mlp_model_floats() floats)
    float* proposal;           // optional per-pixel offsets (NaN where no proposal), may be null
    long long proposal_pitch;
    int* list;                 // pixels (row * cols + col) left to the sweep
    int* count;                // length of list, zeroed before the launch
    int* tile_counter;         // tiles claimed so far, zeroed before the launch
    float drop;                // accepted when rho(x) >= rho(0) - drop
    int vec16;                 // frames 16-byte aligned with 16-byte pitches and row widths
};
cudaError_t launch_learned(const LearnedParams& p, bool dbl, cudaStream_t st);
// the reference sweep over the pixels of a list (agree.cu); xs: the sweep's
// nx offsets (-1, then float-accumulated steps while <= 1)
cudaError_t launch_subpixel_list(const AgreeParams& p, bool dbl, const int* list, const int* count,
                                 const float* xs, int nx, cudaStream_t st);

// subpixel network (learned.cu); a model buffer holds mlp_model_floats()
// floats: the parameters, then the input means and standard deviations
int mlp_param_count();
int mlp_model_floats();
cudaError_t launch_mlp_grad(const float* model, const float* samples, int count, float* grad, float* loss,
                            cudaStream_t st);
cudaError_t launch_mlp_adam(float* params, float* grad, float* m, float* v, int step, float lr, float scale,
                            cudaStream_t st);
// proposals for `count` feature rows of 8 floats (BF16 weights, tensor cores)
cudaError_t launch_mlp_propose(const float* model, const float* features, int count, float* out,
                               cudaStream_t st);
unsigned int read_mlp_faults();
// device copy of the installed model for the current device (nullptr and a
// message when none is installed)
const float* learned_model_device(cudaStream_t st, std::string* err);

// batch API (batch_api.cu; the kernels in transform.cu and agree.cu): all
// jobs of one kernel class in one persistent launch over a work table
// (batch.cuh: BatchWork, BatchLaunch)
template<typename P>
struct BatchArgs;
struct BatchLaunch;
struct TransformJob {
    StackParams s;
    uint32_t* d0;
    uint32_t* d1;
};
// class key: full ? n : descriptor words; virtual grid per job
// (ceil(cols / block), rows, 2)
cudaError_t launch_transform_batch(int elem_bytes, bool full, int key, const BatchArgs<TransformJob>& args,
                                   const BatchLaunch& l, cudaStream_t st);
// agreement classes: kind 0 agree (in place, int16), 1 single-precision
// sweep, 2 double-precision sweep; nmax the frame bucket (agree_bucket(n));
// virtual grid per job (ceil(cols / agree_block(kind)), rows, 1)
int agree_bucket(int n);
int agree_block(int kind);
size_t agree_smem(int kind, int nmax);
cudaError_t launch_agree_batch(int elem_bytes, int kind, bool dbl, int nmax, const BatchArgs<AgreeParams>& args,
                               const BatchLaunch& l, cudaStream_t st);
// the sweep's offsets generated on the device (the same float additions as
// the reference's loop); nx from sweep_offset_count
int sweep_offset_count(float step);
cudaError_t launch_sweep_offsets(float step, float* xs, int nx, cudaStream_t st);

// sets the per-thread message bicos_last_error() returns (defined in capi.cu)
void set_last_error(const std::string& msg);

}  // namespace bicos_gb300
