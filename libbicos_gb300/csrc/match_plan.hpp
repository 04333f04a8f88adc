// One match broken into its pieces: validation and scratch layout
// (plan_match), and the three stages enqueued on a stream.  bicos_match_v1
// runs them in order on one stream; the batch API (batch_api.cu) runs the
// transform and the reference-form agreement of many stacks in persistent
// multi-stack launches and the rest per stack, all from the same plans.
#pragma once

#include <cuda_runtime.h>

#include "../../include/bicos_c.h"
#include "kernels.cuh"

namespace bicos_gb300 {

struct MatchPlan {
    StackParams s;
    const bicos_config* cfg = nullptr;
    bicos_image* disparity = nullptr;
    bicos_image* corrmap = nullptr;  // null when absent or without threshold
    int n = 0, eb = 0, rows = 0, cols = 0, nw = 0;
    bool full = false, thr = false, sub = false, dbl = false, consistency = false;
    bool moments = false, learned = false;
    // scratch layout: descriptors of both sides, raw disparity (subpixel
    // runs), consistency bests, the learned form's buffers, the search's
    // FP8 candidate tiles
    size_t desc_bytes = 0, raw_bytes = 0, best_bytes = 0, learned_bytes = 0, expand_bytes = 0;
    size_t scratch_bytes() const;
    // optional point cloud (bicos_match_points_v1): written by the
    // reference-form agreement kernels as they write the disparity, or by
    // the reprojection pass after the match in every other case
    float* pts = nullptr;
    long long pts_pitch = 0;
    float q[16] = {};
};

struct MatchBuffers {
    uint32_t* d0;
    uint32_t* d1;
    int16_t* raw;  // raw disparity: scratch (subpixel) or the caller's int16 disparity
    long long raw_pitch;
    int32_t* fwd;
    int32_t* rev;
    void* learned;
    uint8_t* expand;  // null: the search expands its candidate tiles in every CTA
};

// the reference's validation (src/impl/cuda.cu.in:233-292) with its error
// texts; fills the plan
bicos_status plan_match(const bicos_image* stack0, const bicos_image* stack1, uint32_t n, bicos_image* disparity,
                        bicos_image* corrmap, const bicos_config* cfg, MatchPlan* plan);
MatchBuffers match_buffers(const MatchPlan& plan, void* scratch);
cudaError_t enqueue_transform(const MatchPlan& plan, const MatchBuffers& m, cudaStream_t st);
// tiles_written: enqueue_transform wrote the candidate tiles into m.expand
// (a persistent multi-stack transform does not)
cudaError_t enqueue_search(const MatchPlan& plan, const MatchBuffers& m, cudaStream_t st, bool tiles_written);
// parameters of the reference-form agreement (in place on int16 without a
// step, float output with one)
AgreeParams agree_params(const MatchPlan& plan, const MatchBuffers& m);
// the agreement stage in the plan's form (model: the learned form's device
// model, else unused)
cudaError_t enqueue_agree(const MatchPlan& plan, const MatchBuffers& m, const float* model, cudaStream_t st);
// the agreement kernels of the plan's form; ap.pts set has them write the
// point cloud in the same pass
cudaError_t enqueue_agree_form(const MatchPlan& plan, const MatchBuffers& m, const AgreeParams& ap,
                               const float* model, cudaStream_t st);

}  // namespace bicos_gb300
