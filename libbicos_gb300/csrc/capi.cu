// C ABI and host orchestration of the matching path.
//
// Follows the control flow of libBICOS src/impl/cuda.cu.in:54-292 (input
// validation, descriptor width dispatch, transform -> search -> agree), but
// GB300-first: one stream (the caller's), no per-call cudaMalloc /
// cudaHostRegister / stream or event creation, kernel parameters by value,
// and the disparity output written by the kernels themselves (no fills).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/bicos_c.h"
#include "kernels.cuh"
#include "match_plan.hpp"

using namespace bicos_gb300;

namespace {

thread_local std::string g_last_error;

bicos_status fail(bicos_status s, const std::string& msg) {
    g_last_error = msg;
    return s;
}

bicos_status cuda_fail(cudaError_t e, const char* where) {
    return fail(BICOS_ERR_CUDA, std::string("libBICOS CUDA error in ") + where + ": " + cudaGetErrorString(e));
}

#define BICOS_CUDA_TRY(call)                       \
    do {                                           \
        cudaError_t e_ = (call);                   \
        if (e_ != cudaSuccess)                     \
            return cuda_fail(e_, #call);           \
    } while (0)

// ---- per-device scratch cache ------------------------------------------

struct Scratch {
    std::mutex mu;
    void* buf = nullptr;
    size_t cap = 0;
    cudaEvent_t ev = nullptr;
    cudaStream_t last = nullptr;
    bool used = false;
};

constexpr int kMaxDevices = 64;
Scratch g_scratch[kMaxDevices];
Scratch g_staging[kMaxDevices];  // device copies of host inputs/outputs (bicos_match_host_v1)

// the host path's second stream (row bands alternate between it and the
// caller's stream) and its fork/join events, per device
struct HostPipe {
    std::mutex mu;
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};
HostPipe g_host_pipe[kMaxDevices];

// Returns a buffer of >= bytes usable on `st`, ordered after its last use.
cudaError_t scratch_acquire(Scratch& s, size_t bytes, cudaStream_t st, void** out) {
    if (!s.ev) {
        cudaError_t e = cudaEventCreateWithFlags(&s.ev, cudaEventDisableTiming);
        if (e != cudaSuccess)
            return e;
    }
    if (s.cap < bytes) {
        if (s.used) {
            cudaError_t e = cudaEventSynchronize(s.ev);
            if (e != cudaSuccess)
                return e;
        }
        if (s.buf)
            cudaFree(s.buf);
        s.buf = nullptr;
        s.cap = 0;
        const size_t want = (bytes + (2u << 20) - 1) & ~size_t((2u << 20) - 1);
        cudaError_t e = cudaMalloc(&s.buf, want);
        if (e != cudaSuccess)
            return e;
        s.cap = want;
        s.used = false;
    } else if (s.used && s.last != st) {
        cudaError_t e = cudaStreamWaitEvent(st, s.ev, 0);
        if (e != cudaSuccess)
            return e;
    }
    *out = s.buf;
    return cudaSuccess;
}

cudaError_t scratch_release(Scratch& s, cudaStream_t st) {
    s.last = st;
    s.used = true;
    return cudaEventRecord(s.ev, st);
}

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// ---- optional stage timing (measurement tools) --------------------------

struct StageTiming {
    std::mutex mu;
    bool on = false;
    static constexpr int kCalls = 1024;
    cudaEvent_t ev[kCalls][4] = {};
    int used = 0;
    int dropped = 0;
};
StageTiming g_timing;

// events for one call: before transform, before search, before agree, end
cudaEvent_t* timing_slot() {
    std::lock_guard<std::mutex> lk(g_timing.mu);
    if (!g_timing.on)
        return nullptr;
    if (g_timing.used >= StageTiming::kCalls) {
        g_timing.dropped++;
        return nullptr;
    }
    cudaEvent_t* e = g_timing.ev[g_timing.used];
    for (int i = 0; i < 4; ++i)
        if (!e[i] && cudaEventCreate(&e[i]) != cudaSuccess)
            return nullptr;
    g_timing.used++;
    return e;
}

// ---- validation ----------------------------------------------------------

int elem_bytes_of(int type) {
    switch (type) {
        case BICOS_8U: return 1;
        case BICOS_16U: return 2;
        case BICOS_16S: return 2;
        case BICOS_32F: return 4;
        case BICOS_64F: return 8;
        case BICOS_32FC3: return 12;
        default: return 0;
    }
}

int required_bits(int n, bool full) { return full ? n * n - 2 * n + 3 : 4 * n - 7; }

// bit positions the transform writes (0 .. positions-1): the full layout
// fills exactly required_bits; the limited layout (3 bits per step, n-4
// pair-sum bits, 4 tail bits: include/impl/cpu/descriptor_transform.hpp:
// 32-73) ends one position past the reference's count
int descriptor_positions(int n, bool full) {
    return full ? required_bits(n, true) : 3 * (n - 2) + std::max(0, n - 4) + 4;
}

int words_for(int n, bool full, int max_bits) {
    const int bits = required_bits(n, full);
    if (bits <= 32) return 1;
    if (bits <= 64) return 2;
    if (bits <= 128) return 4;
    if (bits <= 256) return 8;
    // past the reference's 256 bits: full mode only, up to 512 bits
    if (full && max_bits > 256 && bits <= std::min(max_bits, 512))
        return ((bits + 127) / 128) * 4;
    return -1;
}

bool image_ok(const bicos_image* im, int rows, int cols, int type) {
    return im && im->data && im->rows == rows && im->cols == cols && im->type == type &&
           im->step >= (size_t)cols * elem_bytes_of(type);
}

bicos_status check_stacks(const bicos_image* s0, const bicos_image* s1, uint32_t n, int* eb) {
    if (n < 2)
        return fail(BICOS_ERR_EXCEPTION, "need at least two images");
    if (!s0 || !s1)
        return fail(BICOS_ERR_EXCEPTION, "null stack");
    const int type = s0[0].type;
    if (type != BICOS_8U && type != BICOS_16U)
        return fail(BICOS_ERR_EXCEPTION, "bad input depths, only CV_8UC1 and CV_16UC1 are supported");
    const int rows = s0[0].rows, cols = s0[0].cols;
    if (rows < 1 || cols < 1)
        return fail(BICOS_ERR_EXCEPTION, "empty images");
    if (cols > 32767)
        return fail(BICOS_ERR_EXCEPTION, "image width exceeds the int16 disparity range");
    for (uint32_t i = 0; i < n; ++i)
        if (!image_ok(&s0[i], rows, cols, type) || !image_ok(&s1[i], rows, cols, type))
            return fail(BICOS_ERR_EXCEPTION, "all images of both stacks must share size and type");
    *eb = elem_bytes_of(type);
    return BICOS_OK;
}

void fill_stack(StackParams& p, const bicos_image* s0, const bicos_image* s1, uint32_t n, int eb) {
    std::memset(&p, 0, sizeof p);
    for (uint32_t t = 0; t < n; ++t) {
        p.frame[0][t] = static_cast<const uint8_t*>(s0[t].data);
        p.pitch[0][t] = (long long)s0[t].step;
        p.frame[1][t] = static_cast<const uint8_t*>(s1 ? s1[t].data : s0[t].data);
        p.pitch[1][t] = (long long)(s1 ? s1[t].step : s0[t].step);
    }
    p.n = (int)n;
    p.rows = s0[0].rows;
    p.cols = s0[0].cols;
    p.elem_bytes = eb;
}

bool step_ok(float step) { return std::isfinite(step) && step >= 1e-4f; }

struct DeviceGuard {
    int dev = 0;
    cudaError_t err = cudaSuccess;
    DeviceGuard() { err = cudaGetDevice(&dev); }
};

// the learned form accepts a proposal when rho(x) >= rho(0) - kLearnedDrop
constexpr float kLearnedDrop = 0.002f;

// scratch of the learned form: the fallback list (one int per pixel), its
// length, the sweep's offsets (step >= 1e-4: at most 20001 of them)
constexpr size_t kMaxOffsets = 20480;
size_t learned_scratch_bytes(size_t px) { return align_up(px * 4, 256) + 256 + kMaxOffsets * 4; }

// 16-byte loads of whole rows are possible: frames and pitches 16-byte
// aligned, row width a multiple of 16 bytes
bool frames_vec16(const StackParams& s) {
    if ((s.cols * s.elem_bytes) % 16 != 0)
        return false;
    for (int side = 0; side < 2; ++side)
        for (int t = 0; t < s.n; ++t)
            if (reinterpret_cast<uintptr_t>(s.frame[side][t]) % 16 != 0 || s.pitch[side][t] % 16 != 0)
                return false;
    return true;
}

// Learned subpixel stage: one fused pass (features -> network -> one
// reference NCC check per pixel), then the reference sweep over the pixels
// whose check failed.  `ap` carries the raw disparity, the float output,
// the corrmap and the sweep step; `scratch` holds learned_scratch_bytes(px).
cudaError_t learned_subpixel(const AgreeParams& ap, bool dbl, const float* model, void* scratch,
                             int* fallback_count_out, float* proposal, long long proposal_pitch,
                             cudaStream_t st) {
    const size_t px = (size_t)ap.s.rows * ap.s.cols;
    char* b = static_cast<char*>(scratch);
    int* list = reinterpret_cast<int*>(b);
    int* count = reinterpret_cast<int*>(b + align_up(px * 4, 256));
    float* xs = reinterpret_cast<float*>(b + align_up(px * 4, 256) + 256);
    const int nx = sweep_offset_count(ap.step);
    if (nx > (int)kMaxOffsets)
        return cudaErrorInvalidValue;
    cudaError_t e = launch_sweep_offsets(ap.step, xs, nx, st);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(count, 0, 2 * sizeof(int), st);  // list length and tile counter
    if (e == cudaSuccess) {
        LearnedParams lp;
        std::memset(&lp, 0, sizeof lp);
        lp.a = ap;
        lp.model = model;
        lp.proposal = proposal;
        lp.proposal_pitch = proposal_pitch;
        lp.list = list;
        lp.count = count;
        lp.tile_counter = count + 1;
        lp.drop = kLearnedDrop;
        lp.vec16 = frames_vec16(ap.s) ? 1 : 0;
        e = launch_learned(lp, dbl, st);
    }
    if (e == cudaSuccess)
        e = launch_subpixel_list(ap, dbl, list, count, xs, nx, st);
    if (e == cudaSuccess && fallback_count_out)
        e = cudaMemcpyAsync(fallback_count_out, count, sizeof(int), cudaMemcpyDeviceToHost, st);
    return e;
}

}  // namespace

void bicos_gb300::set_last_error(const std::string& msg) { g_last_error = msg; }

// ---- one match: validation, scratch layout, stages (also used by the batch API)

size_t MatchPlan::scratch_bytes() const {
    return 2 * desc_bytes + raw_bytes + 2 * best_bytes + learned_bytes + expand_bytes;
}

bicos_status bicos_gb300::plan_match(const bicos_image* stack0, const bicos_image* stack1, uint32_t n,
                                     bicos_image* disparity, bicos_image* corrmap, const bicos_config* cfg,
                                     MatchPlan* plan) {
    if (!cfg)
        return fail(BICOS_ERR_INVALID_ARGUMENT, "null config");
    int eb = 0;
    if (bicos_status s = check_stacks(stack0, stack1, n, &eb))
        return s;
    MatchPlan& P = *plan;
    P = MatchPlan{};
    P.cfg = cfg;
    P.full = cfg->mode == BICOS_MODE_FULL;
    const int bits = required_bits((int)n, P.full);
    P.nw = n <= (uint32_t)kMaxFrames ? words_for((int)n, P.full, cfg->max_bits) : -1;
    if (P.nw < 0)
        return fail(BICOS_ERR_INVALID_ARGUMENT,
                    "input stacks too large, would require " + std::to_string(bits) + " bits");
    P.rows = stack0[0].rows;
    P.cols = stack0[0].cols;
    P.n = (int)n;
    P.eb = eb;
    P.thr = cfg->has_threshold != 0;
    P.sub = P.thr && cfg->has_subpixel_step != 0;
    P.dbl = cfg->precision == BICOS_PRECISION_DOUBLE;
    if (P.sub && !step_ok(cfg->subpixel_step))
        return fail(BICOS_ERR_EXCEPTION, "subpixel step must be a finite value >= 1e-4");
    P.consistency = cfg->variant == BICOS_VARIANT_CONSISTENCY;
    if (cfg->nxcorr_form < BICOS_NXCORR_REFERENCE || cfg->nxcorr_form > BICOS_NXCORR_LEARNED)
        return fail(BICOS_ERR_INVALID_ARGUMENT, "unknown nxcorr_form " + std::to_string(cfg->nxcorr_form));
    if (!image_ok(disparity, P.rows, P.cols, P.sub ? BICOS_32F : BICOS_16S))
        return fail(BICOS_ERR_EXCEPTION, P.sub ? "disparity must be a float32 image of the stack's size"
                                               : "disparity must be an int16 image of the stack's size");
    if (P.thr && corrmap && !image_ok(corrmap, P.rows, P.cols, P.dbl ? BICOS_64F : BICOS_32F))
        return fail(BICOS_ERR_EXCEPTION, P.dbl ? "corrmap must be a float64 image of the stack's size"
                                               : "corrmap must be a float32 image of the stack's size");
    P.moments = P.thr && cfg->nxcorr_form == BICOS_NXCORR_MOMENTS;
    P.learned = P.sub && cfg->nxcorr_form == BICOS_NXCORR_LEARNED;
    P.disparity = disparity;
    P.corrmap = P.thr ? corrmap : nullptr;
    fill_stack(P.s, stack0, stack1, n, eb);
    const size_t px = (size_t)P.rows * P.cols;
    P.desc_bytes = align_up(px * P.nw * 4, 256);
    P.raw_bytes = P.sub ? align_up(px * 2, 256) : 0;
    P.best_bytes = P.consistency ? align_up(px * 4, 256) : 0;
    P.learned_bytes = P.learned ? learned_scratch_bytes(px) : 0;
    P.expand_bytes = align_up(search_expand_bytes(P.rows, P.cols, P.nw, P.consistency ? 2 : 1), 256);
    return BICOS_OK;
}

MatchBuffers bicos_gb300::match_buffers(const MatchPlan& P, void* scratch) {
    char* b = static_cast<char*>(scratch);
    MatchBuffers m;
    m.d0 = reinterpret_cast<uint32_t*>(b);
    m.d1 = reinterpret_cast<uint32_t*>(b + P.desc_bytes);
    m.raw = P.sub ? reinterpret_cast<int16_t*>(b + 2 * P.desc_bytes) : static_cast<int16_t*>(P.disparity->data);
    m.raw_pitch = P.sub ? (long long)P.cols * 2 : (long long)P.disparity->step;
    m.fwd = P.consistency ? reinterpret_cast<int32_t*>(b + 2 * P.desc_bytes + P.raw_bytes) : nullptr;
    m.rev = P.consistency ? reinterpret_cast<int32_t*>(b + 2 * P.desc_bytes + P.raw_bytes + P.best_bytes) : nullptr;
    m.learned = P.learned ? b + 2 * P.desc_bytes + P.raw_bytes + 2 * P.best_bytes : nullptr;
    m.expand = P.expand_bytes
                   ? reinterpret_cast<uint8_t*>(b + 2 * P.desc_bytes + P.raw_bytes + 2 * P.best_bytes + P.learned_bytes)
                   : nullptr;
    return m;
}

// With an expansion buffer the transform also writes the search's FP8
// candidate tiles (side 1's for direction 0, then side 0's for direction
// 1), and enqueue_search finds them there.
cudaError_t bicos_gb300::enqueue_transform(const MatchPlan& P, const MatchBuffers& m, cudaStream_t st) {
    uint8_t *t0 = nullptr, *t1 = nullptr;
    if (m.expand) {
        const size_t ntiles = (size_t)(P.cols + 127) / 128;
        t1 = m.expand;
        if (P.consistency)
            t0 = m.expand + (size_t)P.rows * ntiles * 128 * P.nw * 32;
    }
    return launch_transform(P.s, 2, P.full, P.nw, m.d0, m.d1, st, t0, t1, descriptor_positions(P.n, P.full));
}

cudaError_t bicos_gb300::enqueue_search(const MatchPlan& P, const MatchBuffers& m, cudaStream_t st,
                                        bool tiles_written) {
    const int bits = descriptor_positions(P.n, P.full);
    if (P.consistency) {
        cudaError_t e = launch_search(m.d0, m.d1, P.rows, P.cols, P.nw, bits, P.cfg->no_dupes != 0, 2, nullptr, 0,
                                      m.fwd, m.rev, st, m.expand, tiles_written && m.expand);
        if (e == cudaSuccess)
            e = launch_consistency(m.fwd, m.rev, P.rows, P.cols, P.cfg->max_lr_diff, m.raw, m.raw_pitch, st);
        return e;
    }
    return launch_search(m.d0, m.d1, P.rows, P.cols, P.nw, bits, true, 1, m.raw, m.raw_pitch, nullptr, nullptr,
                         st, m.expand, tiles_written && m.expand);
}

AgreeParams bicos_gb300::agree_params(const MatchPlan& P, const MatchBuffers& m) {
    AgreeParams ap;
    std::memset(&ap, 0, sizeof ap);
    ap.one = 1.0f;
    ap.s = P.s;
    ap.thr = P.cfg->nxcorr_threshold;
    ap.step = P.sub ? P.cfg->subpixel_step : -1.f;
    ap.has_minvar = P.cfg->has_min_variance != 0;
    ap.minvar = P.cfg->has_min_variance ? P.cfg->min_variance * (float)P.n : 0.f;  // src/impl/cpu.cpp:123
    ap.corr = P.corrmap ? P.corrmap->data : nullptr;
    ap.corr_pitch = P.corrmap ? (long long)P.corrmap->step : 0;
    ap.raw = m.raw;
    ap.raw_pitch = m.raw_pitch;
    if (P.sub) {
        ap.out = P.disparity->data;
        ap.out_pitch = (long long)P.disparity->step;
    } else {
        ap.raw_io = m.raw;
    }
    return ap;
}

namespace {
// the plan's point cloud from its finished disparity (a separate pass)
cudaError_t reproject_after(const MatchPlan& P, cudaStream_t st) {
    ReprojectParams rp;
    rp.disp = P.disparity->data;
    rp.disp_pitch = (long long)P.disparity->step;
    rp.pts = P.pts;
    rp.pts_pitch = P.pts_pitch;
    rp.rows = P.rows;
    rp.cols = P.cols;
    for (int i = 0; i < 16; ++i)
        rp.q[i] = P.q[i];
    return launch_reproject(rp, P.disparity->type == BICOS_32F, st);
}
}  // namespace

cudaError_t bicos_gb300::enqueue_agree(const MatchPlan& P, const MatchBuffers& m, const float* model,
                                       cudaStream_t st) {
    if (!P.thr)
        return P.pts ? reproject_after(P, st) : cudaSuccess;
    AgreeParams ap = agree_params(P, m);
    // every form's agreement kernels write the points of the pixels they
    // finish (the learned form: accepted proposals in k_learned, the rest in
    // the sweep over its list)
    if (P.pts) {
        ap.pts = P.pts;
        ap.pts_pitch = P.pts_pitch;
        for (int i = 0; i < 16; ++i)
            ap.q[i] = P.q[i];
    }
    return enqueue_agree_form(P, m, ap, model, st);
}

cudaError_t bicos_gb300::enqueue_agree_form(const MatchPlan& P, const MatchBuffers& m, const AgreeParams& ap,
                                            const float* model, cudaStream_t st) {
    if (P.moments) {
        MomentParams mp;
        std::memset(&mp, 0, sizeof mp);
        mp.s = ap.s;
        mp.raw = m.raw;
        mp.raw_pitch = m.raw_pitch;
        mp.out = P.sub ? P.disparity->data : m.raw;
        mp.out_pitch = P.sub ? (long long)P.disparity->step : m.raw_pitch;
        mp.corr = ap.corr;
        mp.corr_pitch = ap.corr_pitch;
        mp.thr = ap.thr;
        mp.step = ap.step;
        mp.has_minvar = ap.has_minvar;
        mp.minvar = ap.minvar;
        mp.pts = ap.pts;
        mp.pts_pitch = ap.pts_pitch;
        for (int i = 0; i < 16; ++i)
            mp.q[i] = ap.q[i];
        return launch_moments(mp, P.sub ? 1 : 0, P.dbl, st);
    }
    if (P.learned)
        return learned_subpixel(ap, P.dbl, model, m.learned, nullptr, nullptr, 0, st);
    return P.sub ? launch_agree_subpixel(ap, P.dbl, st) : launch_agree(ap, P.dbl, st);
}

extern "C" {

const char* bicos_version(void) { return "bicos_gb300 0.1.0 (libBICOS 2.2.0 matching path, sm_103a)"; }

const char* bicos_last_error(void) { return g_last_error.c_str(); }

bicos_status bicos_config_default(bicos_config* c) {
    if (!c)
        return fail(BICOS_ERR_INVALID_ARGUMENT, "null config");
    std::memset(c, 0, sizeof *c);
    c->has_threshold = 1;
    c->nxcorr_threshold = 0.5f;
    c->mode = BICOS_MODE_LIMITED;
    c->precision = BICOS_PRECISION_SINGLE;
    c->variant = BICOS_VARIANT_NODUPLICATES;
    c->max_lr_diff = 1;
    c->no_dupes = 0;
    c->max_bits = 256;
    c->nxcorr_form = BICOS_NXCORR_REFERENCE;
    return BICOS_OK;
}

bicos_status bicos_output_types(const bicos_config* cfg, int32_t* dt, int32_t* ct) {
    if (!cfg || !dt || !ct)
        return fail(BICOS_ERR_INVALID_ARGUMENT, "null argument");
    const bool thr = cfg->has_threshold != 0;
    *dt = (thr && cfg->has_subpixel_step) ? BICOS_32F : BICOS_16S;
    *ct = thr ? (cfg->precision == BICOS_PRECISION_DOUBLE ? BICOS_64F : BICOS_32F) : -1;
    return BICOS_OK;
}

int32_t bicos_descriptor_words(uint32_t n, int32_t mode, int32_t max_bits) {
    if (n < 2 || n > (uint32_t)kMaxFrames)
        return -1;
    return words_for((int)n, mode == BICOS_MODE_FULL, max_bits);
}

int32_t bicos_kernel_faults(void) {
    return (int32_t)(read_tc_faults() + read_moment_faults() + read_mlp_faults() + read_rate_faults());
}

bicos_status bicos_stage_timing(int32_t enable) {
    std::lock_guard<std::mutex> lk(g_timing.mu);
    g_timing.on = enable != 0;
    g_timing.used = 0;
    g_timing.dropped = 0;
    return BICOS_OK;
}

bicos_status bicos_stage_times(float* ms, int32_t* calls) {
    if (!ms || !calls)
        return fail(BICOS_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lk(g_timing.mu);
    ms[0] = ms[1] = ms[2] = 0.f;
    for (int c = 0; c < g_timing.used; ++c) {
        cudaEvent_t* e = g_timing.ev[c];
        BICOS_CUDA_TRY(cudaEventSynchronize(e[3]));
        for (int i = 0; i < 3; ++i) {
            float t = 0.f;
            BICOS_CUDA_TRY(cudaEventElapsedTime(&t, e[i], e[i + 1]));
            ms[i] += t;
        }
    }
    *calls = g_timing.used;
    g_timing.used = 0;
    return BICOS_OK;
}

bicos_status bicos_release_scratch(void) {
    DeviceGuard g;
    if (g.err != cudaSuccess)
        return cuda_fail(g.err, "cudaGetDevice");
    for (Scratch* sp : {&g_scratch[g.dev % kMaxDevices], &g_staging[g.dev % kMaxDevices]}) {
        Scratch& s = *sp;
        std::lock_guard<std::mutex> lk(s.mu);
        if (s.used && s.ev)
            cudaEventSynchronize(s.ev);
        if (s.buf)
            BICOS_CUDA_TRY(cudaFree(s.buf));
        s.buf = nullptr;
        s.cap = 0;
        s.used = false;
    }
    return BICOS_OK;
}

}  // extern "C"

namespace {

// the three stages of a planned match on `stream`, scratch from the cache
bicos_status run_plan(const MatchPlan& plan, bicos_stream_t stream) {
    DeviceGuard g;
    if (g.err != cudaSuccess)
        return cuda_fail(g.err, "cudaGetDevice");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const float* model = nullptr;
    if (plan.learned) {
        std::string err;
        model = learned_model_device(st, &err);
        if (!model)
            return fail(BICOS_ERR_INVALID_ARGUMENT, err);
    }
    Scratch& s = g_scratch[g.dev % kMaxDevices];
    std::lock_guard<std::mutex> lk(s.mu);
    void* base = nullptr;
    BICOS_CUDA_TRY(scratch_acquire(s, plan.scratch_bytes(), st, &base));
    const MatchBuffers bufs = match_buffers(plan, base);

    cudaEvent_t* tev = timing_slot();
    if (tev)
        cudaEventRecord(tev[0], st);
    cudaError_t e = enqueue_transform(plan, bufs, st);
    if (tev)
        cudaEventRecord(tev[1], st);
    if (e == cudaSuccess)
        e = enqueue_search(plan, bufs, st, true);
    if (tev)
        cudaEventRecord(tev[2], st);
    if (e == cudaSuccess)
        e = enqueue_agree(plan, bufs, model, st);
    if (tev)
        cudaEventRecord(tev[3], st);
    cudaError_t er = scratch_release(s, st);
    if (e != cudaSuccess)
        return cuda_fail(e, "bicos_match_v1 launch");
    if (er != cudaSuccess)
        return cuda_fail(er, "cudaEventRecord");
    return BICOS_OK;
}

}  // namespace

extern "C" {

bicos_status bicos_match_v1(const bicos_image* stack0, const bicos_image* stack1, uint32_t n,
                            bicos_image* disparity, bicos_image* corrmap, const bicos_config* cfg,
                            bicos_stream_t stream) {
    MatchPlan plan;
    if (bicos_status s = plan_match(stack0, stack1, n, disparity, corrmap, cfg, &plan))
        return s;
    return run_plan(plan, stream);
}

bicos_status bicos_match_points_v1(const bicos_image* stack0, const bicos_image* stack1, uint32_t n,
                                   bicos_image* disparity, bicos_image* corrmap, const bicos_config* cfg,
                                   const double* q, bicos_image* points, bicos_stream_t stream) {
    if (!q || !points)
        return fail(BICOS_ERR_INVALID_ARGUMENT, "null argument");
    MatchPlan plan;
    if (bicos_status s = plan_match(stack0, stack1, n, disparity, corrmap, cfg, &plan))
        return s;
    if (!image_ok(points, plan.rows, plan.cols, BICOS_32FC3))
        return fail(BICOS_ERR_EXCEPTION, "points must be a three-channel float32 image of the stack's size");
    for (int i = 0; i < 16; ++i) {
        if (!std::isfinite(q[i]))
            return fail(BICOS_ERR_INVALID_ARGUMENT, "Q must be finite");
        plan.q[i] = (float)q[i];
    }
    plan.pts = static_cast<float*>(points->data);
    plan.pts_pitch = (long long)points->step;
    return run_plan(plan, stream);
}

// Host buffers in, host buffers out.  The image is processed in row bands
// (every stage is row-local, so a band is a bicos_match_v1 call on a
// sub-image and gives the same rows bit for bit): band k's upload runs on one
// of two streams while band k-1 computes on the other, each side's band
// uploaded by one 2-D copy whose rows are whole frame bands (wide rows keep
// the copy engine near its 1-D rate when the frames of a side are evenly
// spaced in host memory).  Synchronous on return.
bicos_status bicos_match_host_v1(const void* const* frames0, const void* const* frames1, uint32_t n, int32_t rows,
                                 int32_t cols, int32_t type, size_t host_step, void* disparity,
                                 size_t disparity_step, void* corrmap, size_t corrmap_step, const bicos_config* cfg,
                                 bicos_stream_t stream) {
    if (!cfg || !frames0 || !frames1 || !disparity)
        return fail(BICOS_ERR_INVALID_ARGUMENT, "null argument");
    if (n < 2)
        return fail(BICOS_ERR_EXCEPTION, "need at least two images");
    if (type != BICOS_8U && type != BICOS_16U)
        return fail(BICOS_ERR_EXCEPTION, "bad input depths, only CV_8UC1 and CV_16UC1 are supported");
    if (rows < 1 || cols < 1)
        return fail(BICOS_ERR_EXCEPTION, "empty images");
    const int eb = elem_bytes_of(type);
    if (host_step < (size_t)cols * eb)
        return fail(BICOS_ERR_INVALID_ARGUMENT, "host row step smaller than a row");
    const bool full = cfg->mode == BICOS_MODE_FULL;
    if (n > (uint32_t)kMaxFrames || words_for((int)n, full, cfg->max_bits) < 0)
        return fail(BICOS_ERR_INVALID_ARGUMENT, "input stacks too large, would require " +
                                                    std::to_string(required_bits((int)n, full)) + " bits");
    int32_t dt = 0, ct = 0;
    bicos_output_types(cfg, &dt, &ct);
    const bool want_corr = corrmap && ct >= 0;

    DeviceGuard g;
    if (g.err != cudaSuccess)
        return cuda_fail(g.err, "cudaGetDevice");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    HostPipe& hp = g_host_pipe[g.dev % kMaxDevices];
    std::lock_guard<std::mutex> hlk(hp.mu);
    if (!hp.side) {
        BICOS_CUDA_TRY(cudaStreamCreateWithFlags(&hp.side, cudaStreamNonBlocking));
        BICOS_CUDA_TRY(cudaEventCreateWithFlags(&hp.fork, cudaEventDisableTiming));
        BICOS_CUDA_TRY(cudaEventCreateWithFlags(&hp.join, cudaEventDisableTiming));
    }
    const size_t row_bytes = (size_t)cols * eb;
    const size_t plane = (size_t)rows * row_bytes;  // device frames packed: band copies stay 2-D
    const size_t disp_row = (size_t)cols * elem_bytes_of(dt);
    const size_t corr_row = want_corr ? (size_t)cols * elem_bytes_of(ct) : 0;
    const size_t disp_bytes = align_up((size_t)rows * disp_row, 256);
    const size_t corr_bytes = align_up((size_t)rows * corr_row, 256);
    Scratch& s = g_staging[g.dev % kMaxDevices];
    std::lock_guard<std::mutex> lk(s.mu);
    void* base = nullptr;
    BICOS_CUDA_TRY(scratch_acquire(s, align_up(2 * n * plane, 256) + disp_bytes + corr_bytes, st, &base));
    char* b = static_cast<char*>(base);
    char* dd = b + align_up(2 * n * plane, 256);
    char* cd = dd + disp_bytes;

    // a side's frames evenly spaced in host memory: one 2-D copy per band
    auto spacing = [&](const void* const* f) -> long long {
        const long long d = (long long)((const char*)f[1] - (const char*)f[0]);
        for (uint32_t t = 2; t < n; ++t)
            if ((long long)((const char*)f[t] - (const char*)f[t - 1]) != d)
                return 0;
        return d;
    };
    const long long sp0 = spacing(frames0), sp1 = spacing(frames1);
    const bool dense = host_step == row_bytes;
    // large stacks: two short leading bands (5 % and 12 % of the rows: the
    // first upload is the one that nothing hides, the second has to land
    // while the first band computes), then three equal bands
    const int bands = (size_t)rows * cols * n >= ((size_t)32 << 20) && rows >= 64 ? 5 : 1;
    auto band_start = [&](int k) -> int {
        if (bands == 1)
            return k == 0 ? 0 : rows;
        const int s1 = rows * 5 / 100, s2 = rows * 17 / 100;
        return k == 0 ? 0 : k == 1 ? s1 : k == 2 ? s2 : s2 + (int)((long long)(rows - s2) * (k - 2) / 3);
    };

    cudaError_t e = cudaEventRecord(hp.fork, st);
    if (e == cudaSuccess)
        e = cudaStreamWaitEvent(hp.side, hp.fork, 0);
    bicos_status rs = BICOS_OK;
    for (int k = 0; k < bands && e == cudaSuccess && rs == BICOS_OK; ++k) {
        const int r0 = band_start(k), nr = band_start(k + 1) - r0;
        if (nr <= 0)
            break;
        cudaStream_t bs = (k & 1) ? hp.side : st;
        for (int side = 0; side < 2 && e == cudaSuccess; ++side) {
            const void* const* f = side ? frames1 : frames0;
            const long long sp = side ? sp1 : sp0;
            char* dst = b + (size_t)side * n * plane + (size_t)r0 * row_bytes;
            if (dense && sp >= (long long)plane) {  // the band of every frame: n rows of nr * row_bytes
                e = cudaMemcpy2DAsync(dst, plane, (const char*)f[0] + (size_t)r0 * host_step, (size_t)sp,
                                      (size_t)nr * row_bytes, n, cudaMemcpyHostToDevice, bs);
            } else {
                for (uint32_t t = 0; t < n && e == cudaSuccess; ++t)
                    e = dense ? cudaMemcpyAsync(dst + (size_t)t * plane, (const char*)f[t] + (size_t)r0 * host_step,
                                                (size_t)nr * row_bytes, cudaMemcpyHostToDevice, bs)
                              : cudaMemcpy2DAsync(dst + (size_t)t * plane, row_bytes,
                                                  (const char*)f[t] + (size_t)r0 * host_step, host_step, row_bytes, nr,
                                                  cudaMemcpyHostToDevice, bs);
            }
        }
        if (e != cudaSuccess)
            break;
        bicos_image im0[kMaxFrames], im1[kMaxFrames];
        for (uint32_t t = 0; t < n; ++t) {
            im0[t] = bicos_image {b + (size_t)t * plane + (size_t)r0 * row_bytes, row_bytes, nr, cols, type, 0};
            im1[t] = bicos_image {b + (size_t)(n + t) * plane + (size_t)r0 * row_bytes, row_bytes, nr, cols, type, 0};
        }
        bicos_image dimg {dd + (size_t)r0 * disp_row, disp_row, nr, cols, dt, 0};
        bicos_image cimg {cd + (size_t)r0 * corr_row, corr_row, nr, cols, ct, 0};
        rs = bicos_match_v1(im0, im1, n, &dimg, want_corr ? &cimg : nullptr, cfg, bs);
        if (rs != BICOS_OK)
            break;
        auto download = [&](void* host, size_t step, const void* src, size_t row) {
            char* h = (char*)host + (size_t)r0 * step;
            return step == row ? cudaMemcpyAsync(h, src, (size_t)nr * row, cudaMemcpyDeviceToHost, bs)
                               : cudaMemcpy2DAsync(h, step, src, row, row, nr, cudaMemcpyDeviceToHost, bs);
        };
        e = download(disparity, disparity_step, dimg.data, disp_row);
        if (e == cudaSuccess && want_corr)
            e = download(corrmap, corrmap_step, cimg.data, corr_row);
    }
    cudaError_t ej = cudaEventRecord(hp.join, hp.side);
    if (ej == cudaSuccess)
        ej = cudaStreamWaitEvent(st, hp.join, 0);
    cudaError_t er = scratch_release(s, st);
    cudaError_t es = cudaStreamSynchronize(st);
    if (rs != BICOS_OK)
        return rs;
    if (e != cudaSuccess)
        return cuda_fail(e, "bicos_match_host_v1 copies");
    if (ej != cudaSuccess)
        return cuda_fail(ej, "bicos_match_host_v1 join");
    if (er != cudaSuccess)
        return cuda_fail(er, "cudaEventRecord");
    if (es != cudaSuccess)
        return cuda_fail(es, "cudaStreamSynchronize");
    return BICOS_OK;
}

bicos_status bicos_descriptor_transform_v1(const bicos_image* stack, uint32_t n, int32_t mode, uint32_t nwords,
                                           uint32_t* descriptors, bicos_stream_t stream) {
    int eb = 0;
    if (bicos_status s = check_stacks(stack, stack, n, &eb))
        return s;
    const bool full = mode == BICOS_MODE_FULL;
    const int nw = n <= (uint32_t)kMaxFrames ? words_for((int)n, full, 512) : -1;
    if (nw < 0)
        return fail(BICOS_ERR_INVALID_ARGUMENT, "input stacks too large, would require " +
                                                    std::to_string(required_bits((int)n, full)) + " bits");
    if ((int)nwords != nw)
        return fail(BICOS_ERR_INVALID_ARGUMENT, "descriptor width does not match the stack size and mode");
    if (!descriptors)
        return fail(BICOS_ERR_INVALID_ARGUMENT, "null descriptor buffer");
    StackParams p;
    fill_stack(p, stack, nullptr, n, eb);
    cudaError_t e = launch_transform(p, 1, full, nw, descriptors, descriptors, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess)
        return cuda_fail(e, "descriptor transform launch");
    return BICOS_OK;
}

namespace {

bicos_status search_stage(const uint32_t* desc0, const uint32_t* desc1, int32_t rows, int32_t cols,
                          uint32_t nwords, int bits, int32_t flags, int32_t max_lr_diff, bicos_image* disparity,
                          bicos_stream_t stream) {
    if (!desc0 || !desc1 || rows < 1 || cols < 1 || cols > 32767)
        return fail(BICOS_ERR_INVALID_ARGUMENT, "bad descriptor arguments");
    if (nwords != 1 && nwords != 2 && nwords != 4 && nwords != 8 && nwords != 12 && nwords != 16)
        return fail(BICOS_ERR_INVALID_ARGUMENT, "unsupported descriptor width");
    if (bits < 0 || bits > 32 * (int)nwords)
        return fail(BICOS_ERR_INVALID_ARGUMENT, "descriptor bit count out of range");
    if (!image_ok(disparity, rows, cols, BICOS_16S))
        return fail(BICOS_ERR_EXCEPTION, "disparity must be an int16 image of the descriptor size");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const bool nodup = (flags & BICOS_FLAG_NODUPES) != 0;
    const bool cons = (flags & BICOS_FLAG_CONSISTENCY) != 0;
    DeviceGuard g;
    if (g.err != cudaSuccess)
        return cuda_fail(g.err, "cudaGetDevice");
    // scratch: consistency bests, then the FP8 candidate tiles
    Scratch& s = g_scratch[g.dev % kMaxDevices];
    std::lock_guard<std::mutex> lk(s.mu);
    const size_t bb = cons ? align_up((size_t)rows * cols * 4, 256) : 0;
    const size_t xb = align_up(search_expand_bytes(rows, cols, (int)nwords, cons ? 2 : 1), 256);
    void* base = nullptr;
    cudaError_t e = cudaSuccess;
    if (bb + xb > 0)
        BICOS_CUDA_TRY(scratch_acquire(s, 2 * bb + xb, st, &base));
    uint8_t* xbuf = xb ? static_cast<uint8_t*>(base) + 2 * bb : nullptr;
    if (cons) {
        int32_t* fwd = static_cast<int32_t*>(base);
        int32_t* rev = reinterpret_cast<int32_t*>(static_cast<char*>(base) + bb);
        e = launch_search(desc0, desc1, rows, cols, (int)nwords, bits, nodup, 2, nullptr, 0, fwd, rev, st, xbuf);
        if (e == cudaSuccess)
            e = launch_consistency(fwd, rev, rows, cols, max_lr_diff, static_cast<int16_t*>(disparity->data),
                                   (long long)disparity->step, st);
    } else {
        e = launch_search(desc0, desc1, rows, cols, (int)nwords, bits, nodup, 1, static_cast<int16_t*>(disparity->data),
                          (long long)disparity->step, nullptr, nullptr, st, xbuf);
    }
    if (bb + xb > 0) {
        cudaError_t er = scratch_release(s, st);
        if (e == cudaSuccess)
            e = er;
    }
    if (e != cudaSuccess)
        return cuda_fail(e, "search launch");
    return BICOS_OK;
}

}  // namespace

bicos_status bicos_search_v1(const uint32_t* desc0, const uint32_t* desc1, int32_t rows, int32_t cols,
                             uint32_t nwords, int32_t flags, int32_t max_lr_diff, bicos_image* disparity,
                             bicos_stream_t stream) {
    return search_stage(desc0, desc1, rows, cols, nwords, 0, flags, max_lr_diff, disparity, stream);
}

bicos_status bicos_search_bits_v1(const uint32_t* desc0, const uint32_t* desc1, int32_t rows, int32_t cols,
                                  uint32_t nwords, int32_t bits, int32_t flags, int32_t max_lr_diff,
                                  bicos_image* disparity, bicos_stream_t stream) {
    if (bits < 1)
        return fail(BICOS_ERR_INVALID_ARGUMENT, "descriptor bit count out of range");
    return search_stage(desc0, desc1, rows, cols, nwords, bits, flags, max_lr_diff, disparity, stream);
}

bicos_status bicos_agree_v1(bicos_image* disparity, const bicos_image* stack0, const bicos_image* stack1,
                            uint32_t n, float nxcorr_threshold, int32_t has_min_var, float min_var,
                            int32_t precision, bicos_image* corrmap, bicos_stream_t stream) {
    int eb = 0;
    if (bicos_status s = check_stacks(stack0, stack1, n, &eb))
        return s;
    if (n > (uint32_t)kMaxFrames)
        return fail(BICOS_ERR_EXCEPTION, "Bad number of images");
    const int rows = stack0[0].rows, cols = stack0[0].cols;
    const bool dbl = precision == BICOS_PRECISION_DOUBLE;
    if (!image_ok(disparity, rows, cols, BICOS_16S))
        return fail(BICOS_ERR_EXCEPTION, "disparity must be an int16 image of the stack's size");
    if (corrmap && !image_ok(corrmap, rows, cols, dbl ? BICOS_64F : BICOS_32F))
        return fail(BICOS_ERR_EXCEPTION, "corrmap type or size mismatch");
    AgreeParams ap;
    std::memset(&ap, 0, sizeof ap);
    ap.one = 1.0f;
    fill_stack(ap.s, stack0, stack1, n, eb);
    ap.raw_io = static_cast<int16_t*>(disparity->data);
    ap.raw_pitch = (long long)disparity->step;
    ap.thr = nxcorr_threshold;
    ap.has_minvar = has_min_var != 0;
    ap.minvar = min_var;
    ap.corr = corrmap ? corrmap->data : nullptr;
    ap.corr_pitch = corrmap ? (long long)corrmap->step : 0;
    cudaError_t e = launch_agree(ap, dbl, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess)
        return cuda_fail(e, "agree launch");
    return BICOS_OK;
}

bicos_status bicos_agree_subpixel_v1(const bicos_image* raw_disparity, const bicos_image* stack0,
                                     const bicos_image* stack1, uint32_t n, float nxcorr_threshold,
                                     float subpixel_step, int32_t has_min_var, float min_var, int32_t precision,
                                     bicos_image* disparity, bicos_image* corrmap, bicos_stream_t stream) {
    int eb = 0;
    if (bicos_status s = check_stacks(stack0, stack1, n, &eb))
        return s;
    if (n > (uint32_t)kMaxFrames)
        return fail(BICOS_ERR_EXCEPTION, "Bad number of images");
    const int rows = stack0[0].rows, cols = stack0[0].cols;
    const bool dbl = precision == BICOS_PRECISION_DOUBLE;
    if (!step_ok(subpixel_step))
        return fail(BICOS_ERR_EXCEPTION, "subpixel step must be a finite value >= 1e-4");
    if (!image_ok(raw_disparity, rows, cols, BICOS_16S))
        return fail(BICOS_ERR_EXCEPTION, "raw disparity must be an int16 image of the stack's size");
    if (!image_ok(disparity, rows, cols, BICOS_32F))
        return fail(BICOS_ERR_EXCEPTION, "disparity must be a float32 image of the stack's size");
    if (corrmap && !image_ok(corrmap, rows, cols, dbl ? BICOS_64F : BICOS_32F))
        return fail(BICOS_ERR_EXCEPTION, "corrmap type or size mismatch");
    AgreeParams ap;
    std::memset(&ap, 0, sizeof ap);
    ap.one = 1.0f;
    fill_stack(ap.s, stack0, stack1, n, eb);
    ap.raw = static_cast<const int16_t*>(raw_disparity->data);
    ap.raw_pitch = (long long)raw_disparity->step;
    ap.out = disparity->data;
    ap.out_pitch = (long long)disparity->step;
    ap.thr = nxcorr_threshold;
    ap.step = subpixel_step;
    ap.has_minvar = has_min_var != 0;
    ap.minvar = min_var;
    ap.corr = corrmap ? corrmap->data : nullptr;
    ap.corr_pitch = corrmap ? (long long)corrmap->step : 0;
    cudaError_t e = launch_agree_subpixel(ap, dbl, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess)
        return cuda_fail(e, "agree_subpixel launch");
    return BICOS_OK;
}

bicos_status bicos_subpixel_features_v1(const bicos_image* raw_disparity, const bicos_image* stack0,
                                        const bicos_image* stack1, uint32_t n, bicos_image* features,
                                        bicos_stream_t stream) {
    int eb = 0;
    if (bicos_status s = check_stacks(stack0, stack1, n, &eb))
        return s;
    if (n > (uint32_t)kMaxFrames)
        return fail(BICOS_ERR_EXCEPTION, "Bad number of images");
    const int rows = stack0[0].rows, cols = stack0[0].cols;
    if (!image_ok(raw_disparity, rows, cols, BICOS_16S))
        return fail(BICOS_ERR_EXCEPTION, "raw disparity must be an int16 image of the stack's size");
    if (!features || !features->data || features->rows != rows || features->cols != 8 * cols ||
        features->type != BICOS_32F || features->step < (size_t)cols * 32 || features->step % 16 != 0 ||
        reinterpret_cast<uintptr_t>(features->data) % 16 != 0)
        return fail(BICOS_ERR_EXCEPTION, "features must be a 16-byte aligned float32 image of rows x 8*cols");
    MomentParams mp;
    std::memset(&mp, 0, sizeof mp);
    fill_stack(mp.s, stack0, stack1, n, eb);
    mp.raw = static_cast<const int16_t*>(raw_disparity->data);
    mp.raw_pitch = (long long)raw_disparity->step;
    mp.out = features->data;
    mp.out_pitch = (long long)features->step;
    cudaError_t e = launch_moments(mp, 2, false, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess)
        return cuda_fail(e, "features launch");
    return BICOS_OK;
}

bicos_status bicos_agree_learned_v1(const bicos_image* raw_disparity, const bicos_image* stack0,
                                    const bicos_image* stack1, uint32_t n, float nxcorr_threshold,
                                    float subpixel_step, int32_t has_min_var, float min_var, int32_t precision,
                                    bicos_image* disparity, bicos_image* corrmap, bicos_image* proposals,
                                    int32_t* fallback_count, bicos_stream_t stream) {
    int eb = 0;
    if (bicos_status s = check_stacks(stack0, stack1, n, &eb))
        return s;
    if (n > (uint32_t)kMaxFrames)
        return fail(BICOS_ERR_EXCEPTION, "Bad number of images");
    const int rows = stack0[0].rows, cols = stack0[0].cols;
    const bool dbl = precision == BICOS_PRECISION_DOUBLE;
    if (!step_ok(subpixel_step))
        return fail(BICOS_ERR_EXCEPTION, "subpixel step must be a finite value >= 1e-4");
    if (!image_ok(raw_disparity, rows, cols, BICOS_16S))
        return fail(BICOS_ERR_EXCEPTION, "raw disparity must be an int16 image of the stack's size");
    if (!image_ok(disparity, rows, cols, BICOS_32F))
        return fail(BICOS_ERR_EXCEPTION, "disparity must be a float32 image of the stack's size");
    if (corrmap && !image_ok(corrmap, rows, cols, dbl ? BICOS_64F : BICOS_32F))
        return fail(BICOS_ERR_EXCEPTION, "corrmap type or size mismatch");
    if (proposals && !image_ok(proposals, rows, cols, BICOS_32F))
        return fail(BICOS_ERR_EXCEPTION, "proposals must be a float32 image of the stack's size");
    DeviceGuard g;
    if (g.err != cudaSuccess)
        return cuda_fail(g.err, "cudaGetDevice");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    std::string err;
    const float* model = learned_model_device(st, &err);
    if (!model)
        return fail(BICOS_ERR_INVALID_ARGUMENT, err);
    AgreeParams ap;
    std::memset(&ap, 0, sizeof ap);
    ap.one = 1.0f;
    fill_stack(ap.s, stack0, stack1, n, eb);
    ap.raw = static_cast<const int16_t*>(raw_disparity->data);
    ap.raw_pitch = (long long)raw_disparity->step;
    ap.out = disparity->data;
    ap.out_pitch = (long long)disparity->step;
    ap.thr = nxcorr_threshold;
    ap.step = subpixel_step;
    ap.has_minvar = has_min_var != 0;
    ap.minvar = min_var;
    ap.corr = corrmap ? corrmap->data : nullptr;
    ap.corr_pitch = corrmap ? (long long)corrmap->step : 0;
    Scratch& s = g_scratch[g.dev % kMaxDevices];
    std::lock_guard<std::mutex> lk(s.mu);
    void* base = nullptr;
    BICOS_CUDA_TRY(scratch_acquire(s, learned_scratch_bytes((size_t)rows * cols), st, &base));
    cudaError_t e = learned_subpixel(ap, dbl, model, base, fallback_count,
                                     proposals ? static_cast<float*>(proposals->data) : nullptr,
                                     proposals ? (long long)proposals->step : 0, st);
    cudaError_t er = scratch_release(s, st);
    if (e == cudaSuccess)
        e = er;
    if (e != cudaSuccess)
        return cuda_fail(e, "learned agree launch");
    return BICOS_OK;
}

bicos_status bicos_reproject_v1(const bicos_image* disparity, const double* q, bicos_image* points,
                                bicos_stream_t stream) {
    if (!disparity || !q || !points)
        return fail(BICOS_ERR_INVALID_ARGUMENT, "null argument");
    if (disparity->type != BICOS_16S && disparity->type != BICOS_32F)
        return fail(BICOS_ERR_EXCEPTION, "disparity must be an int16 or float32 image");
    if (disparity->rows < 1 || disparity->cols < 1 || !image_ok(disparity, disparity->rows, disparity->cols,
                                                               disparity->type))
        return fail(BICOS_ERR_EXCEPTION, "bad disparity image");
    if (!image_ok(points, disparity->rows, disparity->cols, BICOS_32FC3))
        return fail(BICOS_ERR_EXCEPTION, "points must be a three-channel float32 image of the disparity's size");
    ReprojectParams p;
    p.disp = disparity->data;
    p.disp_pitch = (long long)disparity->step;
    p.pts = static_cast<float*>(points->data);
    p.pts_pitch = (long long)points->step;
    p.rows = disparity->rows;
    p.cols = disparity->cols;
    for (int i = 0; i < 16; ++i) {
        if (!std::isfinite(q[i]))
            return fail(BICOS_ERR_INVALID_ARGUMENT, "Q must be finite");
        p.q[i] = (float)q[i];
    }
    cudaError_t e = launch_reproject(p, disparity->type == BICOS_32F, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess)
        return cuda_fail(e, "reprojection launch");
    return BICOS_OK;
}

}  // extern "C"
