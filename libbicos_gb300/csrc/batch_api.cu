// Batch API: many stereo stacks of mixed size, depth, input type and
// configuration in one call (no counterpart in libBICOS, whose match()
// takes one stack, src/impl/cuda.cu.in:233-292).
//
// One call = one CUDA graph, captured once per batch signature (the items'
// shapes, types, configurations, buffer addresses and the launch tuning)
// and replayed afterwards:
//   1. one persistent multi-stack launch per descriptor-transform class
//      (input type x mode x descriptor width) over a work table of
//      (stack, column block, row, side) virtual blocks (batch.cuh);
//   2. the Hamming search (+ consistency) of each stack, on `branches`
//      concurrent graph branches;
//   3. one persistent multi-stack launch per reference-form agreement class
//      (input type x kind x precision x frame bucket); the moment and
//      learned forms run per stack on the branches.
// Every kernel is the one bicos_match_v1 runs (block bodies shared through
// batch.cuh), so each stack's results are bit-identical to a sequential
// bicos_match_v1 call.  The autotuner times graph replays over the launch
// shapes (transform block width, persistent CTAs per SM, virtual blocks per
// claim, branch count) -- none of which changes a result.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/bicos_c.h"
#include "batch.cuh"
#include "kernels.cuh"
#include "match_plan.hpp"

using namespace bicos_gb300;

namespace {

constexpr int kMaxBranches = 4;
constexpr size_t kMaxGraphs = 4;

struct Tuning {
    int transform_block = 256;
    int ctas_per_sm = 8;
    int claim = 2;
    int branches = 4;
    int persistent = 3;  // bit 0: transform, bit 1: agreement as persistent multi-stack launches
};

struct GraphEntry {
    std::string key;
    cudaGraphExec_t exec = nullptr;
    void* scratch = nullptr;  // per-stack scratch regions
    void* tables = nullptr;   // work tables and claim counters
    cudaEvent_t done = nullptr;
    bool launched = false;
    unsigned long long last_use = 0;
};

void release(GraphEntry& g) {
    if (g.done && g.launched)
        cudaEventSynchronize(g.done);
    if (g.exec)
        cudaGraphExecDestroy(g.exec);
    if (g.scratch)
        cudaFree(g.scratch);
    if (g.tables)
        cudaFree(g.tables);
    if (g.done)
        cudaEventDestroy(g.done);
    g = GraphEntry{};
}

size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

template<typename T>
void put(std::string& k, const T& v) {
    k.append(reinterpret_cast<const char*>(&v), sizeof v);
}

// the batch's signature: with_addresses false gives the shape signature
// the tuning table is keyed by
std::string batch_key(const bicos_batch_item* items, uint32_t count, const std::vector<MatchPlan>& plans,
                      bool with_addresses) {
    std::string k;
    put(k, count);
    for (uint32_t i = 0; i < count; ++i) {
        const MatchPlan& P = plans[i];
        put(k, P.n);
        put(k, P.eb);
        put(k, P.rows);
        put(k, P.cols);
        put(k, *P.cfg);
        put(k, P.corrmap != nullptr);
        if (with_addresses) {
            for (int t = 0; t < P.n; ++t) {
                put(k, P.s.frame[0][t]);
                put(k, P.s.pitch[0][t]);
                put(k, P.s.frame[1][t]);
                put(k, P.s.pitch[1][t]);
            }
            put(k, P.disparity->data);
            put(k, P.disparity->step);
            if (P.corrmap) {
                put(k, P.corrmap->data);
                put(k, P.corrmap->step);
            }
        }
    }
    (void)items;
    return k;
}

}  // namespace

struct bicos_batch {
    int device = -1;
    int sms = 0;
    cudaStream_t cap = nullptr;
    cudaStream_t branch[kMaxBranches] = {};
    cudaEvent_t fork[2] = {};
    cudaEvent_t join[2][kMaxBranches] = {};
    Tuning tuning;
    bool fixed_tuning = false;  // set by bicos_batch_set_tuning_v1
    std::map<std::string, Tuning> tuned;
    std::vector<GraphEntry> graphs;
    unsigned long long clock = 0;
    int captures = 0;
};

namespace {

bicos_status batch_fail(bicos_status s, const std::string& msg) {
    set_last_error(msg);
    return s;
}

bicos_status batch_cuda_fail(cudaError_t e, const char* where) {
    return batch_fail(BICOS_ERR_CUDA, std::string("libBICOS CUDA error in ") + where + ": " + cudaGetErrorString(e));
}

cudaError_t ensure_device(bicos_batch* b) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    if (b->device == dev)
        return cudaSuccess;
    if (b->device >= 0)
        return cudaErrorInvalidDevice;  // a handle serves one device
    e = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking);
    for (int k = 0; k < kMaxBranches && e == cudaSuccess; ++k)
        e = cudaStreamCreateWithFlags(&b->branch[k], cudaStreamNonBlocking);
    for (int f = 0; f < 2 && e == cudaSuccess; ++f) {
        e = cudaEventCreateWithFlags(&b->fork[f], cudaEventDisableTiming);
        for (int k = 0; k < kMaxBranches && e == cudaSuccess; ++k)
            e = cudaEventCreateWithFlags(&b->join[f][k], cudaEventDisableTiming);
    }
    if (e == cudaSuccess)
        b->device = dev;
    return e;
}

// the transform class of a plan, and the agreement class of a reference-form plan
struct TfClass {
    int eb;
    bool full;
    int key;
    bool operator<(const TfClass& o) const {
        return std::tie(eb, full, key) < std::tie(o.eb, o.full, o.key);
    }
};
struct AgClass {
    int eb, kind;
    bool dbl;
    int nmax;
    bool operator<(const AgClass& o) const {
        return std::tie(eb, kind, dbl, nmax) < std::tie(o.eb, o.kind, o.dbl, o.nmax);
    }
};

bool batched_agree(const MatchPlan& P) { return P.thr && !P.moments && !P.learned; }

// Builds and instantiates the graph of one batch into g (scratch and claim
// counters allocated before the capture; the stacks' parameters travel in
// the persistent launches' kernel parameters).
cudaError_t build_graph(bicos_batch* b, const std::vector<MatchPlan>& plans, const std::vector<const float*>& models,
                        const Tuning& tn, GraphEntry& g, std::string* where) {
    const size_t count = plans.size();
    // scratch regions
    std::vector<size_t> scr_off(count);
    size_t scr_total = 0;
    for (size_t i = 0; i < count; ++i) {
        scr_off[i] = scr_total;
        scr_total += align256(plans[i].scratch_bytes());
    }
    cudaError_t e = cudaMalloc(&g.scratch, std::max<size_t>(scr_total, 256));
    if (e != cudaSuccess)
        return e;
    std::vector<MatchBuffers> bufs(count);
    for (size_t i = 0; i < count; ++i)
        bufs[i] = match_buffers(plans[i], static_cast<char*>(g.scratch) + scr_off[i]);

    // classes, split into launches of at most kBatchJobs stacks
    std::map<TfClass, std::vector<size_t>> tf_classes;
    std::map<AgClass, std::vector<size_t>> ag_classes;
    const bool tf_persistent = tn.persistent & 1, ag_persistent = tn.persistent & 2;
    for (size_t i = 0; i < count; ++i) {
        const MatchPlan& P = plans[i];
        if (tf_persistent)
            tf_classes[{P.eb, P.full, P.full ? P.n : P.nw}].push_back(i);
        if (ag_persistent && batched_agree(P))
            ag_classes[{P.eb, P.sub ? (P.dbl ? 2 : 1) : 0, P.dbl, agree_bucket(P.n)}].push_back(i);
    }
    auto grid_of = [&](int total) {
        const int want = (total + tn.claim - 1) / tn.claim;
        return std::max(1, std::min(want, b->sms * tn.ctas_per_sm));
    };
    struct TfLaunch {
        TfClass c;
        BatchArgs<TransformJob> a;
        BatchLaunch l;
    };
    struct AgLaunch {
        AgClass c;
        BatchArgs<AgreeParams> a;
        BatchLaunch l;
    };
    std::vector<TfLaunch> tf_launches;
    std::vector<AgLaunch> ag_launches;
    for (auto& kv : tf_classes)
        for (size_t c0 = 0; c0 < kv.second.size(); c0 += kBatchJobs) {
            TfLaunch L;
            std::memset(&L.a, 0, sizeof L.a);
            L.c = kv.first;
            int start = 0, j = 0;
            for (size_t c = c0; c < std::min(kv.second.size(), c0 + kBatchJobs); ++c, ++j) {
                const size_t i = kv.second[c];
                L.a.jobs[j].s = plans[i].s;
                L.a.jobs[j].d0 = bufs[i].d0;
                L.a.jobs[j].d1 = bufs[i].d1;
                L.a.tiles[j] = BatchTile{start, (plans[i].cols + tn.transform_block - 1) / tn.transform_block,
                                         plans[i].rows, 2};
                start += L.a.tiles[j].gx * L.a.tiles[j].gy * 2;
            }
            L.a.nstacks = j;
            L.a.total = start;
            L.a.claim = tn.claim;
            L.l = BatchLaunch{grid_of(start), tn.transform_block};
            tf_launches.push_back(L);
        }
    for (auto& kv : ag_classes)
        for (size_t c0 = 0; c0 < kv.second.size(); c0 += kBatchJobs) {
            AgLaunch L;
            std::memset(&L.a, 0, sizeof L.a);
            L.c = kv.first;
            const int block = agree_block(L.c.kind);
            int start = 0, j = 0;
            for (size_t c = c0; c < std::min(kv.second.size(), c0 + kBatchJobs); ++c, ++j) {
                const size_t i = kv.second[c];
                L.a.jobs[j] = agree_params(plans[i], bufs[i]);
                L.a.tiles[j] = BatchTile{start, (plans[i].cols + block - 1) / block, plans[i].rows, 1};
                start += L.a.tiles[j].gx * L.a.tiles[j].gy;
            }
            L.a.nstacks = j;
            L.a.total = start;
            L.a.claim = tn.claim;
            L.l = BatchLaunch{grid_of(start), block};
            ag_launches.push_back(L);
        }
    const int counters = (int)(tf_launches.size() + ag_launches.size());
    e = cudaMalloc(&g.tables, sizeof(int) * std::max(counters, 1));
    if (e == cudaSuccess)
        e = cudaEventCreateWithFlags(&g.done, cudaEventDisableTiming);
    if (e != cudaSuccess)
        return e;
    int* dcounters = static_cast<int*>(g.tables);
    int next_counter = 0;
    for (TfLaunch& L : tf_launches)
        L.a.counter = dcounters + next_counter++;
    for (AgLaunch& L : ag_launches)
        L.a.counter = dcounters + next_counter++;
    const int branches = std::max(1, std::min(tn.branches, kMaxBranches));

    // capture (a stale error of this thread would be read back by the
    // launches' cudaGetLastError)
    cudaGetLastError();
    e = cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess)
        return e;
    cudaError_t ce = cudaMemsetAsync(dcounters, 0, sizeof(int) * std::max(counters, 1), b->cap);
    if (ce != cudaSuccess)
        *where = "counter reset";
    for (const TfLaunch& L : tf_launches)
        if (ce == cudaSuccess) {
            ce = launch_transform_batch(L.c.eb, L.c.full, L.c.key, L.a, L.l, b->cap);
            if (ce != cudaSuccess)
                *where = "transform launch (key " + std::to_string(L.c.key) + ")";
        }
    auto fork_join = [&](int f, auto&& body) {
        cudaError_t r = cudaEventRecord(b->fork[f], b->cap);
        for (int k = 0; k < branches && r == cudaSuccess; ++k)
            r = cudaStreamWaitEvent(b->branch[k], b->fork[f], 0);
        if (r == cudaSuccess)
            r = body();
        for (int k = 0; k < branches; ++k) {
            cudaError_t r2 = cudaEventRecord(b->join[f][k], b->branch[k]);
            if (r2 == cudaSuccess)
                r2 = cudaStreamWaitEvent(b->cap, b->join[f][k], 0);
            if (r == cudaSuccess)
                r = r2;
        }
        return r;
    };
    if (ce == cudaSuccess)
        ce = fork_join(0, [&]() {
            cudaError_t r = cudaSuccess;
            for (size_t i = 0; i < count && r == cudaSuccess; ++i) {
                cudaStream_t bs = b->branch[i % branches];
                if (!tf_persistent) {
                    r = enqueue_transform(plans[i], bufs[i], bs);
                    if (r != cudaSuccess) {
                        *where = "transform of item " + std::to_string(i);
                        break;
                    }
                }
                r = enqueue_search(plans[i], bufs[i], bs, !tf_persistent);
                if (r != cudaSuccess)
                    *where = "search of item " + std::to_string(i);
            }
            return r;
        });
    for (const AgLaunch& L : ag_launches)
        if (ce == cudaSuccess) {
            ce = launch_agree_batch(L.c.eb, L.c.kind, L.c.dbl, L.c.nmax, L.a, L.l, b->cap);
            if (ce != cudaSuccess)
                *where = "agreement launch (kind " + std::to_string(L.c.kind) + ", frames " +
                         std::to_string(L.c.nmax) + ")";
        }
    auto per_stack_agree = [&](const MatchPlan& P) { return P.thr && (!ag_persistent || !batched_agree(P)); };
    bool per_stack = false;
    for (const MatchPlan& P : plans)
        per_stack |= per_stack_agree(P);
    if (ce == cudaSuccess && per_stack)
        ce = fork_join(1, [&]() {
            cudaError_t r = cudaSuccess;
            int k = 0;
            for (size_t i = 0; i < count && r == cudaSuccess; ++i)
                if (per_stack_agree(plans[i])) {
                    r = enqueue_agree(plans[i], bufs[i], models[i], b->branch[k++ % branches]);
                    if (r != cudaSuccess)
                        *where = "agreement of item " + std::to_string(i);
                }
            return r;
        });
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(b->cap, &graph);
    if (e != cudaSuccess && where->empty())
        *where = "end of capture";
    if (ce != cudaSuccess)
        e = ce;
    if (e == cudaSuccess) {
        e = cudaGraphInstantiate(&g.exec, graph, 0);
        if (e != cudaSuccess)
            *where = "graph instantiation";
    }
    if (graph)
        cudaGraphDestroy(graph);
    b->captures++;
    return e;
}

bicos_status plan_all(const bicos_batch_item* items, uint32_t count, std::vector<MatchPlan>& plans) {
    plans.resize(count);
    for (uint32_t i = 0; i < count; ++i) {
        const bicos_batch_item& it = items[i];
        bicos_status s = plan_match(it.stack0, it.stack1, it.n, it.disparity, it.corrmap, it.cfg, &plans[i]);
        if (s != BICOS_OK) {
            const std::string msg = bicos_last_error();
            return batch_fail(s, "batch item " + std::to_string(i) + ": " + msg);
        }
    }
    return BICOS_OK;
}

// runs the batch with tuning tn: cached graph or a new capture
bicos_status run_batch(bicos_batch* b, const bicos_batch_item* items, uint32_t count, cudaStream_t st,
                       const std::vector<MatchPlan>& plans, const Tuning& tn, GraphEntry** used) {
    std::vector<const float*> models(count, nullptr);
    for (uint32_t i = 0; i < count; ++i)
        if (plans[i].learned) {
            std::string err;
            models[i] = learned_model_device(st, &err);
            if (!models[i])
                return batch_fail(BICOS_ERR_INVALID_ARGUMENT, "batch item " + std::to_string(i) + ": " + err);
        }
    std::string key = batch_key(items, count, plans, true);
    put(key, tn);
    GraphEntry* g = nullptr;
    for (GraphEntry& x : b->graphs)
        if (x.key == key)
            g = &x;
    if (!g) {
        if (b->graphs.size() >= kMaxGraphs) {
            auto old = std::min_element(b->graphs.begin(), b->graphs.end(),
                                        [](const GraphEntry& a, const GraphEntry& c) { return a.last_use < c.last_use; });
            release(*old);
            b->graphs.erase(old);
        }
        b->graphs.emplace_back();
        g = &b->graphs.back();
        g->key = key;
        std::string where;
        cudaError_t e = build_graph(b, plans, models, tn, *g, &where);
        if (e != cudaSuccess) {
            cudaGetLastError();  // the failed capture's error is reported here, not by later calls
            release(*g);
            b->graphs.pop_back();
            return batch_cuda_fail(e, ("batch graph capture, " + (where.empty() ? std::string("set-up") : where)).c_str());
        }
    }
    // replays of one graph share its scratch: order them on the caller's streams
    cudaError_t e = g->launched ? cudaStreamWaitEvent(st, g->done, 0) : cudaSuccess;
    if (e == cudaSuccess)
        e = cudaGraphLaunch(g->exec, st);
    if (e == cudaSuccess)
        e = cudaEventRecord(g->done, st);
    if (e != cudaSuccess)
        return batch_cuda_fail(e, "cudaGraphLaunch");
    g->launched = true;
    g->last_use = ++b->clock;
    if (used)
        *used = g;
    return BICOS_OK;
}

Tuning from_c(const bicos_batch_tuning& t) {
    Tuning r;
    r.transform_block = t.transform_block;
    r.ctas_per_sm = t.ctas_per_sm;
    r.claim = t.claim;
    r.branches = t.branches;
    r.persistent = t.persistent;
    return r;
}

bicos_batch_tuning to_c(const Tuning& t) {
    bicos_batch_tuning r;
    r.transform_block = t.transform_block;
    r.ctas_per_sm = t.ctas_per_sm;
    r.claim = t.claim;
    r.branches = t.branches;
    r.persistent = t.persistent;
    return r;
}

bool tuning_ok(const bicos_batch_tuning& t) {
    return (t.transform_block == 64 || t.transform_block == 128 || t.transform_block == 256) &&
           t.ctas_per_sm >= 1 && t.ctas_per_sm <= 32 && t.claim >= 1 && t.claim <= 64 && t.branches >= 1 &&
           t.branches <= kMaxBranches && t.persistent >= 0 && t.persistent <= 3;
}

}  // namespace

extern "C" {

bicos_status bicos_batch_create(bicos_batch** out) {
    if (!out)
        return batch_fail(BICOS_ERR_INVALID_ARGUMENT, "null handle pointer");
    *out = new bicos_batch();
    return BICOS_OK;
}

bicos_status bicos_batch_destroy(bicos_batch* b) {
    if (!b)
        return BICOS_OK;
    for (GraphEntry& g : b->graphs)
        release(g);
    if (b->cap)
        cudaStreamDestroy(b->cap);
    for (int k = 0; k < kMaxBranches; ++k)
        if (b->branch[k])
            cudaStreamDestroy(b->branch[k]);
    for (int f = 0; f < 2; ++f) {
        if (b->fork[f])
            cudaEventDestroy(b->fork[f]);
        for (int k = 0; k < kMaxBranches; ++k)
            if (b->join[f][k])
                cudaEventDestroy(b->join[f][k]);
    }
    delete b;
    return BICOS_OK;
}

bicos_status bicos_match_batch_v1(bicos_batch* b, const bicos_batch_item* items, uint32_t count,
                                  bicos_stream_t stream) {
    if (!b)
        return batch_fail(BICOS_ERR_INVALID_ARGUMENT, "null batch handle");
    if (count == 0)
        return BICOS_OK;
    if (!items)
        return batch_fail(BICOS_ERR_INVALID_ARGUMENT, "null batch items");
    std::vector<MatchPlan> plans;
    if (bicos_status s = plan_all(items, count, plans))
        return s;
    cudaError_t e = ensure_device(b);
    if (e != cudaSuccess)
        return batch_cuda_fail(e, "batch set-up");
    Tuning tn = b->tuning;
    if (!b->fixed_tuning) {
        auto it = b->tuned.find(batch_key(items, count, plans, false));
        if (it != b->tuned.end())
            tn = it->second;
    }
    return run_batch(b, items, count, reinterpret_cast<cudaStream_t>(stream), plans, tn, nullptr);
}

bicos_status bicos_batch_autotune_v1(bicos_batch* b, const bicos_batch_item* items, uint32_t count,
                                     bicos_stream_t stream, bicos_batch_tuning* chosen) {
    if (!b || !items || count == 0)
        return batch_fail(BICOS_ERR_INVALID_ARGUMENT, "batch autotune needs a handle and items");
    std::vector<MatchPlan> plans;
    if (bicos_status s = plan_all(items, count, plans))
        return s;
    cudaError_t e = ensure_device(b);
    if (e != cudaSuccess)
        return batch_cuda_fail(e, "batch set-up");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    cudaEvent_t t0, t1;
    if ((e = cudaEventCreate(&t0)) != cudaSuccess || (e = cudaEventCreate(&t1)) != cudaSuccess)
        return batch_cuda_fail(e, "cudaEventCreate");
    // time of one batch with tuning tn: best of three replays after a warm-up
    auto measure = [&](const Tuning& tn, float* ms) -> bicos_status {
        GraphEntry* g = nullptr;
        if (bicos_status s = run_batch(b, items, count, st, plans, tn, &g))
            return s;
        float best = 1e30f;
        for (int r = 0; r < 3; ++r) {
            cudaEventRecord(t0, st);
            if (bicos_status s = run_batch(b, items, count, st, plans, tn, &g))
                return s;
            cudaEventRecord(t1, st);
            cudaError_t ee = cudaEventSynchronize(t1);
            float v = 0.f;
            if (ee == cudaSuccess)
                ee = cudaEventElapsedTime(&v, t0, t1);
            if (ee != cudaSuccess)
                return batch_cuda_fail(ee, "autotune timing");
            best = std::min(best, v);
        }
        *ms = best;
        return BICOS_OK;
    };
    // coordinate descent over the launch shapes
    Tuning cur = b->tuning;
    float cur_ms = 0.f;
    bicos_status s = measure(cur, &cur_ms);
    const std::vector<int> pers = {0, 1, 2, 3}, blocks = {64, 128, 256}, ctas = {2, 4, 8, 16}, claims = {1, 2, 4},
                           brs = {1, 2, 4};
    for (int dim = 0; dim < 5 && s == BICOS_OK; ++dim) {
        const std::vector<int>& cands =
            dim == 0 ? pers : dim == 1 ? blocks : dim == 2 ? ctas : dim == 3 ? claims : brs;
        for (int v : cands) {
            Tuning t = cur;
            int& field = dim == 0   ? t.persistent
                         : dim == 1 ? t.transform_block
                         : dim == 2 ? t.ctas_per_sm
                         : dim == 3 ? t.claim
                                    : t.branches;
            if (field == v)
                continue;
            field = v;
            float ms = 0.f;
            s = measure(t, &ms);
            if (s != BICOS_OK)
                break;
            if (ms < cur_ms) {
                cur = t;
                cur_ms = ms;
            }
        }
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    if (s != BICOS_OK)
        return s;
    b->tuned[batch_key(items, count, plans, false)] = cur;
    // keep only the chosen tuning's graph
    std::string keep = batch_key(items, count, plans, true);
    put(keep, cur);
    for (size_t i = 0; i < b->graphs.size();) {
        if (b->graphs[i].key != keep) {
            release(b->graphs[i]);
            b->graphs.erase(b->graphs.begin() + i);
        } else {
            ++i;
        }
    }
    if (chosen)
        *chosen = to_c(cur);
    return BICOS_OK;
}

bicos_status bicos_batch_get_tuning_v1(const bicos_batch* b, bicos_batch_tuning* out) {
    if (!b || !out)
        return batch_fail(BICOS_ERR_INVALID_ARGUMENT, "null argument");
    *out = to_c(b->tuning);
    return BICOS_OK;
}

bicos_status bicos_batch_set_tuning_v1(bicos_batch* b, const bicos_batch_tuning* t) {
    if (!b)
        return batch_fail(BICOS_ERR_INVALID_ARGUMENT, "null batch handle");
    if (!t) {
        b->tuning = Tuning{};
        b->fixed_tuning = false;
        return BICOS_OK;
    }
    if (!tuning_ok(*t))
        return batch_fail(BICOS_ERR_INVALID_ARGUMENT,
                          "batch tuning out of range (transform_block 64/128/256, ctas_per_sm 1..32, "
                          "claim 1..64, branches 1..4, persistent 0..3)");
    b->tuning = from_c(*t);
    b->fixed_tuning = true;
    return BICOS_OK;
}

int32_t bicos_batch_captures(const bicos_batch* b) { return b ? b->captures : 0; }

}  // extern "C"
