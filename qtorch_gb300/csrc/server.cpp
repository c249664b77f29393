// Continuous-batching request server.
//
// Requests (a plan plus its leaf values) are admitted in arrival order while
// their device footprint (plan workspace + leaves, per precision) fits the
// memory budget and an in-flight slot is free.  Light requests (plans the
// grouped interpreter takes) are grouped into waves that run as one grouped
// launch; a heavy request (a plan run step by step with the whole-GPU
// kernels) is a wave of its own, and so is a request larger than the whole
// budget, which is sliced at submission (qt_plan_slice) and runs slice by
// slice.  Waves run on lanes, each lane with its own
// CUDA stream, so a wave formed from requests that arrived while another wave
// is on the GPU runs concurrently with it.  Lane 0 (highest stream priority)
// takes the small requests (grouped, at most 2^20 complex MACs) and nothing
// else, so they never queue behind a heavy one nor run on a low-priority
// stream beside one; the other lanes take the rest, lane 1 the pending medium
// requests (grouped, above the small bound) before any heavy one.  Each
// request's result is independent of what it was batched with: an instance
// only ever touches its
// own leaves and its CTA's workspace.
#include <algorithm>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <thread>
#include <unordered_map>

#include "gemm_tc.h"
#include "kernels.h"
#include "plan.h"

using namespace qtg;

namespace {

struct Request {
    int64_t ticket;
    qt_plan *plan;
    const qt_sliced *sliced = nullptr;   // the plan sliced to fit the budget (runs alone, slice by slice)
    std::vector<double> leaves;
    std::chrono::steady_clock::time_point t_submit;
    std::chrono::steady_clock::time_point t_admit;   // taken into a wave
    uint64_t footprint;
    bool heavy;
    bool small;   // lane 0 material: grouped and at most kLaneZeroMaxMacs
    int retries = 0;      // runs that ran out of device memory
    bool alone = false;   // after one: admitted only when nothing else is in flight
};

// A heavy request that runs out of device memory while others hold it (the
// budget counts plans' workspaces, not the blocks the lanes' allocators keep)
// goes back to the head of the queue and runs again alone, up to this many times.
constexpr int kMaxOomRetries = 2;

struct Result {
    int state = 0;   // 0 pending, 1 done, <0 -status
    double v[2] = {0, 0};
    double latency = 0;
    double queued = 0;   // seconds from submission to admission into a wave
    int lane = -1;
};

}  // namespace

struct qt_server {
    qt_ctx *ctx = nullptr;                 // the caller's context (device, budget)
    int max_inflight = 64;
    qt_precision prec = QT_PREC_FP64;
    int64_t max_macs = 0;                  // work cap of one request (complex MACs, all slices); 0: none
    int64_t refused = 0;                   // submissions refused by the work cap or the budget
    int64_t oom_retries = 0;               // heavy runs repeated alone after running out of memory
    uint64_t wave_ends = 0;                // waves finished (or returned for a retry) so far
    std::mutex m;
    std::condition_variable cv;            // new work or a lane became free
    std::condition_variable done_cv;       // a request finished
    std::deque<Request> pending;
    std::unordered_map<int64_t, Result> results;
    int64_t next_ticket = 0;
    int inflight = 0;
    uint64_t inflight_bytes = 0;
    bool stop = false;
    std::vector<double> latencies;
    int64_t completed = 0;
    int64_t launches = 0;
    int64_t waves = 0, wave_requests = 0;
    double wave_seconds = 0;                 // lane time spent on waves (batch build, launch, read-back)
    struct Lane {
        qt_ctx *ctx = nullptr;
        std::thread th;
        std::vector<Request> wave;
        bool busy = false;
    };
    std::vector<Lane> lanes;
    std::thread dispatcher;
};

// slicings are cached in the plans, which several servers may share
static std::mutex g_slicing_lock;
// cut wires a request may be sliced over to fit the budget (4^16 slices, run
// in chunks; the work cap bounds what that costs)
constexpr int kServerMaxCuts = 16;

// Lane 0 serves small requests only (a QAOA term is 1e4-3e5 complex MACs):
// a mid-size request (a 12-14 qubit circuit, 1e6-1.6e7 MACs) takes one CTA
// for a millisecond or more and would hold up the small ones behind it.
constexpr int64_t kLaneZeroMaxMacs = 1ll << 20;
constexpr size_t kLaneMinBlock = 1u << 20;
constexpr int kLaneWarmBlocks = 8;

static uint64_t footprint(const qt_plan *p, qt_precision prec) {
    return p->ws_bytes[prec] + p->leaf_bytes[prec] + 4096;
}

// a plan run step by step also holds, during its largest tensor-core step,
// that step's packed operands (gemm_tc.h)
static uint64_t stepwise_scratch(const qt_plan *p, qt_precision prec) {
    if (prec != QT_PREC_MIXED) return 0;
    uint64_t m = 0;
    for (const auto &d : p->steps[prec])
        if (gemm_eligible(d)) m = std::max<uint64_t>(m, sizeof(float) * gemm_scratch_floats(d));
    return m;
}

static void lane_main(qt_server *s, int li) {
    auto &lane = s->lanes[li];
    for (;;) {
        std::vector<Request> wave;
        {
            std::unique_lock<std::mutex> g(s->m);
            s->cv.wait(g, [&] { return s->stop || (lane.busy && !lane.wave.empty()); });
            if (s->stop && lane.wave.empty()) return;
            wave.swap(lane.wave);
        }
        std::vector<double> vals(2 * wave.size(), 0.0);
        const auto t_wave = std::chrono::steady_clock::now();
        qt_batch *b = nullptr;
        qt_status st = QT_OK;
        int nl = 0;
        if (wave.size() == 1 && wave[0].sliced) {
            const Request &r = wave[0];
            st = qt_sliced_execute_leaves(lane.ctx, r.sliced, s->prec, r.leaves.empty() ? nullptr : r.leaves.data(),
                                          vals.data());
        } else {
            st = qt_batch_create(lane.ctx, &b);
            if (st == QT_OK) {
                b->stepwise_macs = lone_instance_max_macs(s->prec);   // waves are small: big plans take the whole GPU
                // the wide interpreter takes a whole SM per instance: a wave
                // larger than its lanes' share of the SMs uses two CTAs per SM
                if ((int) wave.size() * (int) s->lanes.size() > plan_num_sms()) b->policy.kernel_ctas = 2;
            }
            for (auto &r : wave)
                if (st == QT_OK) st = qt_batch_add(b, r.plan, r.leaves.empty() ? nullptr : r.leaves.data(), nullptr);
            if (st == QT_OK) st = qt_batch_execute(b, s->prec, vals.data());
            nl = b ? qt_batch_launches_per_run(b) : 0;
            if (b) qt_batch_free(b);
        }
        const auto now = std::chrono::steady_clock::now();
        if (st == QT_ERR_OUT_OF_MEMORY && wave.size() == 1 && wave[0].heavy && wave[0].retries < kMaxOomRetries) {
            std::lock_guard<std::mutex> g(s->m);
            Request r = std::move(wave[0]);
            s->inflight--;
            s->inflight_bytes -= r.footprint;
            r.retries++;
            r.alone = true;
            s->oom_retries++;
            s->pending.push_front(std::move(r));
            s->wave_ends++;
            lane.busy = false;
            s->cv.notify_all();
            continue;
        }
        if (st != QT_OK) {
            // the lane's message goes to the server's context, where the caller reads it
            std::string msg;
            {
                std::lock_guard<std::mutex> eg(lane.ctx->err_lock);
                msg = lane.ctx->last_error;
            }
            set_error(s->ctx, st, "lane " + std::to_string(li) + ": " + msg);
        }
        {
            std::lock_guard<std::mutex> g(s->m);
            for (size_t i = 0; i < wave.size(); i++) {
                Result &res = s->results[wave[i].ticket];
                if (st == QT_OK) {
                    res.state = 1;
                    res.v[0] = vals[2 * i];
                    res.v[1] = vals[2 * i + 1];
                } else {
                    res.state = -(int) st;
                }
                res.latency = std::chrono::duration<double>(now - wave[i].t_submit).count();
                res.queued = std::chrono::duration<double>(wave[i].t_admit - wave[i].t_submit).count();
                res.lane = li;
                s->latencies.push_back(res.latency);
                s->completed++;
                s->inflight--;
                s->inflight_bytes -= wave[i].footprint;
            }
            s->launches += nl;
            s->waves++;
            s->wave_ends++;
            s->wave_requests += (int64_t) wave.size();
            s->wave_seconds += std::chrono::duration<double>(now - t_wave).count();
            lane.busy = false;
        }
        s->cv.notify_all();
        s->done_cv.notify_all();
    }
}

static void dispatcher_main(qt_server *s) {
    std::unique_lock<std::mutex> g(s->m);
    // A lane class (0: the light lane, 1: the others) whose next request could
    // not be admitted stays blocked until the next wave ends and returns its
    // memory; the other class keeps being served meanwhile (a light request
    // that arrives while the heavy lanes wait for memory is not held up).
    uint64_t blocked_at[2] = {UINT64_MAX, UINT64_MAX};
    auto lane_open = [&](int i, bool any_small, bool any_big) {
        const int cls = i > 0 ? 1 : 0;
        return !s->lanes[i].busy && (cls ? any_big : any_small) && blocked_at[cls] != s->wave_ends;
    };
    for (;;) {
        s->cv.wait(g, [&] {
            if (s->stop) return true;
            if (s->pending.empty()) return false;
            bool any_small = false, any_big = false;
            for (auto &r : s->pending) (r.small ? any_small : any_big) = true;
            for (int i = 0; i < (int) s->lanes.size(); i++)
                if (lane_open(i, any_small, any_big)) return true;
            return false;
        });
        if (s->stop) return;
        bool any_small = false, any_big = false;
        const Request *first_big = nullptr;
        for (auto &r : s->pending) {
            (r.small ? any_small : any_big) = true;
            if (!r.small && !first_big) first_big = &r;
        }
        int li = -1;
        for (int i = 0; i < (int) s->lanes.size(); i++)
            if (lane_open(i, any_small, any_big)) {
                li = i;
                break;
            }
        if (li < 0) continue;
        // admission: arrival order within a class, bounded by slots and the
        // memory budget; a heavy request at the head of the queue goes alone
        std::vector<Request> wave;
        const uint64_t budget = s->ctx->memory_budget;
        // lane 0 serves the small requests, at the highest stream priority; the
        // other lanes the rest (a heavy request alone), so that a small request
        // never runs on a low-priority stream beside a heavy one
        // lane 1 serves the pending medium requests (grouped, above the small
        // bound) before any heavy one, the other lanes take them in arrival
        // order: a medium request then rarely waits for a heavy one to finish
        bool any_medium = false;
        for (auto &r : s->pending) any_medium = any_medium || (!r.small && !r.heavy);
        const bool take_heavy = li > 0 && (li == 1 ? !any_medium : first_big->heavy);
        for (auto it = s->pending.begin(); it != s->pending.end() && s->inflight < s->max_inflight;) {
            if (it->heavy != take_heavy || (li == 0) != it->small) {
                ++it;
                continue;
            }
            if (budget && s->inflight_bytes + it->footprint > budget && s->inflight > 0) break;
            if (it->alone && s->inflight > 0) break;
            s->inflight++;
            s->inflight_bytes += it->footprint;
            it->t_admit = std::chrono::steady_clock::now();
            wave.push_back(std::move(*it));
            it = s->pending.erase(it);
            if (take_heavy) break;
        }
        if (wave.empty()) {
            // nothing admissible on this lane class until a running wave
            // returns its memory: the class waits for the next wave to end,
            // the other class does not
            blocked_at[li > 0 ? 1 : 0] = s->wave_ends;
            continue;
        }
        s->lanes[li].wave = std::move(wave);
        s->lanes[li].busy = true;
        s->cv.notify_all();
    }
}

extern "C" {

qt_status qt_server_create(qt_ctx *ctx, int max_inflight, qt_precision prec, qt_server **out) {
    if (!ctx || !out || max_inflight < 1 || (prec != QT_PREC_FP64 && prec != QT_PREC_MIXED)) return QT_ERR_INVALID_ARGUMENT;
    auto *s = new qt_server();
    s->ctx = ctx;
    ctx_retain(ctx);
    s->max_inflight = max_inflight;
    s->prec = prec;
    const int n_lanes = 4;   // lane 0: light waves only
    s->lanes.resize(n_lanes);
    for (int i = 0; i < n_lanes; i++) {
        // lane 0 (light waves) launches at the highest stream priority
        qt_status st = ctx_create_prioritised(ctx->device, i == 0, &s->lanes[i].ctx);
        if (st != QT_OK) {
            for (int j = 0; j < i; j++) qt_ctx_destroy(s->lanes[j].ctx);
            ctx_release(ctx);
            delete s;
            return st;
        }
        // the heavy lanes share the device's stream-ordered pool: their blocks
        // change size from request to request, and a pool neither keeps them
        // apart per lane nor frees them with a device-wide cudaFree (without a
        // pool they keep the caching allocator)
        cudaMemPool_t pool = nullptr;
        if (i > 0 && device_pool(ctx->device, &pool) == QT_OK) s->lanes[i].ctx->pool = pool;
    }
    // Every lane's batches: 1 MB size classes, a few blocks of each kind cached
    // from the start, so that waves never call cudaMallocHost (nor, on the
    // light lane, cudaMalloc) while other lanes run: a serving run measured
    // single cudaMallocHost calls of up to 0.37 s on the heavy lanes.  The
    // heavy lanes' device blocks come from the pool.
    for (int i = 0; i < n_lanes; i++) {
        qt_ctx *lc = s->lanes[i].ctx;
        lc->min_class = kLaneMinBlock;
        void *d[kLaneWarmBlocks] = {}, *h[kLaneWarmBlocks] = {};
        for (int k = 0; k < kLaneWarmBlocks; k++) {
            if (!lc->pool) dev_alloc(lc, kLaneMinBlock, &d[k]);
            host_alloc(lc, kLaneMinBlock, &h[k]);
        }
        for (int k = 0; k < kLaneWarmBlocks; k++) {
            dev_free(lc, d[k]);
            host_free(lc, h[k]);
        }
        ensure_pinned(lc, kLaneMinBlock);
    }
    for (int i = 0; i < n_lanes; i++) s->lanes[i].th = std::thread(lane_main, s, i);
    s->dispatcher = std::thread(dispatcher_main, s);
    *out = s;
    return QT_OK;
}

qt_status qt_server_free(qt_server *s) {
    if (!s) return QT_ERR_INVALID_ARGUMENT;
    qt_server_drain(s);
    {
        std::lock_guard<std::mutex> g(s->m);
        s->stop = true;
    }
    s->cv.notify_all();
    s->dispatcher.join();
    for (auto &l : s->lanes) l.th.join();
    for (auto &l : s->lanes) qt_ctx_destroy(l.ctx);
    ctx_release(s->ctx);
    delete s;
    return QT_OK;
}

qt_status qt_server_submit(qt_server *s, qt_plan *plan, const double *leaves, int64_t *ticket) {
    if (!s || !plan || !ticket) return QT_ERR_INVALID_ARGUMENT;
    Request r;
    r.plan = plan;
    if (leaves) r.leaves.assign(leaves, leaves + 2 * plan->leaf_values.size());
    r.t_submit = std::chrono::steady_clock::now();
    r.footprint = footprint(plan, s->prec);
    r.heavy = !plan->grouped || plan->flops > lone_instance_max_macs(s->prec);
    r.small = !r.heavy && plan->flops <= kLaneZeroMaxMacs;
    if (r.heavy) r.footprint += stepwise_scratch(plan, s->prec);
    auto refuse = [&](qt_status st, const char *why) {
        std::lock_guard<std::mutex> g(s->m);
        s->refused++;
        return set_error(s->ctx, st, why);
    };
    if (s->max_macs > 0 && plan->flops > s->max_macs) return refuse(QT_ERR_REFUSED, "request over the work cap");
    const uint64_t budget = s->ctx->memory_budget;
    if (budget && r.footprint > budget) {
        // larger than the whole budget: sliced so that one slice fits, run alone
        const uint64_t fixed = plan->leaf_bytes[s->prec] + 4096;
        if (budget <= fixed) return refuse(QT_ERR_OUT_OF_MEMORY, "request larger than the budget");
        const uint64_t target = budget - fixed;
        {
            std::lock_guard<std::mutex> g(g_slicing_lock);
            for (auto &e : plan->slicings[s->prec])
                if (e.first == target) r.sliced = e.second;
            if (!r.sliced) {
                qt_sliced *sl = nullptr;
                qt_status st = qt_plan_slice(s->ctx, plan, s->prec, target, kServerMaxCuts, &sl);
                if (st != QT_OK) {
                    std::lock_guard<std::mutex> g2(s->m);
                    s->refused++;
                    return set_error(s->ctx, st, "request larger than the budget, and no slicing fits it");
                }
                plan->slicings[s->prec].push_back({target, sl});
                r.sliced = sl;
            }
        }
        const qt_plan *sp = qt_sliced_plan(r.sliced);
        const double total = (double) sp->flops * std::ldexp(1.0, 2 * qt_sliced_num_cuts(r.sliced));
        if (s->max_macs > 0 && total > (double) s->max_macs)
            return refuse(QT_ERR_REFUSED, "sliced request over the work cap");
        r.footprint = qt_plan_workspace_bytes(sp, s->prec) + fixed + stepwise_scratch(sp, s->prec);
        r.heavy = true;
        r.small = false;
    }
    // the plan that will run (a slice of it, when sliced) must stay within the
    // step kernels' largest intermediate
    if ((r.sliced ? qt_sliced_plan(r.sliced)->peak_rank : plan->peak_rank) > kMaxStepwiseRank)
        return refuse(QT_ERR_REFUSED, "request with an intermediate above 4^15 elements");
    {
        std::lock_guard<std::mutex> g(s->m);
        r.ticket = s->next_ticket++;
        s->results[r.ticket] = Result();
        *ticket = r.ticket;
        s->pending.push_back(std::move(r));
    }
    s->cv.notify_all();
    return QT_OK;
}

int qt_server_poll(qt_server *s, int64_t ticket, double *v, double *latency) {
    if (!s) return -(int) QT_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->m);
    auto it = s->results.find(ticket);
    if (it == s->results.end()) return -(int) QT_ERR_INVALID_ARGUMENT;
    if (it->second.state == 1) {
        if (v) {
            v[0] = it->second.v[0];
            v[1] = it->second.v[1];
        }
        if (latency) *latency = it->second.latency;
    }
    return it->second.state;
}

int qt_server_poll_detail(qt_server *s, int64_t ticket, double *v, double *latency, double *queued, int *lane) {
    const int st = qt_server_poll(s, ticket, v, latency);
    if (st != 1) return st;
    std::lock_guard<std::mutex> g(s->m);
    const Result &r = s->results.at(ticket);
    if (queued) *queued = r.queued;
    if (lane) *lane = r.lane;
    return st;
}

qt_status qt_server_drain(qt_server *s) {
    if (!s) return QT_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> g(s->m);
    s->done_cv.wait(g, [&] { return s->pending.empty() && s->inflight == 0; });
    return QT_OK;
}

qt_status qt_server_wave_stats(qt_server *s, int64_t *waves, int64_t *requests, double *lane_seconds) {
    if (!s) return QT_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->m);
    if (waves) *waves = s->waves;
    if (requests) *requests = s->wave_requests;
    if (lane_seconds) *lane_seconds = s->wave_seconds;
    return QT_OK;
}

qt_status qt_server_set_max_macs(qt_server *s, int64_t max_macs) {
    if (!s || max_macs < 0) return QT_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->m);
    s->max_macs = max_macs;
    return QT_OK;
}

int64_t qt_server_refused(qt_server *s) {
    if (!s) return -1;
    std::lock_guard<std::mutex> g(s->m);
    return s->refused;
}

int64_t qt_server_oom_retries(qt_server *s) {
    if (!s) return -1;
    std::lock_guard<std::mutex> g(s->m);
    return s->oom_retries;
}

qt_status qt_server_stats(qt_server *s, double *p50, double *p99, int64_t *completed, int64_t *launches) {
    if (!s) return QT_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->m);
    std::vector<double> l = s->latencies;
    std::sort(l.begin(), l.end());
    auto q = [&](double f) {
        if (l.empty()) return 0.0;
        size_t i = (size_t) std::min<double>((double) l.size() - 1, std::ceil(f * (double) l.size()) - 1);
        return l[i];
    };
    if (p50) *p50 = q(0.50);
    if (p99) *p99 = q(0.99);
    if (completed) *completed = s->completed;
    if (launches) *launches = s->launches;
    return QT_OK;
}

}  // extern "C"
