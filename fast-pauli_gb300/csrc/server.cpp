// server.cpp -- device-resident request loop with continuous admission.
//
// A serving front end for the two request kinds of the hot path:
// SummedPauliOp::expectation_value (reference __summed_pauli_op.hpp:520-614)
// and SummedPauliOp::apply_weighted (__summed_pauli_op.hpp:365-503).  The
// reference has no server; this is the request loop around the engine.
//
//  * Operators (fpg_operator) and request arrays stay resident on the device;
//    a request carries device pointers only.
//  * Admission: a request is admitted when a slot (one CUDA stream each) is
//    free and its scratch bytes fit the remaining HBM budget; otherwise it
//    waits in the queue.  The scheduler scans the queue in arrival order and
//    admits every request that fits (smaller ones may pass a large one that
//    does not fit yet).  A request larger than the whole budget is refused at
//    submission (FPG_ERR_BUSY).
//  * Priorities: requests fall in three classes by work (amplitude-terms
//    n_strings * 2^n * n_states): small (<= kSmallWork, milliseconds), medium
//    (<= kMediumWork, up to ~0.2 s) and large.  The slots are split into
//    three tiers of streams at the device's highest, middle and lowest
//    priority; a request takes a free slot of its own tier, else of a lower
//    tier, never of a higher one.  The block scheduler starts the CTAs of
//    higher-priority streams first as SMs free up, so short requests are not
//    stuck behind long ones and medium ones not behind the largest.
//  * Continuous: the scheduler thread admits new requests the moment slots
//    and memory free up, while earlier requests are still running; admitted
//    requests run concurrently on their slots' streams, so their kernels
//    overlap on the device.
//  * Batching: small expectation requests (the small class above) always run
//    through the merged path (run_merged_expect, batch.cu): every such
//    request admitted in one scheduling round -- those that arrived while
//    the GPU was busy, up to kMaxMerge -- shares one launch sequence (one
//    work-queue kernel per chunk class, one reduction, one contraction) on
//    one slot, instead of a stream and ~10 launches each.  A request alone
//    runs the same path as a merge of one.
//  * Each request runs the same deterministic kernels it would run alone
//    (the merged path's per-request results do not depend on the other
//    requests of the merge), so its result does not depend on the mix
//    (tests check this).
//  * Outputs are overwritten (zeroed, then computed).
//  * Latency per ticket: submit -> admission -> completion (host steady
//    clock, completion observed through a CUDA event).
#include <algorithm>
#include <cmath>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "fpg.h"

#include "host_internal.hpp"

using namespace fpg;

namespace
{

using clock_type = std::chrono::steady_clock;

double us_since(clock_type::time_point t0, clock_type::time_point t)
{
    return std::chrono::duration<double, std::micro>(t - t0).count();
}

struct Ticket
{
    fpg_request req{};
    size_t need = 0;
    int status = 0; // 0 queued, 1 running, 2 done, 3 failed
    int rc = FPG_OK;
    std::string err;
    clock_type::time_point t_submit, t_start, t_done;
    int slot = -1;
    int tier = 2;       // 0 small, 1 medium, 2 large
    bool merge = false; // small expectation request: the merged path
};

// Most small expectation requests one merged launch sequence takes.
constexpr int kMaxMerge = 64;

// Work classes in amplitude-terms (n_strings * 2^n * n_states): small is a
// few milliseconds of GPU time, medium up to ~0.2 s.
constexpr double kSmallWork = 4.0e9;
constexpr double kMediumWork = 2.0e11;

int work_tier(double work)
{
    return work <= kSmallWork ? 0 : (work <= kMediumWork ? 1 : 2);
}

} // namespace

struct fpg_server
{
    fpg_server_config cfg{};
    int device = 0;
    clock_type::time_point t0 = clock_type::now();
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<uint64_t> queue;
    std::unordered_map<uint64_t, Ticket> tickets;
    struct Slot
    {
        cudaStream_t stream = nullptr;
        cudaEvent_t event = nullptr;
        std::vector<uint64_t> tickets; // one request, or the requests of a merged run
        bool busy = false;
        int tier = 2; // 0: the device's highest stream priority, 1: middle, 2: lowest
    };
    std::vector<Slot> slots;
    size_t reserved = 0;
    uint64_t next_ticket = 1;
    bool stop = false;
    std::thread worker;
    // counters
    uint64_t completed = 0, failed = 0, refused = 0;
    uint64_t merged_runs = 0, merged_requests = 0;
    size_t peak_reserved = 0;
    int peak_running = 0;

    void run();
    int dispatch(Slot &s, Ticket &t);
    int dispatch_merged(Slot &s, const std::vector<uint64_t> &ids);
    std::vector<Slot>::iterator free_slot_for(int tier);
};

std::vector<fpg_server::Slot>::iterator fpg_server::free_slot_for(int tier)
{
    // a free slot of the request's tier, else of a lower-priority tier:
    // higher tiers stay free for the shorter requests
    auto it = slots.end();
    for (int tr = tier; tr <= 2 && it == slots.end(); ++tr)
        it = std::find_if(slots.begin(), slots.end(), [tr](const Slot &s) { return !s.busy && s.tier == tr; });
    return it;
}

int fpg_server::dispatch_merged(Slot &s, const std::vector<uint64_t> &ids)
{
    std::vector<MergedExpect> probs;
    probs.reserve(ids.size());
    for (uint64_t id : ids)
    {
        const fpg_request &r = tickets[id].req;
        probs.push_back(MergedExpect{r.op, r.coeffs, r.n_operators, r.states, r.out, r.n_states});
    }
    if (int rc = run_merged_expect(cfg.dtype, probs.data(), (int)probs.size(), s.stream))
        return rc;
    if (cudaError_t e = cudaEventRecord(s.event, s.stream))
        return cuda_error(e, "cudaEventRecord");
    return FPG_OK;
}

int fpg_server::dispatch(Slot &s, Ticket &t)
{
    const fpg_request &r = t.req;
    const size_t csz = cfg.dtype == FPG_C64 ? 8 : 16;
    cudaError_t e;
    int rc;
    if (r.kind == FPG_REQ_EXPECT)
    {
        if ((e = cudaMemsetAsync(r.out, 0, (size_t)r.n_operators * (size_t)r.n_states * csz, s.stream)))
            return cuda_error(e, "cudaMemsetAsync");
        rc = fpg_summed_expect(r.op, r.coeffs, r.n_operators, r.states, r.out, r.n_states, cfg.dtype, s.stream);
    }
    else
    {
        int32_t n = 0;
        fpg_operator_info(r.op, &n, nullptr, nullptr);
        if ((e = cudaMemsetAsync(r.out, 0, ((size_t)1 << n) * (size_t)r.n_states * csz, s.stream)))
            return cuda_error(e, "cudaMemsetAsync");
        rc = fpg_summed_apply_weighted(r.op, r.coeffs, r.n_operators, r.states, r.data, r.out, r.n_states,
                                       cfg.dtype, s.stream);
    }
    if (rc != FPG_OK)
        return rc;
    if ((e = cudaEventRecord(s.event, s.stream)))
        return cuda_error(e, "cudaEventRecord");
    return FPG_OK;
}

void fpg_server::run()
{
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    while (true)
    {
        // 1. retire finished slots
        bool progressed = false;
        int running = 0;
        for (Slot &s : slots)
        {
            if (!s.busy)
                continue;
            const cudaError_t q = cudaEventQuery(s.event);
            if (q == cudaErrorNotReady)
            {
                ++running;
                continue;
            }
            const auto now = clock_type::now();
            for (uint64_t id : s.tickets)
            {
                Ticket &t = tickets[id];
                t.t_done = now;
                if (q == cudaSuccess)
                {
                    t.status = 2;
                    ++completed;
                }
                else
                {
                    t.status = 3;
                    t.rc = FPG_ERR_CUDA;
                    t.err = cudaGetErrorString(q);
                    ++failed;
                }
                reserved -= t.need;
            }
            s.tickets.clear();
            s.busy = false;
            progressed = true;
        }
        if (progressed)
            cv_done.notify_all();
        // 2. admit queued requests into free slots while the budget allows;
        // small expectation requests admitted in this pass of the loop go to
        // one merged run on one slot
        auto merge_slot = slots.end();
        std::vector<uint64_t> merge_ids;
        for (auto it = queue.begin(); it != queue.end();)
        {
            Ticket &t = tickets[*it];
            if (reserved + t.need > (size_t)cfg.hbm_budget_bytes)
            {
                ++it; // does not fit yet: let later, smaller requests pass
                continue;
            }
            if (t.merge)
            {
                if (merge_slot == slots.end())
                    merge_slot = free_slot_for(t.tier);
                if (merge_slot == slots.end() || (int)merge_ids.size() >= kMaxMerge)
                {
                    ++it;
                    continue;
                }
                merge_slot->busy = true; // held for the merged run dispatched below
                reserved += t.need;
                peak_reserved = std::max(peak_reserved, reserved);
                t.status = 1;
                t.t_start = clock_type::now();
                t.slot = (int)(merge_slot - slots.begin());
                merge_ids.push_back(*it);
                it = queue.erase(it);
                progressed = true;
                continue;
            }
            auto free_slot = free_slot_for(t.tier);
            if (free_slot == slots.end())
            {
                ++it; // no slot of its class: later requests of the other class may pass
                continue;
            }
            reserved += t.need;
            peak_reserved = std::max(peak_reserved, reserved);
            t.status = 1;
            t.t_start = clock_type::now();
            t.slot = (int)(free_slot - slots.begin());
            const int rc = dispatch(*free_slot, t);
            if (rc != FPG_OK)
            {
                t.status = 3;
                t.rc = rc;
                t.err = fpg_last_error();
                t.t_done = clock_type::now();
                reserved -= t.need;
                ++failed;
                cv_done.notify_all();
            }
            else
            {
                free_slot->busy = true;
                free_slot->tickets.assign(1, *it);
                ++running;
            }
            it = queue.erase(it);
            progressed = true;
        }
        if (!merge_ids.empty())
        {
            const int rc = dispatch_merged(*merge_slot, merge_ids);
            if (rc != FPG_OK)
            {
                const std::string err = fpg_last_error();
                for (uint64_t id : merge_ids)
                {
                    Ticket &t = tickets[id];
                    t.status = 3;
                    t.rc = rc;
                    t.err = err;
                    t.t_done = clock_type::now();
                    reserved -= t.need;
                    ++failed;
                }
                merge_slot->busy = false;
                cv_done.notify_all();
            }
            else
            {
                merge_slot->tickets = merge_ids;
                ++merged_runs;
                merged_requests += merge_ids.size();
                ++running;
            }
        }
        peak_running = std::max(peak_running, running);
        if (stop && queue.empty() && running == 0)
            break;
        if (!progressed)
        {
            // nothing changed: sleep briefly (work arrives via cv_work)
            if (running > 0)
                cv_work.wait_for(lk, std::chrono::microseconds(20));
            else
                cv_work.wait_for(lk, std::chrono::milliseconds(5));
        }
    }
}

extern "C"
{

    int fpg_server_create(const fpg_server_config *config, fpg_server **out)
    {
        if (!config || !out)
            return set_error(FPG_ERR_INVALID, "null argument");
        *out = nullptr;
        if (config->dtype != FPG_C128 && config->dtype != FPG_C64)
            return set_error(FPG_ERR_INVALID, "dtype must be FPG_C128 or FPG_C64");
        if (config->n_slots < 1 || config->n_slots > 64)
            return set_error(FPG_ERR_INVALID, "n_slots must be in [1, 64]");
        if (config->hbm_budget_bytes <= 0)
            return set_error(FPG_ERR_INVALID, "hbm_budget_bytes must be > 0");
        fpg_server *s = new (std::nothrow) fpg_server();
        if (!s)
            return set_error(FPG_ERR_NOMEM, "host allocation failed");
        s->cfg = *config;
        if (s->cfg.max_queue <= 0)
            s->cfg.max_queue = 1 << 20;
        cudaError_t e = cudaGetDevice(&s->device);
        s->slots.resize((size_t)config->n_slots);
        // tiers: a third of the slots each for medium and large requests (at
        // least one large slot), the rest for small ones; a single slot is a
        // large-tier slot, which every request may take.  Stream priorities:
        // highest / middle / lowest of the device's range
        int prio_low = 0, prio_high = 0;
        if (e == cudaSuccess)
            e = cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
        const int n = config->n_slots;
        const int n_large = n > 1 ? std::max(1, n / 3) : 1;
        const int n_medium = n > 2 ? std::max(1, n / 3) : 0;
        const int n_small = n - n_large - n_medium;
        const int prio_of[3] = {prio_high, (prio_high + prio_low) / 2, prio_low};
        for (size_t i = 0; i < s->slots.size(); ++i)
        {
            auto &sl = s->slots[i];
            sl.tier = (int)i < n_small ? 0 : ((int)i < n_small + n_medium ? 1 : 2);
            if (e == cudaSuccess)
                e = cudaStreamCreateWithPriority(&sl.stream, cudaStreamNonBlocking, prio_of[sl.tier]);
            if (e == cudaSuccess)
                e = cudaEventCreateWithFlags(&sl.event, cudaEventDisableTiming);
        }
        if (e != cudaSuccess)
        {
            for (auto &sl : s->slots)
            {
                if (sl.event)
                    cudaEventDestroy(sl.event);
                if (sl.stream)
                    cudaStreamDestroy(sl.stream);
            }
            delete s;
            return cuda_error(e, "fpg_server_create");
        }
        s->worker = std::thread([s] { s->run(); });
        *out = s;
        return FPG_OK;
    }

    int fpg_server_submit(fpg_server *s, const fpg_request *req, uint64_t *ticket)
    {
        if (!s || !req || !ticket)
            return set_error(FPG_ERR_INVALID, "null argument");
        if (req->kind != FPG_REQ_EXPECT && req->kind != FPG_REQ_APPLY_WEIGHTED)
            return set_error(FPG_ERR_INVALID, "unknown request kind");
        if (!req->op || !req->coeffs || !req->states || !req->out ||
            (req->kind == FPG_REQ_APPLY_WEIGHTED && !req->data))
            return set_error(FPG_ERR_INVALID, "null array in request");
        if (req->n_operators < 1 || req->n_states < 1)
            return set_error(FPG_ERR_INVALID, "n_operators and n_states must be >= 1");
        int32_t nq = 0;
        int64_t ps = 0;
        fpg_operator_info(req->op, &nq, &ps, nullptr);
        const int tier = work_tier((double)ps * std::ldexp(1.0, nq) * (double)req->n_states);
        const bool merge = req->kind == FPG_REQ_EXPECT && tier == 0;
        const size_t need =
            merge ? merged_expect_scratch_bytes(req->op, req->n_states, req->states, s->cfg.dtype == FPG_C64)
                  : request_scratch_bytes(req->op, req->n_operators, req->n_states, s->cfg.dtype == FPG_C64,
                                          req->kind == FPG_REQ_APPLY_WEIGHTED);
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop)
            return set_error(FPG_ERR_INVALID, "server is shutting down");
        if (need > (size_t)s->cfg.hbm_budget_bytes)
        {
            ++s->refused;
            return set_error(FPG_ERR_BUSY, "request needs " + std::to_string(need) +
                                               " scratch bytes, more than the whole HBM budget");
        }
        if ((int64_t)s->queue.size() >= s->cfg.max_queue)
        {
            ++s->refused;
            return set_error(FPG_ERR_BUSY, "request queue is full");
        }
        const uint64_t id = s->next_ticket++;
        Ticket t;
        t.req = *req;
        t.need = need;
        t.tier = tier;
        t.merge = merge;
        t.t_submit = clock_type::now();
        s->tickets.emplace(id, std::move(t));
        s->queue.push_back(id);
        *ticket = id;
        s->cv_work.notify_one();
        return FPG_OK;
    }

    int fpg_server_wait(fpg_server *s, uint64_t ticket, int32_t timeout_ms, fpg_ticket_info *info)
    {
        if (!s)
            return set_error(FPG_ERR_INVALID, "server is null");
        std::unique_lock<std::mutex> lk(s->mu);
        auto it = s->tickets.find(ticket);
        if (it == s->tickets.end())
            return set_error(FPG_ERR_INVALID, "unknown ticket");
        const auto deadline = clock_type::now() + std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms);
        while (it->second.status < 2)
        {
            if (timeout_ms >= 0 && s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout &&
                it->second.status < 2)
                return set_error(FPG_ERR_TIMEOUT, "ticket not finished within the timeout");
            if (timeout_ms < 0)
                s->cv_done.wait(lk);
        }
        const Ticket &t = it->second;
        if (info)
        {
            info->status = t.status;
            info->submit_us = us_since(s->t0, t.t_submit);
            info->start_us = us_since(s->t0, t.t_start);
            info->done_us = us_since(s->t0, t.t_done);
            info->scratch_bytes = (int64_t)t.need;
        }
        if (t.status == 3)
            return set_error(t.rc, t.err);
        return FPG_OK;
    }

    int fpg_server_release(fpg_server *s, uint64_t ticket)
    {
        if (!s)
            return set_error(FPG_ERR_INVALID, "server is null");
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->tickets.find(ticket);
        if (it == s->tickets.end())
            return set_error(FPG_ERR_INVALID, "unknown ticket");
        if (it->second.status < 2)
            return set_error(FPG_ERR_INVALID, "ticket still in flight");
        s->tickets.erase(it);
        return FPG_OK;
    }

    int fpg_server_stats(fpg_server *s, fpg_server_stats_t *st)
    {
        if (!s || !st)
            return set_error(FPG_ERR_INVALID, "null argument");
        std::lock_guard<std::mutex> lk(s->mu);
        st->completed = (int64_t)s->completed;
        st->failed = (int64_t)s->failed;
        st->refused = (int64_t)s->refused;
        st->queued = (int64_t)s->queue.size();
        st->peak_running = s->peak_running;
        st->peak_reserved_bytes = (int64_t)s->peak_reserved;
        st->merged_runs = (int64_t)s->merged_runs;
        st->merged_requests = (int64_t)s->merged_requests;
        return FPG_OK;
    }

    int fpg_server_destroy(fpg_server *s)
    {
        if (!s)
            return FPG_OK;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stop = true;
        }
        s->cv_work.notify_all();
        if (s->worker.joinable())
            s->worker.join();
        for (auto &sl : s->slots)
        {
            cudaEventDestroy(sl.event);
            cudaStreamDestroy(sl.stream);
        }
        delete s;
        return FPG_OK;
    }

} // extern "C"
