// serve.cu -- continuous-batching query server over a resident HIBF, and an open-loop load driver.
//
// The server keeps the HIBF on the device and owns `slots` agents, each with its own stream and buffers.  Requests
// (CSR batches of queries from callers) wait in a FIFO.  Each slot has its own thread: whenever it is free it
// coalesces waiting requests, oldest first, into one batch bounded by the slot's capacity and by the device-memory
// admission cap (inputs, task queue, records and result lists of all batches in flight), stages and launches it,
// waits for it and splits the results.  Batches on different slots overlap on the device and their host work runs
// in parallel; a request that arrives while others run joins the next batch a free slot takes.
// Results are split back per request; a batch's results equal each request's results alone because queries are
// independent.  A request that alone needs more than the admission cap is rejected (HIBF_GPU_ERR_ADMISSION).
//
// Reference: the reference has no server; its agents answer one query per call (hierarchical_interleaved_bloom_filter
// .hpp:322-439).  This is the serving loop the batched device path enables.

#include <algorithm>
#include <atomic>
#include <chrono>
#include <array>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <random>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/hibf_gb300_synthetic.h"
#include "common.hpp"

namespace hibf_gb300
{
namespace serve
{

using clock_t_ = std::chrono::steady_clock;

inline double now_s()
{
    return std::chrono::duration<double>(clock_t_::now().time_since_epoch()).count();
}

struct request
{
    uint64_t id{};
    uint64_t nq{}, nv{};
    uint64_t const * values{}; // the request's values, offsets (relative, qoff[0] = 0) and thresholds: either the
    uint64_t const * qoff{};   // caller's buffers (kept alive by the caller until the request is released) or the
    uint64_t const * thr{};    // copies below
    std::vector<uint64_t> own_values, own_qoff, own_thr;
    double t_arrival{};                      // when the request counts as arrived (caller's clock, seconds)
    double t_done{};
    int status{HIBF_GPU_OK};
    std::atomic<bool> done{false}; // set by a slot thread after the results, read by waiters
    bool solo{false};   // run alone (after a batch overflowed)
    bool pinned{false}; // values are in page-locked host memory: copied to the device directly, not staged
    uint64_t const * dev_values{}; // the device's address of `values` when its registered range is mapped, else null
    std::vector<uint64_t> res_off, res_ids;
};

struct slot
{
    hibf_gpu_agent * agent{};
    cudaStream_t stream{};
    cudaEvent_t ev{};
    cudaEvent_t ev_in{}, ev_q{}; // timing: before the batch's input copies, before its launch
    std::vector<request *> reqs;
    uint64_t nq{}, nv{}, bytes{};
    dbuf d_values, d_qoff, d_thr;
    hbuf h_values, h_qoff, h_thr, h_roff, h_ids;
    uint64_t const * d_roff{};
    uint64_t const * d_ids{};
};

} // namespace serve
} // namespace hibf_gb300

using namespace hibf_gb300;
using namespace hibf_gb300::serve;

struct hibf_gpu_server
{
    hibf_gpu_hibf * h{};
    uint64_t max_queries{}, max_values{}, admission_bytes{};
    std::vector<std::unique_ptr<slot>> slots;
    std::deque<request *> waiting;
    std::unordered_map<uint64_t, std::unique_ptr<request>> reqs;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::vector<std::thread> workers; // one per slot
    std::atomic<bool> stop{false};
    uint64_t inflight_bytes{};
    uint64_t next_id{1};
    int device{};
    std::string loop_error;
    // counters
    uint64_t batches{}, batched_queries{}, rejected{};
    // summed seconds per batch phase: queueing of the batch's oldest request, staging + launch, until the batch's
    // device work is done, result fetch, per-request split
    double t_queue{}, t_stage{}, t_device{}, t_fetch{}, t_split{};
    // per batch (the first kBatchLogCap): oldest request's arrival, slot start, launched, device done, results
    // fetched, requests finished (seconds, now_s clock), queries, values, device time of its input copies and of
    // its query kernel (seconds, CUDA events)
    static constexpr size_t kBatchLogCap = 1u << 20;
    static constexpr int kBatchLogCols = 12;
    std::vector<std::array<double, kBatchLogCols>> batch_log;
    // page-locked host ranges [begin, end) registered with the server, and whether the server pinned them
    struct host_range
    {
        uintptr_t begin, end;
        bool pinned_here;
        uint64_t const * dev; // the device's address of `begin` (mapped page-locked memory), else null
    };
    std::vector<host_range> host_ranges;
    // a batch whose requests lie back to back in one mapped registered range is read in place by the kernel
    std::atomic<bool> zero_copy{true};
    // the last open-loop run's load generator: the largest and the 99.9th-percentile lateness of a submission behind
    // its scheduled arrival, the submissions more than 1 ms late, and p99 / p99.9 latency from the actual submission
    double open_loop_detail[5]{};
};

namespace
{

// Device bytes a batch needs: inputs, task queue, records and result lists (the agent's workspace for it).
uint64_t batch_bytes(uint64_t nq, uint64_t nv)
{
    return nv * 8 + (nq + 1) * 8 + nq * 8 + nq * 8 * 8 + nq * 16 * (4 + 4 + 8 + 8 + 8 + 8);
}

void finish(request * r, int status, double t)
{
    r->status = status;
    r->t_done = t;
    r->done.store(true);
}

// Moves the oldest waiting requests that fit into one batch of `sl` (slot capacity, admission cap; a request rerun
// alone after an overflow runs by itself).  Requests that cannot run even alone are rejected.  Caller holds S->mu.
void take_batch(hibf_gpu_server * S, slot & sl)
{
    uint64_t nq = 0, nv = 0;
    while (!S->waiting.empty())
    {
        request * r = S->waiting.front();
        uint64_t const b = batch_bytes(nq + r->nq, nv + r->nv);
        bool const fits_slot = nq + r->nq <= S->max_queries && nv + r->nv <= S->max_values;
        bool const fits_cap = S->inflight_bytes + b <= S->admission_bytes;
        bool const alone_ok = batch_bytes(r->nq, r->nv) <= S->admission_bytes;
        if (sl.reqs.empty() && (!(r->nq <= S->max_queries && r->nv <= S->max_values) || !alone_ok))
        {
            S->waiting.pop_front(); // cannot run even alone in a slot
            finish(r, HIBF_GPU_ERR_ADMISSION, now_s());
            ++S->rejected;
            S->cv_done.notify_all();
            continue;
        }
        if (!fits_slot || !fits_cap || (r->solo && !sl.reqs.empty()))
            break;
        S->waiting.pop_front();
        sl.reqs.push_back(r);
        nq += r->nq;
        nv += r->nv;
        if (r->solo)
            break;
    }
    sl.nq = nq;
    sl.nv = nv;
    sl.bytes = sl.reqs.empty() ? 0 : batch_bytes(nq, nv);
    S->inflight_bytes += sl.bytes;
}

// Stages the slot's requests into pinned memory, copies them to the device and launches the batch; then waits for
// it, fetches the result offsets and ids, and splits them per request.  Runs on the slot's own thread, so batches of
// different slots stage, run and finish concurrently.  Returns the requests to rerun alone (after an overflow).
std::vector<request *> run_batch(hibf_gpu_server * S, slot & sl)
{
    uint64_t const nq = sl.nq, nv = sl.nv;
    double const t_start = now_s();
    double t_oldest = t_start;
    for (request * r : sl.reqs)
        t_oldest = std::min(t_oldest, r->t_arrival);
    uint64_t * hv = sl.h_values.as<uint64_t>();
    uint64_t * ho = sl.h_qoff.as<uint64_t>();
    uint64_t * ht = sl.h_thr.as<uint64_t>();
    uint64_t q = 0, v = 0;
    ho[0] = 0;
    HG_CUDA(cudaEventRecord(sl.ev_in, sl.stream));
    uint64_t staged_from = 0; // start of the current run of staged requests
    uint64_t staged_values = 0; // values copied through the slot's pinned buffer (requests outside registered ranges)
    // Zero copy: when the batch's requests lie back to back in one mapped page-locked range, the kernel reads their
    // values there (over the host link, as it needs them) and no copy precedes the launch.  The batch's offsets are
    // the same as for a compacted copy, relative to its first request's values.
    bool zc = S->zero_copy.load() && !sl.reqs.empty();
    for (size_t k = 0; zc && k < sl.reqs.size(); ++k)
    {
        request const * r = sl.reqs[k];
        zc = r->pinned && r->dev_values &&
             (k == 0 || (r->values == sl.reqs[k - 1]->values + sl.reqs[k - 1]->nv &&
                         r->dev_values == sl.reqs[k - 1]->dev_values + sl.reqs[k - 1]->nv));
    }
    uint64_t const * const batch_values = zc ? sl.reqs.front()->dev_values : sl.d_values.as<uint64_t>();
    auto flush_staged = [&](uint64_t to)
    {
        if (to > staged_from)
            HG_CUDA(cudaMemcpyAsync(sl.d_values.as<uint64_t>() + staged_from, hv + staged_from,
                                    (to - staged_from) * 8, cudaMemcpyHostToDevice, sl.stream));
    };
    for (request * r : sl.reqs)
    {
        if (!r->pinned)
        {
            staged_values += r->nv;
            std::memcpy(hv + v, r->values, r->nv * 8);
        }
        else if (!zc)
        {
            // page-locked caller memory: one DMA straight into the batch's input, no host copy
            flush_staged(v);
            if (r->nv)
                HG_CUDA(cudaMemcpyAsync(sl.d_values.as<uint64_t>() + v, r->values, r->nv * 8, cudaMemcpyHostToDevice,
                                        sl.stream));
            staged_from = v + r->nv;
        }
        for (uint64_t i = 0; i < r->nq; ++i)
        {
            ho[q + i + 1] = v + r->qoff[i + 1];
            ht[q + i] = r->thr[i];
        }
        q += r->nq;
        v += r->nv;
    }
    if (!zc)
        flush_staged(v);
    HG_CUDA(cudaMemcpyAsync(sl.d_qoff.p, ho, (nq + 1) * 8, cudaMemcpyHostToDevice, sl.stream));
    HG_CUDA(cudaMemcpyAsync(sl.d_thr.p, ht, std::max<uint64_t>(nq, 1) * 8, cudaMemcpyHostToDevice, sl.stream));
    void const * cnt = nullptr;
    HG_CUDA(cudaEventRecord(sl.ev_q, sl.stream));
    int st = hibf_gpu_agent_query_batch_d(sl.agent, HIBF_GPU_QUERY_MEMBERSHIP, batch_values,
                                          sl.d_qoff.as<uint64_t>(), nq, sl.d_thr.as<uint64_t>(), 2, &sl.d_roff,
                                          &sl.d_ids, &cnt);
    if (st != HIBF_GPU_OK)
        fail(st, "batch launch failed");
    HG_CUDA(cudaMemcpyAsync(sl.h_roff.p, sl.d_roff, (nq + 1) * 8, cudaMemcpyDeviceToHost, sl.stream));
    double const t_launched = now_s();
    std::vector<request *> requeue;
    st = hibf_gpu_agent_status(sl.agent); // synchronises the slot's stream
    double const t_device_done = now_s();
    if (st == HIBF_GPU_ERR_OVERFLOW)
    {
        // rerun every request alone; a request that overflows alone fails
        double const t = now_s();
        for (request * r : sl.reqs)
        {
            if (sl.reqs.size() == 1 || r->solo)
                finish(r, HIBF_GPU_ERR_OVERFLOW, t);
            else
            {
                r->solo = true;
                requeue.push_back(r);
            }
        }
        return requeue;
    }
    if (st != HIBF_GPU_OK)
    {
        double const t = now_s();
        for (request * r : sl.reqs)
            finish(r, st, t);
        return requeue;
    }
    uint64_t const * ro = sl.h_roff.as<uint64_t>();
    uint64_t const nr = ro[nq];
    if (nr)
    {
        HG_CUDA(cudaMemcpyAsync(sl.h_ids.p, sl.d_ids, nr * 8, cudaMemcpyDeviceToHost, sl.stream));
        HG_CUDA(cudaStreamSynchronize(sl.stream));
    }
    uint64_t const * ids = sl.h_ids.as<uint64_t>();
    double const t_fetched = now_s();
    q = 0;
    for (request * r : sl.reqs)
    {
        uint64_t const base = ro[q];
        r->res_off.resize(r->nq + 1);
        for (uint64_t i = 0; i <= r->nq; ++i)
            r->res_off[i] = ro[q + i] - base;
        r->res_ids.assign(ids + base, ids + ro[q + r->nq]);
        q += r->nq;
    }
    double const t = now_s();
    for (request * r : sl.reqs)
        finish(r, HIBF_GPU_OK, t);
    float copy_ms = 0, kernel_ms = 0;
    if (cudaEventElapsedTime(&copy_ms, sl.ev_in, sl.ev_q) != cudaSuccess ||
        hibf_gpu_agent_kernel_ms(sl.agent, &kernel_ms) != HIBF_GPU_OK)
        (void)cudaGetLastError();
    std::lock_guard<std::mutex> lk(S->mu);
    ++S->batches;
    S->batched_queries += nq;
    S->t_queue += std::max(0.0, t_start - t_oldest);
    S->t_stage += t_launched - t_start;
    S->t_device += t_device_done - t_launched;
    S->t_fetch += t_fetched - t_device_done;
    S->t_split += t - t_fetched;
    if (S->batch_log.size() < hibf_gpu_server::kBatchLogCap)
        S->batch_log.push_back({t_oldest, t_start, t_launched, t_device_done, t_fetched, t, static_cast<double>(nq),
                                static_cast<double>(sl.nv), copy_ms * 1e-3, kernel_ms * 1e-3,
                                static_cast<double>(staged_values), zc ? 1.0 : 0.0});
    return requeue;
}

// One thread per slot: take the oldest waiting requests that fit, run them as one batch, complete them, repeat.
void slot_loop(hibf_gpu_server * S, slot * sl)
{
    cudaSetDevice(S->device);
    while (true)
    {
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv_work.wait(lk, [&] { return S->stop.load() || !S->waiting.empty(); });
            if (S->stop.load())
                return;
            take_batch(S, *sl);
            if (sl->reqs.empty())
            {
                // the admission cap is taken by batches in flight: wait for one to finish
                S->cv_work.wait_for(lk, std::chrono::microseconds(200));
                continue;
            }
        }
        std::vector<request *> requeue;
        try
        {
            requeue = run_batch(S, *sl);
        }
        catch (status_error const & err)
        {
            double const t = now_s();
            std::lock_guard<std::mutex> lk(S->mu);
            S->loop_error = err.what();
            for (request * r : sl->reqs)
                if (!r->done.load())
                    finish(r, err.status, t);
        }
        std::lock_guard<std::mutex> lk(S->mu);
        S->inflight_bytes -= sl->bytes;
        for (auto it = requeue.rbegin(); it != requeue.rend(); ++it)
            S->waiting.push_front(*it);
        sl->reqs.clear();
        S->cv_done.notify_all();
        S->cv_work.notify_all();
    }
}

// The device's first read of a page-locked host page is several times slower than later ones (4-25 MB copies:
// 20-40 GB/s the first time, 130-190 GB/s after, on a host with 64 KB pages), and pages read long ago turn slow again
// after gigabytes of other transfers.  A registered range is read once, in 64 MB pieces into scratch, so that the
// requests borrowed from it start with warm pages.
void warm_host_range(void const * ptr, uint64_t bytes)
{
    uint64_t const piece = std::min<uint64_t>(bytes, 64ull << 20);
    dbuf scratch;
    scratch.ensure(piece);
    cudaStream_t st{};
    HG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    struct stream_guard
    {
        cudaStream_t s;
        ~stream_guard()
        {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    } guard{st};
    char const * const b = static_cast<char const *>(ptr);
    for (uint64_t o = 0; o < bytes; o += piece)
        HG_CUDA(cudaMemcpyAsync(scratch.p, b + o, std::min(piece, bytes - o), cudaMemcpyHostToDevice, st));
    HG_CUDA(cudaStreamSynchronize(st));
}
} // namespace

extern "C"
{

    int hibf_gpu_server_create(hibf_gpu_hibf * h, int n_slots, uint64_t max_batch_queries, uint64_t max_batch_values,
                               uint64_t admission_bytes, hibf_gpu_server ** out)
    {
        return guarded(
            [&]
            {
                if (!h || !out || n_slots <= 0 || max_batch_queries == 0 || max_batch_values == 0)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "bad argument");
                *out = nullptr;
                auto S = std::make_unique<hibf_gpu_server>();
                S->h = h;
                S->max_queries = max_batch_queries;
                S->max_values = max_batch_values;
                S->admission_bytes = admission_bytes;
                HG_CUDA(cudaGetDevice(&S->device));
                for (int i = 0; i < n_slots; ++i)
                {
                    auto sl = std::make_unique<slot>();
                    int st = hibf_gpu_agent_create(h, &sl->agent);
                    if (st != HIBF_GPU_OK)
                        fail(st, "agent creation failed");
                    HG_CUDA(cudaStreamCreateWithFlags(&sl->stream, cudaStreamNonBlocking));
                    HG_CUDA(cudaEventCreateWithFlags(&sl->ev, cudaEventDisableTiming));
                    HG_CUDA(cudaEventCreate(&sl->ev_in));
                    HG_CUDA(cudaEventCreate(&sl->ev_q));
                    st = hibf_gpu_agent_set_stream(sl->agent, sl->stream);
                    if (st != HIBF_GPU_OK)
                        fail(st, "agent stream");
                    uint64_t const mq = max_batch_queries, mv = max_batch_values;
                    st = hibf_gpu_agent_reserve(sl->agent, mq, mv, mq * 8 + 4096, mq * 16 + 4096);
                    if (st != HIBF_GPU_OK)
                        fail(st, "agent reserve");
                    sl->d_values.ensure(mv * 8);
                    sl->d_qoff.ensure((mq + 1) * 8);
                    sl->d_thr.ensure(mq * 8);
                    sl->h_values.ensure(mv * 8);
                    sl->h_qoff.ensure((mq + 1) * 8);
                    sl->h_thr.ensure(mq * 8);
                    sl->h_roff.ensure((mq + 1) * 8);
                    sl->h_ids.ensure((mq * 16 + 4096) * 8);
                    S->slots.push_back(std::move(sl));
                }
                // warm every slot: one single-value query in latency mode and one in throughput mode, so that the
                // first requests do not pay for loading kernels or first-touching buffers
                for (auto & sl : S->slots)
                {
                    uint64_t * hv = sl->h_values.as<uint64_t>();
                    uint64_t * ho = sl->h_qoff.as<uint64_t>();
                    uint64_t * ht = sl->h_thr.as<uint64_t>();
                    hv[0] = 0;
                    ho[0] = 0;
                    ho[1] = 1;
                    ht[0] = 1;
                    HG_CUDA(cudaMemcpyAsync(sl->d_values.p, hv, 8, cudaMemcpyHostToDevice, sl->stream));
                    HG_CUDA(cudaMemcpyAsync(sl->d_qoff.p, ho, 16, cudaMemcpyHostToDevice, sl->stream));
                    HG_CUDA(cudaMemcpyAsync(sl->d_thr.p, ht, 8, cudaMemcpyHostToDevice, sl->stream));
                    hibf_gpu_tuning t{}, warm{};
                    hibf_gpu_agent_get_tuning(sl->agent, &t);
                    for (uint32_t bq : {t.block_queries, 0u})
                    {
                        warm = t;
                        warm.block_queries = bq;
                        int st = hibf_gpu_agent_set_tuning(sl->agent, &warm);
                        uint64_t const *ro = nullptr, *ri = nullptr;
                        void const * rc = nullptr;
                        if (st == HIBF_GPU_OK)
                            st = hibf_gpu_agent_query_batch_d(sl->agent, HIBF_GPU_QUERY_MEMBERSHIP, sl->d_values.as<uint64_t>(),
                                                              sl->d_qoff.as<uint64_t>(), 1, sl->d_thr.as<uint64_t>(), 2,
                                                              &ro, &ri, &rc);
                        if (st == HIBF_GPU_OK)
                            st = hibf_gpu_agent_status(sl->agent);
                        if (st != HIBF_GPU_OK)
                            fail(st, "slot warm-up failed");
                    }
                    int const st = hibf_gpu_agent_set_tuning(sl->agent, &t);
                    if (st != HIBF_GPU_OK)
                        fail(st, "agent tuning");
                }
                hibf_gpu_server * raw = S.release();
                for (auto & sl : raw->slots)
                    raw->workers.emplace_back(slot_loop, raw, sl.get());
                *out = raw;
            });
    }

    int hibf_gpu_server_destroy(hibf_gpu_server * S)
    {
        return guarded(
            [&]
            {
                if (!S)
                    return;
                {
                    std::lock_guard<std::mutex> lk(S->mu);
                    S->stop.store(true);
                }
                S->cv_work.notify_all();
                for (auto & w : S->workers)
                    if (w.joinable())
                        w.join();
                for (auto const & hr : S->host_ranges)
                    if (hr.pinned_here)
                        cudaHostUnregister(reinterpret_cast<void *>(hr.begin));
                for (auto & sl : S->slots)
                {
                    cudaStreamSynchronize(sl->stream);
                    hibf_gpu_agent_destroy(sl->agent);
                    cudaEventDestroy(sl->ev);
                    cudaEventDestroy(sl->ev_in);
                    cudaEventDestroy(sl->ev_q);
                    cudaStreamDestroy(sl->stream);
                }
                delete S;
            });
    }

    int hibf_gpu_server_register_host(hibf_gpu_server * S, void const * ptr, uint64_t bytes, int already_pinned)
    {
        return guarded(
            [&]
            {
                if (!S || !ptr || bytes == 0)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "bad argument");
                if (!already_pinned) // mapped, so that zero-copy batches can read the range in place
                    HG_CUDA(cudaHostRegister(const_cast<void *>(ptr), bytes, cudaHostRegisterMapped));
                try
                {
                    warm_host_range(ptr, bytes);
                }
                catch (...)
                {
                    if (!already_pinned)
                        cudaHostUnregister(const_cast<void *>(ptr));
                    throw;
                }
                uintptr_t const b = reinterpret_cast<uintptr_t>(ptr);
                // the device's address of the range, if it maps page-locked memory (zero-copy batches)
                void * dev = nullptr;
                if (cudaHostGetDevicePointer(&dev, const_cast<void *>(ptr), 0) != cudaSuccess)
                {
                    cudaGetLastError();
                    dev = nullptr;
                }
                std::lock_guard<std::mutex> lk(S->mu);
                S->host_ranges.push_back(
                    hibf_gpu_server::host_range{b, b + bytes, !already_pinned, static_cast<uint64_t const *>(dev)});
            });
    }

    int hibf_gpu_server_set_zero_copy(hibf_gpu_server * S, int on)
    {
        return guarded(
            [&]
            {
                if (!S)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                std::lock_guard<std::mutex> lk(S->mu);
                S->zero_copy = on != 0;
            });
    }

    int hibf_gpu_server_unregister_host(hibf_gpu_server * S, void const * ptr)
    {
        return guarded(
            [&]
            {
                if (!S || !ptr)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "bad argument");
                uintptr_t const b = reinterpret_cast<uintptr_t>(ptr);
                bool pinned_here = false;
                {
                    std::lock_guard<std::mutex> lk(S->mu);
                    auto it = std::find_if(S->host_ranges.begin(), S->host_ranges.end(),
                                           [&](auto const & hr) { return hr.begin == b; });
                    if (it == S->host_ranges.end())
                        fail(HIBF_GPU_ERR_INVALID_ARG, "range not registered");
                    pinned_here = it->pinned_here;
                    S->host_ranges.erase(it);
                }
                if (pinned_here)
                    HG_CUDA(cudaHostUnregister(const_cast<void *>(ptr)));
            });
    }

    // Submits a request.  copy != 0: the data is copied and the caller's buffers may be reused on return; copy == 0:
    // the server reads the caller's buffers until the request is released (query_offsets[0] must be 0).
    // arrival_s: the request's arrival time on the server's steady clock (hibf_gpu_server_now), < 0 for "now".
    int hibf_gpu_server_submit(hibf_gpu_server * S, uint64_t const * values, uint64_t const * query_offsets,
                               uint64_t n_queries, uint64_t const * thresholds, double arrival_s, int copy,
                               uint64_t * id)
    {
        return guarded(
            [&]
            {
                if (!S || !query_offsets || (n_queries && !thresholds) || !id)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                auto r = std::make_unique<request>();
                r->nq = n_queries;
                r->nv = query_offsets[n_queries] - query_offsets[0];
                if (r->nv && !values)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null values");
                for (uint64_t i = 0; i < n_queries; ++i)
                {
                    if (thresholds[i] > 0xFFFFu)
                        fail(HIBF_GPU_ERR_INVALID_ARG, "membership thresholds are uint16");
                    if (query_offsets[i + 1] < query_offsets[i])
                        fail(HIBF_GPU_ERR_INVALID_ARG, "query offsets must be non-decreasing");
                }
                if (copy)
                {
                    r->own_values.assign(values + query_offsets[0], values + query_offsets[0] + r->nv);
                    r->own_qoff.resize(n_queries + 1);
                    for (uint64_t i = 0; i <= n_queries; ++i)
                        r->own_qoff[i] = query_offsets[i] - query_offsets[0];
                    r->own_thr.assign(thresholds, thresholds + n_queries);
                    r->values = r->own_values.data();
                    r->qoff = r->own_qoff.data();
                    r->thr = r->own_thr.data();
                }
                else
                {
                    if (query_offsets[0] != 0)
                        fail(HIBF_GPU_ERR_INVALID_ARG, "borrowed requests need query_offsets[0] == 0");
                    r->values = values;
                    r->qoff = query_offsets;
                    r->thr = thresholds;
                    // registered page-locked memory is copied to the device without staging (a host-side range
                    // check: no CUDA call on the submitting thread)
                    uintptr_t const b = reinterpret_cast<uintptr_t>(values);
                    uintptr_t const e = b + r->nv * 8;
                    std::lock_guard<std::mutex> lk(S->mu);
                    for (auto const & hr : S->host_ranges)
                        if (r->nv && b >= hr.begin && e <= hr.end)
                        {
                            r->pinned = true;
                            r->dev_values =
                                hr.dev ? reinterpret_cast<uint64_t const *>(reinterpret_cast<char const *>(hr.dev) +
                                                                            (b - hr.begin))
                                       : nullptr;
                        }
                }
                r->t_arrival = arrival_s >= 0 ? arrival_s : now_s();
                std::lock_guard<std::mutex> lk(S->mu);
                r->id = S->next_id++;
                *id = r->id;
                S->waiting.push_back(r.get());
                S->reqs.emplace(r->id, std::move(r));
                S->cv_work.notify_one();
            });
    }

    // Waits (up to timeout_ms; < 0 forever) for a request.  On completion *status holds its status and the result
    // pointers (valid until hibf_gpu_server_release) its sorted membership lists per query.
    int hibf_gpu_server_wait(hibf_gpu_server * S, uint64_t id, double timeout_ms, int * status,
                             uint64_t const ** result_offsets, uint64_t const ** result_ids, double * latency_s)
    {
        return guarded(
            [&]
            {
                if (!S || !status)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                std::unique_lock<std::mutex> lk(S->mu);
                auto it = S->reqs.find(id);
                if (it == S->reqs.end())
                    fail(HIBF_GPU_ERR_INVALID_ARG, "unknown request id");
                request * r = it->second.get();
                auto pred = [&] { return r->done.load(); };
                if (timeout_ms < 0)
                    S->cv_done.wait(lk, pred);
                else if (!S->cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), pred))
                    fail(HIBF_GPU_ERR_TIMEOUT, "request not finished within the timeout");
                *status = r->status;
                if (result_offsets)
                    *result_offsets = r->res_off.data();
                if (result_ids)
                    *result_ids = r->res_ids.data();
                if (latency_s)
                    *latency_s = r->t_done - r->t_arrival;
            });
    }

    int hibf_gpu_server_release(hibf_gpu_server * S, uint64_t id)
    {
        return guarded(
            [&]
            {
                if (!S)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                std::lock_guard<std::mutex> lk(S->mu);
                auto it = S->reqs.find(id);
                if (it == S->reqs.end() || !it->second->done)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "unknown or unfinished request");
                S->reqs.erase(it);
            });
    }

    double hibf_gpu_server_now(void)
    {
        return now_s();
    }

    // out: mean seconds per batch of queueing (its oldest request), staging + launch, device work, result fetch, split
    int hibf_gpu_server_phase_times(hibf_gpu_server * S, double out[5])
    {
        return guarded(
            [&]
            {
                if (!S || !out)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                std::lock_guard<std::mutex> lk(S->mu);
                double const n = S->batches ? static_cast<double>(S->batches) : 1.0;
                out[0] = S->t_queue / n;
                out[1] = S->t_stage / n;
                out[2] = S->t_device / n;
                out[3] = S->t_fetch / n;
                out[4] = S->t_split / n;
            });
    }

    int hibf_gpu_server_batch_log(hibf_gpu_server * S, double * out, uint64_t cap, uint64_t * n)
    {
        return guarded(
            [&]
            {
                if (!S || !n || (cap && !out))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                std::lock_guard<std::mutex> lk(S->mu);
                *n = S->batch_log.size();
                for (uint64_t i = 0; i < std::min<uint64_t>(cap, S->batch_log.size()); ++i)
                    std::copy(S->batch_log[i].begin(), S->batch_log[i].end(),
                              out + hibf_gpu_server::kBatchLogCols * i);
            });
    }

    // out: batches, batched queries, rejected requests, bytes in flight
    int hibf_gpu_server_stats(hibf_gpu_server * S, uint64_t out[4])
    {
        return guarded(
            [&]
            {
                if (!S || !out)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                std::lock_guard<std::mutex> lk(S->mu);
                out[0] = S->batches;
                out[1] = S->batched_queries;
                out[2] = S->rejected;
                out[3] = S->inflight_bytes;
            });
    }

    // Open-loop load: requests arrive as a Poisson process (rate = offered queries/s / mean request size), request
    // sizes log-uniform in [1, max_request_queries], queries drawn cyclically from a pool (CSR, host), per-request
    // thresholds ceil(f * length) with f uniform in [thr_lo, thr_hi].  Runs `duration_s`, then waits for every
    // request.  out: achieved queries/s, p50, p99, p99.9 latency (s), requests, queries, rejected, mean batch size.
    int hibf_gpu_server_open_loop(hibf_gpu_server * S, uint64_t const * pool_values, uint64_t const * pool_offsets,
                                  uint64_t pool_queries, double offered_qps, double duration_s,
                                  uint64_t max_request_queries, double thr_lo, double thr_hi, uint64_t seed,
                                  double out[8])
    {
        return guarded(
            [&]
            {
                if (!S || !pool_values || !pool_offsets || pool_queries == 0 || offered_qps <= 0 || !out)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "bad argument");
                std::mt19937_64 rng(seed);
                std::uniform_real_distribution<double> U(0.0, 1.0);
                double const lmax = std::log(static_cast<double>(max_request_queries));
                // mean of floor(exp(U(0, lmax))) ~ (max - 1) / lmax
                double const mean_size = max_request_queries > 1
                                             ? (static_cast<double>(max_request_queries) - 1.0) / lmax
                                             : 1.0;
                double const req_rate = offered_qps / mean_size;
                struct plan
                {
                    double t;
                    uint64_t q0, nq;
                    double f;
                };
                std::vector<plan> plans;
                double t = 0;
                uint64_t q = 0;
                while (true)
                {
                    t += -std::log(1.0 - U(rng)) / req_rate;
                    if (t > duration_s)
                        break;
                    uint64_t nq = static_cast<uint64_t>(std::floor(std::exp(U(rng) * lmax)));
                    nq = std::max<uint64_t>(1, std::min(nq, max_request_queries));
                    nq = std::min(nq, pool_queries);
                    plans.push_back(plan{t, q % pool_queries, nq, thr_lo + (thr_hi - thr_lo) * U(rng)});
                    q += nq;
                }
                // Requests borrow contiguous slices of the pool (a request that would wrap starts at query 0).  The
                // pool is registered with the server for the run, as a client that registers its receive buffers
                // would have it, so the server copies request values to the device without staging them.
                uint64_t const pool_bytes = pool_offsets[pool_queries] * 8;
                bool registered = false;
                if (pool_bytes)
                {
                    // a pool that is already page-locked (cudaHostAlloc) is registered as such
                    cudaPointerAttributes a{};
                    bool const pinned =
                        cudaPointerGetAttributes(&a, pool_values) == cudaSuccess && a.type == cudaMemoryTypeHost;
                    cudaGetLastError();
                    registered = hibf_gpu_server_register_host(S, pool_values, pool_bytes, pinned ? 1 : 0) ==
                                 HIBF_GPU_OK;
                }
                struct unregister_guard
                {
                    hibf_gpu_server * s;
                    void const * p;
                    ~unregister_guard()
                    {
                        if (p)
                            hibf_gpu_server_unregister_host(s, p);
                    }
                } guard{S, registered ? pool_values : nullptr};
                std::vector<std::vector<uint64_t>> offs(plans.size()), thrs(plans.size());
                std::vector<uint64_t const *> vals(plans.size());
                for (size_t i = 0; i < plans.size(); ++i)
                {
                    auto & p = plans[i];
                    if (p.q0 + p.nq > pool_queries)
                        p.q0 = 0;
                    uint64_t const base = pool_offsets[p.q0];
                    vals[i] = pool_values + base;
                    offs[i].push_back(0);
                    for (uint64_t k = 0; k < p.nq; ++k)
                    {
                        uint64_t const qi = p.q0 + k;
                        uint64_t const b = pool_offsets[qi], e = pool_offsets[qi + 1];
                        offs[i].push_back(e - base);
                        thrs[i].push_back(static_cast<uint64_t>(std::ceil(p.f * static_cast<double>(e - b))));
                    }
                }
                std::vector<uint64_t> ids(plans.size(), 0);
                std::vector<double> late(plans.size(), 0.0); // submission behind the scheduled arrival
                double const t0 = now_s() + 0.01;
                for (size_t i = 0; i < plans.size(); ++i)
                {
                    double const ta = t0 + plans[i].t;
                    double tn = now_s();
                    while (tn < ta)
                        tn = now_s();
                    late[i] = tn - ta;
                    int const st = hibf_gpu_server_submit(S, vals[i], offs[i].data(), plans[i].nq, thrs[i].data(), ta,
                                                          0, &ids[i]);
                    if (st != HIBF_GPU_OK)
                        fail(st, "submit failed");
                }
                std::vector<double> lat, lat_sub;
                lat.reserve(plans.size());
                lat_sub.reserve(plans.size());
                uint64_t nqs = 0, rej = 0;
                double t_end = t0;
                for (size_t i = 0; i < plans.size(); ++i)
                {
                    int st = 0;
                    double l = 0;
                    int const w = hibf_gpu_server_wait(S, ids[i], 600000.0, &st, nullptr, nullptr, &l);
                    if (w != HIBF_GPU_OK)
                        fail(w, "wait failed");
                    if (st == HIBF_GPU_OK)
                    {
                        lat.push_back(l);
                        lat_sub.push_back(l - late[i]);
                        nqs += plans[i].nq;
                        t_end = std::max(t_end, t0 + plans[i].t + l);
                    }
                    else
                        ++rej;
                    hibf_gpu_server_release(S, ids[i]);
                }
                std::sort(lat.begin(), lat.end());
                std::sort(lat_sub.begin(), lat_sub.end());
                auto pct_of = [](std::vector<double> const & v, double p) -> double
                {
                    if (v.empty())
                        return 0.0;
                    size_t const k = std::min(v.size() - 1, static_cast<size_t>(std::ceil(p * v.size())) - 1);
                    return v[k];
                };
                auto pct = [&](double p) { return pct_of(lat, p); };
                std::vector<double> late_sorted = late;
                std::sort(late_sorted.begin(), late_sorted.end());
                {
                    std::lock_guard<std::mutex> lk(S->mu);
                    S->open_loop_detail[0] = late_sorted.empty() ? 0.0 : late_sorted.back();
                    S->open_loop_detail[1] = pct_of(late_sorted, 0.999);
                    S->open_loop_detail[2] = static_cast<double>(
                        std::count_if(late.begin(), late.end(), [](double x) { return x > 1e-3; }));
                    S->open_loop_detail[3] = pct_of(lat_sub, 0.99);
                    S->open_loop_detail[4] = pct_of(lat_sub, 0.999);
                }
                uint64_t st4[4];
                hibf_gpu_server_stats(S, st4);
                out[0] = static_cast<double>(nqs) / std::max(1e-9, t_end - t0);
                out[1] = pct(0.50);
                out[2] = pct(0.99);
                out[3] = pct(0.999);
                out[4] = static_cast<double>(plans.size());
                out[5] = static_cast<double>(nqs);
                out[6] = static_cast<double>(rej);
                out[7] = st4[0] ? static_cast<double>(st4[1]) / static_cast<double>(st4[0]) : 0.0;
            });
    }

    int hibf_gpu_server_open_loop_detail(hibf_gpu_server * S, double out[5])
    {
        return guarded(
            [&]
            {
                if (!S || !out)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                std::lock_guard<std::mutex> lk(S->mu);
                std::copy(S->open_loop_detail, S->open_loop_detail + 5, out);
            });
    }

} // extern "C"
