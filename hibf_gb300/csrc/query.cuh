// query.cuh -- the persistent (query, IBF) work-queue kernel of the HIBF query, templated on the hash function count
// H and on a tuning variant V (values hashed per lane, register counter width, bytes fetched per lane).
//
// Query semantics (membership_for_impl HIBF.hpp:322-355, bulk_count_impl HIBF.hpp:463-496): for a query and an IBF,
// count every value per technical bin, then scan the bins in order adding each bin's count to a running sum in the
// counter type: deleted -> no report, no reset;   merged -> descend if sum >= t, reset;   last bin of a user bin ->
// report if sum >= t, reset.  Per bin the host precomputes MERGED, DELETED, RUN_END (last bin of a user bin's run) and HEAD (first bin
// of a summation segment: bin 0 or the bin after a MERGED / RUN_END bin), which turns the scan into a segmented
// prefix sum, done 32 bins at a time by a warp.  Counter wraparound: exact sums reduced modulo 2^(8*width) before
// the comparison equal the reference's wrapping value_t sums.
//
// Work queue: task = (query, depth, IBF).  Claim indices below n_queries are the implicit root tasks; children are
// appended behind them.  A worker that claims an index whose task is not written yet waits (bounded by a time
// limit) until it appears or the count of unfinished tasks drops to zero.  Children are added to that count
// before their parent retires, so zero means no task is queued or running anywhere.  With streamed inputs (a large
// host batch copied while the kernel runs) roots and children are claimed through separate counters, a root only
// once its chunk of values has arrived (k_query).
//
// The kernels are instantiated per H in query_h<H>.cu (one translation unit each, compiled in parallel); the host
// side (hibf.cu) picks one through query_kernel(h, variant).
#pragma once

#include "count.cuh"
#include "device.cuh"
#include "hibf_internal.cuh"

namespace hibf_gb300
{

// query_params::ee_stages value of the adaptive early exit (checks where the outcome can first change, ee_step
// values apart at least); the same as HIBF_GPU_EARLY_EXIT_ADAPTIVE of the C interface.
constexpr uint32_t kEarlyExitAdaptive = 0xFFFFFFFFu;

constexpr uint32_t F_MERGED = 1u;
constexpr uint32_t F_DELETED = 2u;
constexpr uint32_t F_RUN_END = 4u;
constexpr uint32_t F_HEAD = 8u;

constexpr unsigned long long kEmpty = ~0ull;
// stats words: tasks, value visits the reference's traversal implies, value visits executed
constexpr int kStats = 3;
constexpr uint32_t kNodeBits = 26;
constexpr uint32_t kNodeMask = (1u << kNodeBits) - 1u;

// control words
enum : int
{
    C_HEAD = 0,
    C_TAIL = 1,
    C_PENDING = 2,
    C_NREC = 3,
    C_ERROR = 4,
    C_NLARGE = 5,
    C_CHILD = 6, // streamed inputs: claims of child slots (roots and children are then claimed separately)
    C_WORDS = 8
};
// error bits
constexpr unsigned long long E_OVERFLOW_REC = 1ull;
constexpr unsigned long long E_OVERFLOW_TASK = 2ull;
constexpr unsigned long long E_TIMEOUT = 4ull;
constexpr unsigned long long E_CYCLE = 8ull;
constexpr unsigned long long E_VARIANT = 16ull; // a tuned variant met a row of more than 4 words (host rejects this)
constexpr unsigned long long E_ORDER = 32ull;   // a claim-order entry was not a query index (skipped)
constexpr unsigned long long E_TASK = 64ull;    // a task word named a query or IBF out of range (skipped)

// Tuning variants of the counting loop (compile-time), one kernel each:
//   UM  values hashed per lane per pass, as a multiple of max(1, 4 / lanes-per-row): more row loads in flight
//   K   width in bits of the per-lane bit-sliced counters (flushed to shared memory every 2^K - 4 masks)
//   W   64-bit words fetched per lane per row (1: 8-byte loads; 2: 16-byte loads, half the lanes per row)
// Every variant computes the same exact counts; only the schedule differs.
constexpr int kQueryVariants = 6;
// {UM, W, K} of variant V; variant 0 is the default schedule.
constexpr int kVariantTable[kQueryVariants][3] = {{1, 1, 7}, {2, 1, 7}, {1, 1, 5}, {2, 1, 5}, {1, 2, 7}, {1, 2, 5}};
template <int V>
struct qvariant
{
    static constexpr int UM = kVariantTable[V][0];
    static constexpr int W = kVariantTable[V][1];
    static constexpr int K = kVariantTable[V][2];
};

struct query_params
{
    dev_node const * nodes;
    uint2 const * descs; // .x = user bin or next IBF, .y = flags
    uint64_t const * values;
    uint64_t const * qoff;
    uint64_t const * thr;
    uint64_t count_mask;
    uint64_t n_queries;
    uint32_t n_nodes; // IBFs of the hierarchy: a task naming another is skipped (E_TASK), never dereferenced
    uint64_t q_base; // added to the query index in records and per-query counters (plain form)
    uint32_t max_depth;
    uint32_t counters_per_warp;
    unsigned long long * tasks;
    uint64_t task_cap;
    unsigned long long * ctrl;
    uint32_t * rec_q;
    uint32_t * rec_ub;
    unsigned long long * rec_cnt;
    uint64_t rec_cap;
    unsigned int * qcount;
    unsigned long long * stats;
    uint64_t wait_limit_ns;
    int self_init; // single-block launch that resets its own control words first
    // early exit: after counting first + s * step percent of a task's values (s < stages), stop when no segment can
    // reach the threshold any more; tasks shorter than ee_min values are counted in one stage
    uint32_t ee_first;
    uint32_t ee_step;
    uint32_t ee_stages;
    uint32_t ee_min;
    // optional: root tasks are claimed in this order of queries (a permutation of 0..n_queries-1), and the executed
    // value visits of every query are added to qwork[query + q_base]
    uint32_t const * order;
    unsigned long long * qwork;
    // membership mode: a task may also stop once every segment's report/descend decision is final (segment_state)
    uint32_t decide;
    // streamed inputs (host batches): the values of queries [arrive_first[k], arrive_first[k + 1]) are on the device
    // once the chunk counter exceeds k (copied behind chunk k's values on the same stream); the counter is replicated
    // kArrivalReplicas times, kArrivalStride words apart, and block b polls replica b % kArrivalReplicas; null = all
    // inputs are resident
    unsigned int const * arrived;
    uint64_t const * arrive_first;
    uint32_t arrive_chunks;
    uint64_t arrive_limit_ns;
    // level schedule (HIBF_GPU_SCHEDULE_LEVELS): this launch answers one level of tasks and only appends the tasks of
    // the next level (emit_task); claims run from 0 to the level's size and stop there.  The root level (in_tasks
    // null) claims the implicit root tasks; a later level claims in_tasks[0, *in_count), grouped by IBF.
    uint32_t level;
    unsigned long long const * in_tasks;
    unsigned long long const * in_count;
    // in-place host batches under the level schedule: `values` is the host's memory; root tasks store every value
    // they read at stage[same position] and how many they read (from the query's first value) at staged[query], and
    // the lower levels read that prefix from stage and only the rest from the host.  Null otherwise.
    uint64_t * stage;
    uint32_t * staged;
};

using query_kernel_t = void (*)(query_params);

// One 128-byte line per replica of the chunk counter: thousands of warps polling a single line starve the copy
// stream's write of it (and with it the copies queued behind), so blocks spread their polls over 64 lines.
constexpr uint32_t kArrivalReplicas = 64;
constexpr uint32_t kArrivalStride = 32;

__device__ __forceinline__ unsigned int arrival_count(query_params const & p)
{
    return *(reinterpret_cast<volatile unsigned int const *>(p.arrived) +
             (blockIdx.x % kArrivalReplicas) * kArrivalStride);
}

__device__ __forceinline__ unsigned long long make_task(uint64_t q, uint32_t depth, uint32_t node)
{
    return (static_cast<unsigned long long>(q) << 32) | (static_cast<unsigned long long>(depth) << kNodeBits) | node;
}

__device__ inline unsigned long long wait_for_task(query_params const & p, unsigned long long slot)
{
    volatile unsigned long long * t = p.tasks + slot;
    volatile unsigned long long * pending = p.ctrl + C_PENDING;
    uint64_t start = 0;
    for (uint32_t it = 0;; ++it)
    {
        unsigned long long v = *t;
        if (v != kEmpty)
            return v;
        if (*pending == 0ull)
        {
            __threadfence();
            return *t; // still empty: nothing is queued or running, the batch is done
        }
        if (it == 0)
            start = globaltimer_ns();
        else if ((it & 31u) == 0 && globaltimer_ns() - start > p.wait_limit_ns)
        {
            atomicOr(p.ctrl + C_ERROR, E_TIMEOUT);
            return kEmpty;
        }
        __nanosleep(256);
    }
}

// Streamed inputs: the chunk counter value at which query q's values are on the device (its chunk index + 1).  The
// copy stream copies the counter behind each chunk's values (stream order: after they are written), and chunks start
// on 32-byte sector boundaries, so no sector holding values of an unarrived chunk was cached before.
__device__ inline unsigned int arrival_needed(query_params const & p, uint64_t q)
{
    uint32_t lo = 0, hi = p.arrive_chunks - 1u; // the last chunk k with arrive_first[k] <= q
    while (lo < hi)
    {
        uint32_t const mid = (lo + hi + 1u) >> 1;
        if (p.arrive_first[mid] <= q)
            lo = mid;
        else
            hi = mid - 1u;
    }
    return lo + 1u;
}

// Streamed inputs: claims the oldest queued child slot (lane 0) when at least `reserve` reserved slots are unclaimed,
// else kEmpty.  With reserve = the grid's warp count no claim can pass the reserved slots (fewer warps than that claim
// at the same time), so a claimed slot is written soon by its producer; a plain atomicAdd does the claim, since
// compare-and-swap retries of thousands of warps on one word stall its L2 slice.
__device__ inline unsigned long long try_claim_child(query_params const & p, unsigned long long reserve)
{
    volatile unsigned long long * c = p.ctrl;
    unsigned long long const h = c[C_CHILD];
    if (c[C_TAIL] < h + reserve)
        return kEmpty;
    unsigned long long const s = atomicAdd(p.ctrl + C_CHILD, 1ull);
    return s < p.task_cap ? s : kEmpty;
}

// Waits (bounded) until query q's chunk has arrived.  False (and E_TIMEOUT) when the limit expires.
__device__ inline bool wait_arrival(query_params const & p, uint64_t q)
{
    unsigned int const need = arrival_needed(p, q);
    uint64_t start = 0;
    for (uint32_t it = 0;; ++it)
    {
        if (arrival_count(p) >= need)
        {
            __threadfence();
            return true;
        }
        if (it == 0)
            start = globaltimer_ns();
        else if ((it & 15u) == 0 && globaltimer_ns() - start > p.arrive_limit_ns)
        {
            atomicOr(p.ctrl + C_ERROR, E_TIMEOUT);
            return false;
        }
        __nanosleep(512);
    }
}

// The state of a task after counting all but `remaining` of its values, from each summation segment's sum so far x
// and its number of bins w (every bin of a segment adds its count, and a value adds at most one to every bin, so the
// final sum lies in [x, top] with top = x + w * remaining):
//   kHopeless  no segment can reach the threshold (top < t for all): nothing is reported or descended;
//   kDecided   (membership only, `decide`) every segment either has reached the threshold for good (x >= t and no
//              wrap possible: top <= counter mask) or can no longer reach it: the reports and descents are final,
//              and the bin scan on the partial counts makes exactly them;
//   kOpen      otherwise.
// A sum that could exceed the counter range is never decided (its wrapped value is not bounded).  Either early state
// gives the same outcome as counting every value.
//
// `next` (if given) receives how many more values must be counted before the state can change at all (top falls by
// at most w and x grows by at most w per value): an open segment passes for good no sooner than after
// ceil((t - x) / w) values (and ceil((top - mask) / w) for a sum that could wrap), and turns unreachable no sooner
// than after ceil((top - t + 1) / w); a task turns hopeless only once every reachable segment can be unreachable, and
// (membership) decided once every open segment can be settled.  kNever: no later change is possible (a segment that
// reached the threshold keeps a bulk count open).
constexpr int kOpen = 0;
constexpr int kHopeless = 1;
constexpr int kDecided = 2;
constexpr unsigned int kNever = 0xFFFFFFFFu;

__device__ __forceinline__ unsigned long long ceil_div(unsigned long long a, unsigned long long w)
{
    return (a + w - 1u) / w;
}

__device__ inline int segment_state(query_params const & p, dev_node const & nd, uint32_t const * counts,
                                    uint64_t remaining, uint64_t thr, int lane, unsigned int * next = nullptr)
{
    uint2 const * d = p.descs + nd.desc_offset;
    unsigned long long carry = 0, carry_w = 0;
    bool any_reachable = false, any_open = false;
    unsigned int wait = 0; // per lane: the largest earliest-change distance of its segments
    bool never = false;
    unsigned long long const mask = p.count_mask;
    for (uint32_t c = 0; c < nd.bins; c += 32)
    {
        uint32_t const b = c + lane;
        bool const valid = b < nd.bins;
        uint2 const ds = valid ? d[b] : make_uint2(0u, 0u);
        unsigned long long x = valid ? static_cast<unsigned long long>(counts[b]) : 0ull;
        unsigned long long w = valid ? 1ull : 0ull;
        bool f = valid && (ds.y & F_HEAD);
        if (lane == 0 && !f)
        {
            x += carry;
            w += carry_w;
        }
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            unsigned long long const y = __shfl_up_sync(kFullMask, x, o);
            unsigned long long const yw = __shfl_up_sync(kFullMask, w, o);
            int const fy = __shfl_up_sync(kFullMask, static_cast<int>(f), o);
            if (lane >= o)
            {
                if (!f)
                {
                    x += y;
                    w += yw;
                }
                f = f || fy;
            }
        }
        bool const ends = valid && (ds.y & (F_RUN_END | F_MERGED));
        // x + w * remaining, saturated (the product cannot overflow for the sizes a batch admits, but stay safe)
        unsigned long long const top =
            remaining > (~0ull - x) / (w ? w : 1ull) ? ~0ull : x + w * static_cast<unsigned long long>(remaining);
        bool const reachable = ends && (top >= thr || top > mask);
        bool const passed = x >= thr && top <= mask;
        any_reachable = __any_sync(kFullMask, reachable) || any_reachable;
        any_open = __any_sync(kFullMask, reachable && !passed) || any_open;
        unsigned long long const lastx = __shfl_sync(kFullMask, x, 31);
        unsigned long long const lastw = __shfl_sync(kFullMask, w, 31);
        uint32_t const lastf = __shfl_sync(kFullMask, ds.y, 31);
        bool const cut = (lastf & (F_MERGED | F_RUN_END)) != 0;
        carry = cut ? 0ull : lastx;
        carry_w = cut ? 0ull : lastw;
        if (next)
        {
            if (reachable)
            {
                unsigned long long const unreach = ceil_div(top >= thr ? top - thr + 1u : top - mask, w);
                unsigned long long k = 0;
                if (p.decide)
                {
                    if (!passed)
                        k = min(unreach, max(x < thr ? ceil_div(thr - x, w) : 0ull,
                                             top > mask ? ceil_div(top - mask, w) : 0ull));
                }
                else if (x >= thr)
                    never = true; // a reached segment stays reachable: the bulk count never turns hopeless
                else
                    k = unreach;
                wait = max(wait, static_cast<unsigned int>(min(k, 0xFFFFFFFEull)));
            }
        }
        else if (any_reachable && !p.decide)
            return kOpen; // only hopelessness is of interest: one reachable segment settles it
    }
    if (next)
    {
        bool const nv = __any_sync(kFullMask, never);
        unsigned int const wmax = __reduce_max_sync(kFullMask, wait);
        *next = nv ? kNever : max(wmax, 1u);
    }
    if (!any_reachable)
        return kHopeless;
    if (!p.decide)
        return kOpen;
    return any_open ? kOpen : kDecided;
}

// Counting with variant V.  Variant 0 handles every row width; the tuned variants only rows of up to 4 words (the
// host offers them only for such hierarchies, and process_task refuses wider rows).
template <int H, int V>
__device__ __forceinline__ void count_variant(row_params const & rp, uint32_t lpv_log2, uint64_t const * vals,
                                              uint64_t n, uint32_t * counts, int lane, uint64_t * stage)
{
    using Q = qvariant<V>;
    switch (lpv_log2)
    {
    case 0:
        warp_count<1, H, Q::K, false, Q::UM, 1>(rp, vals, n, counts, lane, stage);
        break;
    case 1:
        if constexpr (Q::W == 2)
            warp_count<1, H, Q::K, false, Q::UM, 2>(rp, vals, n, counts, lane, stage);
        else
            warp_count<2, H, Q::K, false, Q::UM, 1>(rp, vals, n, counts, lane, stage);
        break;
    case 2:
        if constexpr (Q::W == 2)
            warp_count<2, H, Q::K, false, Q::UM, 2>(rp, vals, n, counts, lane, stage);
        else
            warp_count<4, H, Q::K, false, Q::UM, 1>(rp, vals, n, counts, lane, stage);
        break;
    default:
        if constexpr (V == 0)
            warp_count_h<H, false>(rp, lpv_log2, vals, n, counts, lane, stage);
    }
}

// The bin scan of a counted task: report user bins and queue child IBFs whose summation segment reaches the
// threshold, then retire the task (one warp; `counts` = the task's per-bin counts).
__device__ inline void emit_task(query_params const & p, dev_node const & nd, uint32_t const * counts, uint64_t q,
                                 uint32_t depth, uint64_t n, uint64_t done, uint64_t thr, int lane,
                                 unsigned long long & n_tasks, unsigned long long & n_visits,
                                 unsigned long long & n_executed)
{
    uint2 const * d = p.descs + nd.desc_offset;
    unsigned long long carry = 0;
    unsigned const lt_mask = (1u << lane) - 1u;
    uint64_t const gq = q + p.q_base;
    for (uint32_t c = 0; c < nd.bins; c += 32)
    {
        uint32_t const b = c + lane;
        bool const valid = b < nd.bins;
        uint2 const ds = valid ? d[b] : make_uint2(0u, 0u);
        unsigned long long x = valid ? counts[b] : 0ull;
        bool f = valid && (ds.y & F_HEAD);
        if (lane == 0 && !f)
            x += carry;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            unsigned long long const y = __shfl_up_sync(kFullMask, x, o);
            int const fy = __shfl_up_sync(kFullMask, static_cast<int>(f), o);
            if (lane >= o)
            {
                if (!f)
                    x += y;
                f = f || fy;
            }
        }
        uint64_t const sum = x & p.count_mask;
        bool const pass = sum >= thr;
        bool const emit_ub = valid && (ds.y & F_RUN_END) && pass;
        bool const emit_child = valid && (ds.y & F_MERGED) && pass;

        unsigned const rb = __ballot_sync(kFullMask, emit_ub);
        if (rb)
        {
            unsigned const nr = __popc(rb);
            unsigned long long base = 0;
            if (lane == 0)
            {
                base = atomicAdd(p.ctrl + C_NREC, static_cast<unsigned long long>(nr));
                atomicAdd(p.qcount + gq, nr);
                if (base + nr > p.rec_cap)
                    atomicOr(p.ctrl + C_ERROR, E_OVERFLOW_REC);
            }
            base = __shfl_sync(kFullMask, base, 0);
            if (emit_ub)
            {
                unsigned long long const r = base + __popc(rb & lt_mask);
                if (r < p.rec_cap)
                {
                    p.rec_q[r] = static_cast<uint32_t>(gq);
                    p.rec_ub[r] = ds.x;
                    p.rec_cnt[r] = sum;
                }
            }
        }
        unsigned const cb = __ballot_sync(kFullMask, emit_child);
        if (cb)
        {
            unsigned const nc = __popc(cb);
            if (depth + 1u > p.max_depth)
            {
                if (lane == 0)
                    atomicOr(p.ctrl + C_ERROR, E_CYCLE);
            }
            else
            {
                unsigned long long base = 0;
                if (lane == 0)
                {
                    atomicAdd(p.ctrl + C_PENDING, static_cast<unsigned long long>(nc));
                    base = atomicAdd(p.ctrl + C_TAIL, static_cast<unsigned long long>(nc));
                }
                base = __shfl_sync(kFullMask, base, 0);
                if (emit_child)
                {
                    unsigned long long const s = base + __popc(cb & lt_mask);
                    if (s < p.task_cap)
                    {
                        atomicExch(p.tasks + s, make_task(q, depth + 1u, ds.x));
                    }
                    else
                    {
                        atomicOr(p.ctrl + C_ERROR, E_OVERFLOW_TASK);
                        atomicAdd(p.ctrl + C_PENDING, ~0ull); // this child will never run
                    }
                    __threadfence();
                }
            }
        }
        unsigned long long const lastx = __shfl_sync(kFullMask, x, 31);
        uint32_t const lastf = __shfl_sync(kFullMask, ds.y, 31);
        carry = (lastf & (F_MERGED | F_RUN_END)) ? 0ull : lastx;
    }
    __syncwarp();
    if (lane == 0)
    {
        if (p.qwork)
            atomicAdd(p.qwork + q + p.q_base, static_cast<unsigned long long>(done));
        __threadfence();
        atomicAdd(p.ctrl + C_PENDING, ~0ull); // this task retires
        ++n_tasks;
        n_visits += n;
        n_executed += done;
    }
}


template <int H, int V>
__device__ void process_task(query_params const & p, unsigned long long task, uint32_t * counts, int lane,
                             unsigned long long & n_tasks, unsigned long long & n_visits,
                             unsigned long long & n_executed)
{
    uint64_t const q = task >> 32;
    uint32_t const depth = static_cast<uint32_t>(task >> kNodeBits) & 63u;
    uint32_t const k = static_cast<uint32_t>(task) & kNodeMask;
    if (q >= p.n_queries || k >= p.n_nodes)
    {
        if (lane == 0)
        {
            atomicOr(p.ctrl + C_ERROR, E_TASK);
            __threadfence();
            atomicAdd(p.ctrl + C_PENDING, ~0ull);
        }
        return;
    }
    dev_node const nd = p.nodes[k];
    uint64_t const b0 = p.qoff[q];
    uint64_t const n = p.qoff[q + 1] - b0;
    uint64_t const thr = p.thr[q];

    if (V != 0 && nd.lpv_log2 > 2)
    {
        if (lane == 0)
        {
            atomicOr(p.ctrl + C_ERROR, E_VARIANT);
            __threadfence();
            atomicAdd(p.ctrl + C_PENDING, ~0ull);
        }
        return;
    }
    uint32_t const ncount = nd.bin_words > 32 ? 64u * nd.bin_words : (64u << nd.lpv_log2);
    for (uint32_t i = lane; i < ncount; i += 32)
        counts[i] = 0;
    __syncwarp();
    row_params const rp{nd.words, nd.bin_size, nd.row_words, nd.bin_words, nd.hash_shift, nd.hash_funs};
    // Count in stages; after each stage stop if the outcome is already fixed (segment_state: exact).  One call site
    // of the counting code for the stages and the rest: each call site inlines every row width's counting path, and a
    // hierarchy of mixed widths runs them all at once, so a second copy would double the instruction footprint.
    uint64_t done = 0;
    // in-place host batch under the level schedule: a root stages what it reads; a lower level reads the staged prefix
    // [0, staged) from device memory and the rest from the host
    bool const stage_root = p.stage && depth == 0;
    uint64_t const staged = p.stage && depth > 0 ? p.staged[q] : 0u;
    bool const adaptive = p.ee_stages == kEarlyExitAdaptive && n >= p.ee_min;
    unsigned int next = kNever;
    int state = segment_state(p, nd, counts, n, thr, lane, adaptive ? &next : nullptr);
    uint32_t const stages = !adaptive && state == kOpen && n >= p.ee_min ? p.ee_stages : 0u;
    uint32_t s = 0;
#pragma unroll 1
    while (state == kOpen && done < n)
    {
        uint64_t stop = n; // the next checkpoint past `done` (checkpoints are below 100%, so below n), else the end
        if (adaptive)
        {
            // the earliest position where the outcome can change, at least ee_step values on
            if (next != kNever)
                stop = min(n, done + static_cast<uint64_t>(max(next, p.ee_step)));
        }
        else
        {
            for (; s < stages; ++s)
            {
                uint64_t const c = n * (p.ee_first + s * p.ee_step) / 100u;
                if (c > done)
                {
                    stop = c;
                    ++s;
                    break;
                }
            }
        }
        // one call site: [done, stop) in at most two pieces, the staged prefix first
        while (done < stop)
        {
            bool const from_stage = done < staged;
            uint64_t const end = from_stage ? min(stop, staged) : stop;
            count_variant<H, V>(rp, nd.lpv_log2, (from_stage ? p.stage : p.values) + b0 + done, end - done, counts,
                                lane, stage_root ? p.stage + b0 + done : nullptr);
            done = end;
        }
        if (done < n)
        {
            __syncwarp();
            state = segment_state(p, nd, counts, n - done, thr, lane, adaptive ? &next : nullptr);
        }
    }
    __syncwarp();
    if (stage_root && lane == 0)
        p.staged[q] = static_cast<uint32_t>(done); // read by the next level's launch
    if (state == kHopeless)
    {
        if (lane == 0)
        {
            if (p.qwork)
                atomicAdd(p.qwork + q + p.q_base, static_cast<unsigned long long>(done));
            __threadfence();
            atomicAdd(p.ctrl + C_PENDING, ~0ull); // retires without results or children
            ++n_tasks;
            n_visits += n;
            n_executed += done;
        }
        return;
    }

    emit_task(p, nd, counts, q, depth, n, done, thr, lane, n_tasks, n_visits, n_executed);
}

// H = the hierarchy's hash function count (one value for all IBFs, as in the reference's build).
// HIBF_QUERY_MIN_BLOCKS blocks of eight warps per SM bound the register budget (2: 128 registers per thread,
// measured fastest: the kernel is limited by the memory system's random-access rate, not by occupancy).
#ifndef HIBF_QUERY_MIN_BLOCKS
#    define HIBF_QUERY_MIN_BLOCKS 2
#endif
template <int H, int V>
__global__ void __launch_bounds__(256, HIBF_QUERY_MIN_BLOCKS) k_query(query_params p)
{
    extern __shared__ uint32_t s_counts[];
    int const lane = threadIdx.x & 31;
    uint32_t * counts = s_counts + (threadIdx.x >> 5) * p.counters_per_warp;
    if (p.self_init)
    {
        if (threadIdx.x == 0)
        {
            p.ctrl[C_HEAD] = 0;
            p.ctrl[C_TAIL] = 0;
            p.ctrl[C_PENDING] = p.n_queries;
            __threadfence();
        }
        __syncthreads();
    }
    unsigned long long n_tasks = 0, n_visits = 0, n_executed = 0;
    // Streamed inputs: roots are claimed through C_HEAD and children through C_CHILD, children first whenever more
    // than a grid's worth of warps of them are queued.  The copy paces the roots, so children run as they appear
    // instead of piling up behind the last chunk; a warp whose claimed root (`held`) has not arrived yet runs queued
    // children meanwhile.
    // The streamed-mode state of each warp lives in shared memory, off the registers of the counting code.
    __shared__ unsigned long long s_held[8], s_held_since[8];
    __shared__ unsigned int s_held_need[8], s_backoff[8], s_polls[8];
    int const w = threadIdx.x >> 5;
    if (lane == 0)
    {
        s_held[w] = kEmpty;
        s_held_since[w] = 0;
        s_held_need[w] = s_backoff[w] = s_polls[w] = 0;
    }
    __syncwarp();
    if (p.level)
    {
        // level schedule: claim the level's tasks in order; no task of this launch waits for another
        uint64_t const n_level = p.in_tasks ? *p.in_count : p.n_queries;
        for (;;)
        {
            unsigned long long idx = 0;
            if (lane == 0)
                idx = atomicAdd(p.ctrl + C_HEAD, 1ull);
            idx = __shfl_sync(kFullMask, idx, 0);
            if (idx >= n_level)
                break;
            unsigned long long task;
            if (p.in_tasks)
            {
                task = p.in_tasks[idx];
            }
            else
            {
                uint64_t const q = p.order ? p.order[idx] : idx;
                if (q >= p.n_queries)
                {
                    if (lane == 0)
                        atomicOr(p.ctrl + C_ERROR, E_ORDER);
                    continue;
                }
                bool ok = true;
                if (p.arrived && lane == 0)
                    ok = wait_arrival(p, q);
                if (!__shfl_sync(kFullMask, static_cast<int>(ok), 0))
                    break; // E_TIMEOUT is set
                task = make_task(q, 0u, 0u);
            }
            process_task<H, V>(p, task, counts, lane, n_tasks, n_visits, n_executed);
        }
    }
    for (; !p.level;)
    {
        unsigned long long task = kEmpty;
        unsigned long long held = s_held[w];
        if (held != kEmpty)
        {
            int action = 0; // 0 wait, 1 run the held root, 2 run a stolen child, 3 give up
            unsigned long long slot = 0;
            if (lane == 0)
            {
                if (arrival_count(p) >= s_held_need[w])
                {
                    __threadfence();
                    action = 1;
                }
                else
                {
                    unsigned long long const reserve = static_cast<unsigned long long>(gridDim.x) * (blockDim.x >> 5);
                    slot = (s_polls[w]++ & 3u) == 0 ? try_claim_child(p, reserve) : kEmpty;
                    if (slot != kEmpty)
                    {
                        action = 2;
                    }
                    else if (s_held_since[w] == 0)
                    {
                        s_held_since[w] = globaltimer_ns();
                    }
                    else if (globaltimer_ns() - s_held_since[w] > p.arrive_limit_ns)
                    {
                        atomicOr(p.ctrl + C_ERROR, E_TIMEOUT);
                        action = 3;
                    }
                    if (action == 0)
                    {
                        unsigned int const b = s_backoff[w];
                        s_backoff[w] = b ? min(2u * b, 16384u) : 1024u;
                        __nanosleep(s_backoff[w]);
                    }
                    else
                    {
                        s_backoff[w] = 0;
                        s_polls[w] = 0;
                    }
                }
                if (action == 1)
                    s_held[w] = kEmpty;
            }
            action = __shfl_sync(kFullMask, action, 0);
            __syncwarp();
            if (action == 3)
                break;
            if (action == 0)
                continue;
            if (action == 1)
            {
                task = held;
                held = kEmpty;
            }
            else
            {
                if (lane == 0)
                    task = wait_for_task(p, slot); // a reserved slot: its writer is storing it
                task = __shfl_sync(kFullMask, task, 0);
                if (task == kEmpty)
                    break;
            }
        }
        else
        {
            if (p.arrived)
            {
                unsigned long long slot = kEmpty;
                if (lane == 0)
                    slot = try_claim_child(p, static_cast<unsigned long long>(gridDim.x) * (blockDim.x >> 5));
                slot = __shfl_sync(kFullMask, slot, 0);
                if (slot != kEmpty)
                {
                    if (lane == 0)
                        task = wait_for_task(p, slot);
                    task = __shfl_sync(kFullMask, task, 0);
                    if (task == kEmpty)
                        break;
                }
            }
        }
        if (task == kEmpty && held == kEmpty)
        {
            unsigned long long idx = 0;
            if (lane == 0)
                idx = atomicAdd(p.ctrl + C_HEAD, 1ull);
            idx = __shfl_sync(kFullMask, idx, 0);
            if (idx < p.n_queries)
            {
                uint64_t const q = p.order ? p.order[idx] : idx;
                if (q >= p.n_queries)
                {
                    if (lane == 0)
                    {
                        atomicOr(p.ctrl + C_ERROR, E_ORDER);
                        __threadfence();
                        atomicAdd(p.ctrl + C_PENDING, ~0ull);
                    }
                    continue;
                }
                if (p.arrived)
                {
                    if (lane == 0)
                    {
                        s_held[w] = make_task(q, 0u, 0u);
                        s_held_need[w] = arrival_needed(p, q);
                        s_held_since[w] = 0;
                    }
                    __syncwarp();
                    continue;
                }
                task = make_task(q, 0u, 0u);
            }
            else
            {
                unsigned long long slot = idx - p.n_queries;
                if (p.arrived)
                {
                    if (lane == 0)
                        slot = atomicAdd(p.ctrl + C_CHILD, 1ull);
                    slot = __shfl_sync(kFullMask, slot, 0);
                }
                if (slot >= p.task_cap)
                    break;
                if (lane == 0)
                    task = wait_for_task(p, slot);
                task = __shfl_sync(kFullMask, task, 0);
                if (task == kEmpty)
                    break;
            }
        }
        process_task<H, V>(p, task, counts, lane, n_tasks, n_visits, n_executed);
    }
    if (lane == 0 && n_tasks)
    {
        atomicAdd(p.stats + 0, n_tasks);
        atomicAdd(p.stats + 1, n_visits);
        atomicAdd(p.stats + 2, n_executed);
    }
}

// Latency mode: a whole block (eight warps) works on one task.  Warp w counts its eighth of the task's values into
// its own shared counters, the block adds the eight count arrays, warp 0 scans and emits.  A task then takes about an
// eighth of the time, which shortens a batch whose tasks are fewer than the GPU's warps (the chain root -> child ->
// grandchild of its slowest query bounds it).  No early exit: a slice's counts do not bound the task's.
constexpr unsigned long long kSkipTask = kEmpty - 1u; // an order entry that was not a query index

template <int H>
__global__ void __launch_bounds__(256, HIBF_QUERY_MIN_BLOCKS) k_query_blk(query_params p)
{
    extern __shared__ uint32_t s_counts[];
    __shared__ unsigned long long s_task;
    int const lane = threadIdx.x & 31;
    int const warp = threadIdx.x >> 5;
    int const nwarps = blockDim.x >> 5;
    uint32_t * counts = s_counts + warp * p.counters_per_warp;
    if (p.self_init)
    {
        if (threadIdx.x == 0)
        {
            p.ctrl[C_HEAD] = 0;
            p.ctrl[C_TAIL] = 0;
            p.ctrl[C_PENDING] = p.n_queries;
            __threadfence();
        }
        __syncthreads();
    }
    unsigned long long n_tasks = 0, n_visits = 0, n_executed = 0;
    for (;;)
    {
        if (threadIdx.x == 0)
        {
            unsigned long long const idx = atomicAdd(p.ctrl + C_HEAD, 1ull);
            unsigned long long task;
            if (idx < p.n_queries)
            {
                uint64_t const q = p.order ? p.order[idx] : idx;
                if (q >= p.n_queries)
                {
                    atomicOr(p.ctrl + C_ERROR, E_ORDER);
                    __threadfence();
                    atomicAdd(p.ctrl + C_PENDING, ~0ull);
                    task = kSkipTask;
                }
                else
                {
                    task = !p.arrived || wait_arrival(p, q) ? make_task(q, 0u, 0u) : kEmpty;
                }
            }
            else
            {
                unsigned long long const slot = idx - p.n_queries;
                task = slot >= p.task_cap ? kEmpty : wait_for_task(p, slot);
            }
            s_task = task;
        }
        __syncthreads();
        unsigned long long const task = s_task;
        if (task == kEmpty)
            break;
        if (task == kSkipTask)
        {
            __syncthreads();
            continue;
        }
        uint64_t const q = task >> 32;
        uint32_t const depth = static_cast<uint32_t>(task >> kNodeBits) & 63u;
        if (q >= p.n_queries || (static_cast<uint32_t>(task) & kNodeMask) >= p.n_nodes)
        {
            if (threadIdx.x == 0)
            {
                atomicOr(p.ctrl + C_ERROR, E_TASK);
                __threadfence();
                atomicAdd(p.ctrl + C_PENDING, ~0ull);
            }
            __syncthreads();
            continue;
        }
        dev_node const nd = p.nodes[static_cast<uint32_t>(task) & kNodeMask];
        uint64_t const b0 = p.qoff[q];
        uint64_t const n = p.qoff[q + 1] - b0;
        uint32_t const ncount = nd.bin_words > 32 ? 64u * nd.bin_words : (64u << nd.lpv_log2);
        for (uint32_t i = lane; i < ncount; i += 32)
            counts[i] = 0;
        __syncwarp();
        row_params const rp{nd.words, nd.bin_size, nd.row_words, nd.bin_words, nd.hash_shift, nd.hash_funs};
        uint64_t const per = (n + nwarps - 1) / nwarps;
        uint64_t const lo = min(n, static_cast<uint64_t>(warp) * per);
        uint64_t const hi = min(n, lo + per);
        if (hi > lo)
            count_variant<H, 0>(rp, nd.lpv_log2, p.values + b0 + lo, hi - lo, counts, lane, nullptr);
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < ncount; i += blockDim.x)
        {
            uint32_t sum = s_counts[i];
            for (int w = 1; w < nwarps; ++w)
                sum += s_counts[w * p.counters_per_warp + i];
            s_counts[i] = sum;
        }
        __syncthreads();
        if (warp == 0)
            emit_task(p, nd, s_counts, q, depth, n, n, p.thr[q], lane, n_tasks, n_visits, n_executed);
        __syncthreads(); // the counters and s_task are reused by the next task
    }
    if (threadIdx.x == 0 && n_tasks)
    {
        atomicAdd(p.stats + 0, n_tasks);
        atomicAdd(p.stats + 1, n_visits);
        atomicAdd(p.stats + 2, n_executed);
    }
}

// ---------------------------------------------------------------------------------------------------------------
// Features of the learned scheduler (cost_model.cu): cheap per-query inputs from which it predicts a query's work.
// One warp per query counts the query's first `probe` values in the root IBF, then summarises the root's segments:
//   f0 = log2(1 + n) / 16          f1 = min(t / n, 2)               f2 = best segment count / probe values
//   f3 = min(#segments reaching t/n of the probe, 8) / 8               f4 = the same for merged bins only
//   f5 = probe values / probe
// ---------------------------------------------------------------------------------------------------------------
constexpr int kCostFeatures = 6;
using features_kernel_t = void (*)(query_params, uint32_t, float *);

template <int H>
__global__ void __launch_bounds__(256) k_query_features(query_params p, uint32_t probe, float * __restrict__ out)
{
    extern __shared__ uint32_t s_counts[];
    int const lane = threadIdx.x & 31;
    uint32_t * counts = s_counts + (threadIdx.x >> 5) * p.counters_per_warp;
    uint64_t const warp = (blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x) >> 5;
    uint64_t const nwarps = (static_cast<uint64_t>(gridDim.x) * blockDim.x) >> 5;
    dev_node const nd = p.nodes[0];
    row_params const rp{nd.words, nd.bin_size, nd.row_words, nd.bin_words, nd.hash_shift, nd.hash_funs};
    uint32_t const ncount = nd.bin_words > 32 ? 64u * nd.bin_words : (64u << nd.lpv_log2);
    uint2 const * d = p.descs + nd.desc_offset;
    for (uint64_t q = warp; q < p.n_queries; q += nwarps)
    {
        uint64_t const b0 = p.qoff[q];
        uint64_t const n = p.qoff[q + 1] - b0;
        uint64_t const m = n < probe ? n : probe;
        for (uint32_t i = lane; i < ncount; i += 32)
            counts[i] = 0;
        __syncwarp();
        if (m)
            count_variant<H, 0>(rp, nd.lpv_log2, p.values + b0, m, counts, lane, nullptr);
        __syncwarp();
        double const rate = n ? static_cast<double>(p.thr[q]) / static_cast<double>(n) : 0.0;
        unsigned long long const need = static_cast<unsigned long long>(ceil(rate * static_cast<double>(m)));
        unsigned long long best = 0;
        uint32_t pass_seg = 0, pass_merged = 0;
        unsigned long long carry = 0;
        for (uint32_t c = 0; c < nd.bins; c += 32)
        {
            uint32_t const b = c + lane;
            bool const valid = b < nd.bins;
            uint2 const ds = valid ? d[b] : make_uint2(0u, 0u);
            unsigned long long x = valid ? static_cast<unsigned long long>(counts[b]) : 0ull;
            bool f = valid && (ds.y & F_HEAD);
            if (lane == 0 && !f)
                x += carry;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1)
            {
                unsigned long long const y = __shfl_up_sync(kFullMask, x, o);
                int const fy = __shfl_up_sync(kFullMask, static_cast<int>(f), o);
                if (lane >= o)
                {
                    if (!f)
                        x += y;
                    f = f || fy;
                }
            }
            bool const ends = valid && (ds.y & (F_RUN_END | F_MERGED));
            bool const pass = ends && m && x >= need;
            if (ends && x > best)
                best = x;
            pass_seg += __popc(__ballot_sync(kFullMask, pass));
            pass_merged += __popc(__ballot_sync(kFullMask, pass && (ds.y & F_MERGED)));
            unsigned long long const lastx = __shfl_sync(kFullMask, x, 31);
            uint32_t const lastf = __shfl_sync(kFullMask, ds.y, 31);
            carry = (lastf & (F_MERGED | F_RUN_END)) ? 0ull : lastx;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
        {
            unsigned long long const y = __shfl_xor_sync(kFullMask, best, o);
            best = y > best ? y : best;
        }
        if (lane == 0)
        {
            float * f = out + q * kCostFeatures;
            f[0] = log2f(1.0f + static_cast<float>(n)) / 16.0f;
            f[1] = static_cast<float>(rate < 2.0 ? rate : 2.0);
            f[2] = m ? static_cast<float>(best) / static_cast<float>(m) : 0.0f;
            f[3] = static_cast<float>(pass_seg < 8u ? pass_seg : 8u) / 8.0f;
            f[4] = static_cast<float>(pass_merged < 8u ? pass_merged : 8u) / 8.0f;
            f[5] = probe ? static_cast<float>(m) / static_cast<float>(probe) : 0.0f;
        }
        __syncwarp();
    }
}

// The kernel of variant v (0 <= v < kQueryVariants; H > 3 has the default variant only).
template <int H>
query_kernel_t query_kernel_variant(int v)
{
    if constexpr (H > 3)
    {
        (void)v;
        return k_query<H, 0>;
    }
    else
    {
        switch (v)
        {
        case 1:
            return k_query<H, 1>;
        case 2:
            return k_query<H, 2>;
        case 3:
            return k_query<H, 3>;
        case 4:
            return k_query<H, 4>;
        case 5:
            return k_query<H, 5>;
        default:
            return k_query<H, 0>;
        }
    }
}

// Defined in query_h1.cu .. query_h5.cu.
query_kernel_t query_kernel_h1(int v);
query_kernel_t query_kernel_h2(int v);
query_kernel_t query_kernel_h3(int v);
query_kernel_t query_kernel_h4(int v);
query_kernel_t query_kernel_h5(int v);
query_kernel_t query_block_kernel_h1();
query_kernel_t query_block_kernel_h2();
query_kernel_t query_block_kernel_h3();
query_kernel_t query_block_kernel_h4();
query_kernel_t query_block_kernel_h5();
features_kernel_t features_kernel_h1();
features_kernel_t features_kernel_h2();
features_kernel_t features_kernel_h3();
features_kernel_t features_kernel_h4();
features_kernel_t features_kernel_h5();

inline query_kernel_t query_block_kernel(uint32_t h)
{
    switch (h)
    {
    case 1:
        return query_block_kernel_h1();
    case 2:
        return query_block_kernel_h2();
    case 3:
        return query_block_kernel_h3();
    case 4:
        return query_block_kernel_h4();
    default:
        return query_block_kernel_h5();
    }
}

inline features_kernel_t features_kernel(uint32_t h)
{
    switch (h)
    {
    case 1:
        return features_kernel_h1();
    case 2:
        return features_kernel_h2();
    case 3:
        return features_kernel_h3();
    case 4:
        return features_kernel_h4();
    default:
        return features_kernel_h5();
    }
}

inline query_kernel_t query_kernel(uint32_t h, int v)
{
    switch (h)
    {
    case 1:
        return query_kernel_h1(v);
    case 2:
        return query_kernel_h2(v);
    case 3:
        return query_kernel_h3(v);
    case 4:
        return query_kernel_h4(v);
    default:
        return query_kernel_h5(v);
    }
}

} // namespace hibf_gb300
