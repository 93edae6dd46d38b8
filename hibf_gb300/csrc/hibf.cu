// hibf.cu -- hierarchical interleaved Bloom filter on the device: per-IBF bit stores and tables, the persistent
// (query, IBF) work-queue kernel, the result compaction passes, agents and their C-ABI entry points.
//
// Reference interface: seqan::hibf::hierarchical_interleaved_bloom_filter
// (include/hibf/hierarchical_interleaved_bloom_filter.hpp, src/hierarchical_interleaved_bloom_filter.cpp).
//
// The query kernel itself (semantics, work queue, tuning variants, early exit) is in query.cuh; this file holds the
// stores, the result compaction passes, agents (host batches, streamed when large: see host_batch), the autotuner
// and their C-ABI entry points.

#include <algorithm>
#include <atomic>
#include <cstring>
#include <exception>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/hibf_gb300_synthetic.h"
#include "common.hpp"
#include "count.cuh"
#include "device.cuh"
#include "hibf_internal.cuh"
#include "query.cuh"
#include "archive.hpp"

namespace hibf_gb300
{

void set_last_error(std::string msg);

namespace
{


__global__ void k_init_ctrl(unsigned long long * ctrl, unsigned long long * stats, uint64_t n_queries)
{
    if (threadIdx.x < C_WORDS)
        ctrl[threadIdx.x] = threadIdx.x == C_PENDING ? n_queries : 0ull;
    if (threadIdx.x < kStats)
        stats[threadIdx.x] = 0;
}

// ---- level schedule: the tasks one level appended (tasks[0, ctrl[C_TAIL])), grouped by IBF for the next level ----
// Per IBF the number of queued tasks (a block-local histogram in shared memory when the IBFs fit, else global atomics).
__global__ void k_level_hist(unsigned long long const * __restrict__ tasks, unsigned long long const * ctrl,
                             uint64_t task_cap, unsigned int * hist, uint32_t n_ibfs, int use_smem)
{
    extern __shared__ unsigned int s_hist[];
    uint64_t const n = min(static_cast<uint64_t>(ctrl[C_TAIL]), task_cap);
    if (use_smem)
    {
        for (uint32_t i = threadIdx.x; i < n_ibfs; i += blockDim.x)
            s_hist[i] = 0;
        __syncthreads();
    }
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    {
        uint32_t const k = static_cast<uint32_t>(tasks[i]) & kNodeMask;
        if (k < n_ibfs)
            atomicAdd(use_smem ? s_hist + k : hist + k, 1u);
    }
    if (use_smem)
    {
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < n_ibfs; i += blockDim.x)
            if (s_hist[i])
                atomicAdd(hist + i, s_hist[i]);
    }
}

// One block: exclusive scan of the histogram into per-IBF write cursors; the level's task count moves to *count and
// the claim and append counters restart for the next level.
__global__ void k_level_scan(unsigned int * hist, uint32_t n_ibfs, unsigned long long * ctrl, uint64_t task_cap,
                             unsigned long long * count)
{
    __shared__ unsigned int s_warp[32];
    __shared__ unsigned int s_carry;
    int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0)
        s_carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < n_ibfs; base += blockDim.x)
    {
        uint32_t const i = base + threadIdx.x;
        unsigned int const x = i < n_ibfs ? hist[i] : 0u;
        unsigned int y = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            unsigned int const t = __shfl_up_sync(kFullMask, y, o);
            if (lane >= o)
                y += t;
        }
        if (lane == 31)
            s_warp[warp] = y;
        __syncthreads();
        if (warp == 0)
        {
            unsigned int z = lane < static_cast<int>(blockDim.x >> 5) ? s_warp[lane] : 0u;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1)
            {
                unsigned int const t = __shfl_up_sync(kFullMask, z, o);
                if (lane >= o)
                    z += t;
            }
            s_warp[lane] = z;
        }
        __syncthreads();
        unsigned int const excl = s_carry + (warp ? s_warp[warp - 1] : 0u) + y - x;
        if (i < n_ibfs)
            hist[i] = excl;
        __syncthreads();
        if (threadIdx.x == 0)
            s_carry += s_warp[(blockDim.x >> 5) - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0)
    {
        *count = min(static_cast<uint64_t>(ctrl[C_TAIL]), task_cap);
        ctrl[C_TAIL] = 0;
        ctrl[C_HEAD] = 0;
    }
}

// Places every task of the level at its IBF's cursor (the order within one IBF is the atomics' order; results do not
// depend on the order in which tasks run).
__global__ void k_level_scatter(unsigned long long const * __restrict__ tasks, unsigned long long const * count,
                                unsigned int * cursor, unsigned long long * __restrict__ sorted, uint32_t n_ibfs)
{
    uint64_t const n = *count;
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    {
        unsigned long long const t = tasks[i];
        uint32_t const k = static_cast<uint32_t>(t) & kNodeMask;
        if (k < n_ibfs)
            sorted[atomicAdd(cursor + k, 1u)] = t;
    }
}

// ---- exclusive scan of the per-query result counts -> result offsets (n + 1 entries) ----
constexpr int kScanBlock = 1024;

__device__ __forceinline__ unsigned long long warp_incl_scan(unsigned long long x, int lane)
{
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        unsigned long long const y = __shfl_up_sync(kFullMask, x, o);
        if (lane >= o)
            x += y;
    }
    return x;
}

__global__ void __launch_bounds__(kScanBlock) k_scan_local(unsigned int const * __restrict__ in, uint64_t n,
                                                          unsigned long long * __restrict__ out,
                                                          unsigned long long * __restrict__ block_sums)
{
    __shared__ unsigned long long warp_sums[32];
    uint64_t const i = blockIdx.x * static_cast<uint64_t>(kScanBlock) + threadIdx.x;
    int const lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned long long const v = i < n ? in[i] : 0ull;
    unsigned long long x = warp_incl_scan(v, lane);
    if (lane == 31)
        warp_sums[w] = x;
    __syncthreads();
    if (w == 0)
    {
        unsigned long long s = warp_sums[lane];
        s = warp_incl_scan(s, lane);
        warp_sums[lane] = s;
    }
    __syncthreads();
    if (w > 0)
        x += warp_sums[w - 1];
    if (i < n)
        out[i] = x - v; // exclusive
    if (threadIdx.x == kScanBlock - 1)
        block_sums[blockIdx.x] = x;
}

__global__ void __launch_bounds__(kScanBlock) k_scan_sums(unsigned long long * sums, uint64_t nb)
{
    __shared__ unsigned long long warp_sums[32];
    __shared__ unsigned long long carry;
    int const lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0)
        carry = 0;
    __syncthreads();
    for (uint64_t base = 0; base < nb; base += kScanBlock)
    {
        uint64_t const i = base + threadIdx.x;
        unsigned long long const v = i < nb ? sums[i] : 0ull;
        unsigned long long x = warp_incl_scan(v, lane);
        if (lane == 31)
            warp_sums[w] = x;
        __syncthreads();
        if (w == 0)
            warp_sums[lane] = warp_incl_scan(warp_sums[lane], lane);
        __syncthreads();
        if (w > 0)
            x += warp_sums[w - 1];
        unsigned long long const c = carry;
        if (i < nb)
            sums[i] = c + x - v; // exclusive
        __syncthreads();
        if (threadIdx.x == kScanBlock - 1)
            carry = c + x;
        __syncthreads();
    }
    if (threadIdx.x == 0)
        sums[nb] = carry;
}

__global__ void k_scan_add(unsigned long long * out, uint64_t n, unsigned long long const * sums, uint64_t nb)
{
    uint64_t const i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
    if (i < n)
        out[i] += sums[i / kScanBlock];
    if (i == 0)
        out[n] = sums[nb];
}

// ---- scatter records into per-query segments ----
__global__ void k_scatter(unsigned long long const * __restrict__ ctrl, uint32_t const * __restrict__ rec_q,
                          uint32_t const * __restrict__ rec_ub, unsigned long long const * __restrict__ rec_cnt,
                          uint64_t rec_cap, unsigned long long const * __restrict__ roff,
                          unsigned int * __restrict__ cursor, uint64_t * __restrict__ out_ids,
                          uint64_t * __restrict__ out_cnt)
{
    if (ctrl[C_ERROR] & (E_OVERFLOW_REC | E_OVERFLOW_TASK))
        return; // offsets describe records that were not stored; the batch reports OVERFLOW
    uint64_t n = ctrl[C_NREC];
    if (n > rec_cap)
        n = rec_cap;
    for (uint64_t r = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; r < n;
         r += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    {
        uint32_t const q = rec_q[r];
        uint64_t const pos = roff[q] + atomicAdd(cursor + q, 1u);
        out_ids[pos] = rec_ub[r];
        out_cnt[pos] = rec_cnt[r];
    }
}

// ---- sort every query's segment by user bin id ----
constexpr uint32_t kSmallSegment = 32;
constexpr uint32_t kSmemSegment = 2048;

__global__ void k_sort_small(unsigned long long const * __restrict__ roff, uint64_t nq, uint64_t * ids,
                             uint64_t * cnt, uint32_t * large, unsigned long long * ctrl)
{
    if (ctrl[C_ERROR] & (E_OVERFLOW_REC | E_OVERFLOW_TASK))
        return;
    for (uint64_t q = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; q < nq;
         q += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    {
        uint64_t const b = roff[q], e = roff[q + 1];
        uint64_t const len = e - b;
        if (len <= 1)
            continue;
        if (len > kSmallSegment)
        {
            unsigned long long const slot = atomicAdd(ctrl + C_NLARGE, 1ull);
            large[slot] = static_cast<uint32_t>(q);
            continue;
        }
        for (uint64_t i = b + 1; i < e; ++i)
        {
            uint64_t const ki = ids[i], ci = cnt[i];
            uint64_t jx = i;
            while (jx > b && ids[jx - 1] > ki)
            {
                ids[jx] = ids[jx - 1];
                cnt[jx] = cnt[jx - 1];
                --jx;
            }
            ids[jx] = ki;
            cnt[jx] = ci;
        }
    }
}

// Bitonic sort of one segment with only ascending comparators (the "flip" form: the first exchange of every merge
// pairs i with its mirror in the block, the rest are half-cleaners).  Positions >= len are virtual +infinity and,
// being the larger element of every comparator they take part in, never move, so any length works.  The segment is
// staged in shared memory up to kSmemSegment elements and sorted in place in global memory beyond.
__device__ __forceinline__ void cmp_asc(uint64_t * kid, uint64_t * kcn, uint64_t i, uint64_t l, uint64_t len)
{
    if (l >= len)
        return;
    if (kid[i] > kid[l])
    {
        uint64_t t = kid[i];
        kid[i] = kid[l];
        kid[l] = t;
        t = kcn[i];
        kcn[i] = kcn[l];
        kcn[l] = t;
    }
}

__global__ void k_sort_large(unsigned long long const * __restrict__ roff, uint32_t const * __restrict__ large,
                             unsigned long long const * __restrict__ ctrl, uint64_t * ids, uint64_t * cnt)
{
    __shared__ uint64_t s_ids[kSmemSegment];
    __shared__ uint64_t s_cnt[kSmemSegment];
    if (ctrl[C_ERROR] & (E_OVERFLOW_REC | E_OVERFLOW_TASK))
        return;
    unsigned long long const nl = ctrl[C_NLARGE];
    for (unsigned long long li = blockIdx.x; li < nl; li += gridDim.x)
    {
        uint32_t const q = large[li];
        uint64_t const b = roff[q];
        uint64_t const len = roff[q + 1] - b;
        uint64_t P = 1;
        while (P < len)
            P <<= 1;
        bool const in_smem = len <= kSmemSegment;
        uint64_t * kid = in_smem ? s_ids : ids + b;
        uint64_t * kcn = in_smem ? s_cnt : cnt + b;
        if (in_smem)
        {
            for (uint64_t i = threadIdx.x; i < len; i += blockDim.x)
            {
                s_ids[i] = ids[b + i];
                s_cnt[i] = cnt[b + i];
            }
        }
        __syncthreads();
        for (uint64_t k = 2; k <= P; k <<= 1)
        {
            for (uint64_t i = threadIdx.x; i < P; i += blockDim.x)
            {
                uint64_t const l = i ^ (k - 1);
                if (l > i && i < len)
                    cmp_asc(kid, kcn, i, l, len);
            }
            __syncthreads();
            for (uint64_t jj = k >> 2; jj > 0; jj >>= 1)
            {
                for (uint64_t i = threadIdx.x; i < P; i += blockDim.x)
                {
                    uint64_t const l = i ^ jj;
                    if (l > i && i < len)
                        cmp_asc(kid, kcn, i, l, len);
                }
                __syncthreads();
            }
        }
        if (in_smem)
        {
            for (uint64_t i = threadIdx.x; i < len; i += blockDim.x)
            {
                ids[b + i] = s_ids[i];
                cnt[b + i] = s_cnt[i];
            }
        }
        __syncthreads();
    }
}

__global__ void k_narrow(unsigned long long const * __restrict__ roff, uint64_t nq, uint64_t const * __restrict__ in,
                         int width, void * out, unsigned long long const * __restrict__ ctrl)
{
    if (ctrl[C_ERROR] & (E_OVERFLOW_REC | E_OVERFLOW_TASK))
        return;
    uint64_t const n = roff[nq];
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    {
        uint64_t const v = in[i];
        switch (width)
        {
        case 1:
            static_cast<uint8_t *>(out)[i] = static_cast<uint8_t>(v);
            break;
        case 2:
            static_cast<uint16_t *>(out)[i] = static_cast<uint16_t>(v);
            break;
        case 4:
            static_cast<uint32_t *>(out)[i] = static_cast<uint32_t>(v);
            break;
        default:
            static_cast<uint64_t *>(out)[i] = v;
        }
    }
}

// emplace into an IBF (same as the single-level kernel, repeated here to keep the translation units independent).
__global__ void k_hibf_emplace(uint64_t * __restrict__ words, uint64_t bin_size, uint32_t row_words, uint32_t shift,
                               uint32_t h, uint64_t const * __restrict__ values, uint64_t const * __restrict__ bins,
                               uint64_t n, uint64_t bin, uint64_t n_bins)
{
    uint64_t const stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n; i += stride)
    {
        uint64_t const v = values[i];
        uint64_t const b = bins ? bins[i] : bin;
        if (b >= n_bins)
            continue; // out-of-range device-supplied bin: skipped (never written outside the IBF's row)
        unsigned long long const bit = 1ull << (b & 63u);
        uint64_t const wofs = b >> 6;
        for (uint32_t k = 0; k < h; ++k)
        {
            uint64_t const r = hash_row(v, c_hash_seeds[k], shift, bin_size);
            atomicOr(reinterpret_cast<unsigned long long *>(words + r * row_words + wofs), bit);
        }
    }
}

unsigned grid_cap(uint64_t work, unsigned block, unsigned per_sm = 16)
{
    uint64_t const want = (work + block - 1) / block;
    uint64_t const cap = static_cast<uint64_t>(sm_count()) * per_sm;
    return static_cast<unsigned>(std::max<uint64_t>(1, std::min(want, cap)));
}

} // namespace
} // namespace hibf_gb300

using namespace hibf_gb300;

struct hibf_gpu_agent
{
    hibf_gpu_hibf * h{};
    cudaStream_t own{};
    cudaStream_t stream{};
    cudaEvent_t ev_k0{}, ev_k1{}; // around the persistent query kernel of the last batch
    cudaGraphExec_t graph{};      // captured launch sequence of one batch (hibf_gpu_agent_capture_batch_d)
    int status{HIBF_GPU_OK};
    uint64_t last_tasks{}, last_visits{}, last_executed{};
    uint64_t cap_queries{}, cap_tasks{}, cap_results{};
    hibf_gpu_tuning tune{};                // schedule of the persistent kernel
    int variant{0};                        // kernel variant of `tune`
    int child_variant{0};                  // kernel variant of the levels below the root (level schedule)
    int max_blocks[kQueryVariants]{};      // resident 256-thread blocks per SM of each variant
    int max_blocks_blk{};                  // and of the block-per-task kernel
    uint32_t const * order{};              // claim order of the root tasks (device; null = query order)
    uint64_t order_n{};                    // its length: batches must have exactly this many queries
    unsigned long long * qwork{};          // executed value visits per query (device; null = not recorded)
    uint64_t qwork_n{};                    // its length: batches may have at most this many queries
    // device workspace
    dbuf ctrl, stats, tasks, rec_q, rec_ub, rec_cnt, qcount, cursor, roff, bsum, out_ids, out_cnt, out_cntw, large;
    // level schedule: a level's tasks grouped by IBF, the per-IBF histogram / cursors, the level's task count; an
    // event after each level of the last batch (timing)
    dbuf lvl_tasks, lvl_hist, lvl_count;
    // level schedule: each level's tasks, value visits and executed value visits (kStats words per level)
    dbuf lvl_stats;
    hbuf h_lvl_stats;
    std::vector<uint64_t> last_level_stats;
    std::vector<cudaEvent_t> ev_lvl;
    uint32_t last_levels{};
    bool force_queue{}; // set for the duration of a streamed host batch
    bool host_read{true}; // host batches in mapped page-locked memory are read in place (hibf_gpu_agent_set_host_read)
    bool last_in_place{}; // the last host batch was read in place
    // set for the duration of an in-place host batch: where its roots stage the values they read (device) and how
    // many of each query's values they staged
    uint64_t * stage_values{};
    uint32_t * stage_counts{};
    dbuf staged;
    // host-call staging
    dbuf in_values, in_qoff, in_thr;
    // streamed host batches: value chunks copied on copy_stream while the kernel answers the arrived ones
    cudaStream_t copy_stream{};
    cudaEvent_t ev_ready{}, ev_copied{};
    dbuf arrived, arrive_first;
    hbuf h_arrive_first, h_arrive_counts;
    unsigned int const * arrive{};  // set for the duration of one streamed host batch
    uint32_t arrive_chunks{};
    uint64_t arrive_limit_ns{};
    uint32_t last_chunks{}; // chunks of the last host batch (0: not streamed)
    // timeline of the last host batch: its start, each value chunk's copy done, results back (timing events)
    cudaEvent_t tl_t0{}, tl_done{};
    std::vector<cudaEvent_t> tl_chunk;
    uint32_t tl_n{};
    hbuf h_roff, h_ids, h_cnt, h_ctrl, h_stats;
    std::vector<uint64_t> single_ids;
    std::vector<uint8_t> dense;
    std::vector<uint64_t> thr_tmp, qoff_tmp;
};

namespace
{

void ensure_capacity(hibf_gpu_agent * a, uint64_t nq, uint64_t tasks, uint64_t results)
{
    if (nq > a->cap_queries)
    {
        a->qcount.ensure(nq * 4);
        a->cursor.ensure(nq * 4);
        a->roff.ensure((nq + 1) * 8);
        a->bsum.ensure(((nq + kScanBlock - 1) / kScanBlock + 1) * 8);
        a->large.ensure(nq * 4);
        a->cap_queries = nq;
    }
    if (tasks > a->cap_tasks)
    {
        a->tasks.ensure(tasks * 8);
        a->cap_tasks = tasks;
    }
    if (a->tune.schedule == HIBF_GPU_SCHEDULE_LEVELS) // no-ops once large enough
    {
        a->lvl_tasks.ensure(a->cap_tasks * 8);
        a->lvl_hist.ensure(a->h->n_ibfs * 4);
        a->lvl_count.ensure(8);
        a->lvl_stats.ensure((a->h->max_depth + 1) * kStats * 8);
        a->h_lvl_stats.ensure((a->h->max_depth + 1) * kStats * 8);
    }
    if (results > a->cap_results)
    {
        a->rec_q.ensure(results * 4);
        a->rec_ub.ensure(results * 4);
        a->rec_cnt.ensure(results * 8);
        a->out_ids.ensure(results * 8);
        a->out_cnt.ensure(results * 8);
        a->out_cntw.ensure(results * 8);
        a->cap_results = results;
    }
}

query_params base_params(hibf_gpu_agent * a, uint64_t const * d_values, uint64_t const * d_qoff,
                         uint64_t const * d_thr, uint64_t nq, uint64_t count_mask)
{
    hibf_gpu_hibf * h = a->h;
    query_params p{};
    p.nodes = h->d_nodes.as<dev_node>();
    p.descs = h->d_descs.as<uint2>();
    p.values = d_values;
    p.qoff = d_qoff;
    p.thr = d_thr;
    p.count_mask = count_mask;
    p.n_queries = nq;
    p.n_nodes = static_cast<uint32_t>(h->n_ibfs);
    p.q_base = 0;
    p.max_depth = h->max_depth;
    p.counters_per_warp = h->counters_per_warp;
    p.tasks = a->tasks.as<unsigned long long>();
    p.task_cap = a->cap_tasks;
    p.ctrl = a->ctrl.as<unsigned long long>();
    p.rec_q = a->rec_q.as<uint32_t>();
    p.rec_ub = a->rec_ub.as<uint32_t>();
    p.rec_cnt = a->rec_cnt.as<unsigned long long>();
    p.rec_cap = a->cap_results;
    p.qcount = a->qcount.as<unsigned int>();
    p.stats = a->stats.as<unsigned long long>();
    p.wait_limit_ns = 10ull * 1000 * 1000 * 1000;
    p.self_init = 0;
    p.ee_first = a->tune.early_exit_first;
    p.ee_step = a->tune.early_exit_step;
    p.ee_stages = a->tune.early_exit_stages;
    p.ee_min = a->tune.early_exit_min;
    p.order = a->order;
    p.qwork = a->qwork;
    p.arrived = a->arrive;
    p.arrive_first = a->arrive ? a->arrive_first.as<uint64_t>() : nullptr;
    p.arrive_chunks = a->arrive_chunks;
    p.arrive_limit_ns = a->arrive_limit_ns;
    p.stage = nullptr;
    p.staged = nullptr;
    return p;
}

uint64_t mask_for(int mode, int width)
{
    int const w = mode == HIBF_GPU_QUERY_MEMBERSHIP ? 2 : width;
    return w >= 8 ? ~0ull : ((1ull << (8 * w)) - 1u);
}

size_t query_smem(hibf_gpu_hibf const * h)
{
    return static_cast<size_t>(8) * h->counters_per_warp * sizeof(uint32_t);
}

void launch_postprocess(hibf_gpu_agent * a, uint64_t nq, int mode, int width)
{
    cudaStream_t s = a->stream;
    uint64_t const nb = (nq + kScanBlock - 1) / kScanBlock;
    if (nq)
    {
        k_scan_local<<<static_cast<unsigned>(nb), kScanBlock, 0, s>>>(
            a->qcount.as<unsigned int>(), nq, a->roff.as<unsigned long long>(), a->bsum.as<unsigned long long>());
        HG_CUDA(cudaGetLastError());
    }
    k_scan_sums<<<1, kScanBlock, 0, s>>>(a->bsum.as<unsigned long long>(), nb);
    HG_CUDA(cudaGetLastError());
    k_scan_add<<<static_cast<unsigned>(std::max<uint64_t>(1, (nq + 255) / 256)), 256, 0, s>>>(
        a->roff.as<unsigned long long>(), nq, a->bsum.as<unsigned long long>(), nb);
    HG_CUDA(cudaGetLastError());
    HG_CUDA(cudaMemsetAsync(a->cursor.p, 0, std::max<uint64_t>(nq, 1) * 4, s));
    k_scatter<<<grid_cap(a->cap_results, 256, 8), 256, 0, s>>>(
        a->ctrl.as<unsigned long long>(), a->rec_q.as<uint32_t>(), a->rec_ub.as<uint32_t>(),
        a->rec_cnt.as<unsigned long long>(), a->cap_results, a->roff.as<unsigned long long>(),
        a->cursor.as<unsigned int>(), a->out_ids.as<uint64_t>(), a->out_cnt.as<uint64_t>());
    HG_CUDA(cudaGetLastError());
    k_sort_small<<<grid_cap(nq, 256, 8), 256, 0, s>>>(a->roff.as<unsigned long long>(), nq, a->out_ids.as<uint64_t>(),
                                                     a->out_cnt.as<uint64_t>(), a->large.as<uint32_t>(),
                                                     a->ctrl.as<unsigned long long>());
    HG_CUDA(cudaGetLastError());
    k_sort_large<<<static_cast<unsigned>(sm_count()), 256, 0, s>>>(
        a->roff.as<unsigned long long>(), a->large.as<uint32_t>(), a->ctrl.as<unsigned long long>(),
        a->out_ids.as<uint64_t>(), a->out_cnt.as<uint64_t>());
    HG_CUDA(cudaGetLastError());
    if (mode == HIBF_GPU_QUERY_COUNT && width != 8)
    {
        k_narrow<<<grid_cap(a->cap_results, 256, 8), 256, 0, s>>>(a->roff.as<unsigned long long>(), nq,
                                                                 a->out_cnt.as<uint64_t>(), width, a->out_cntw.p,
                                                                 a->ctrl.as<unsigned long long>());
        HG_CUDA(cudaGetLastError());
    }
}

// One persistent launch over all queries plus compaction.  Asynchronous.
void check_order_and_work(hibf_gpu_agent const * a, uint64_t nq, bool plain)
{
    if (a->order && !plain && a->order_n != nq)
        fail(HIBF_GPU_ERR_INVALID_ARG, "the claim order set on the agent has a different length than the batch");
    if (a->qwork && a->qwork_n < nq)
        fail(HIBF_GPU_ERR_INVALID_ARG, "the per-query work array set on the agent is shorter than the batch");
}

void launch_batch(hibf_gpu_agent * a, int mode, uint64_t const * d_values, uint64_t const * d_qoff,
                  uint64_t const * d_thr, uint64_t nq, int width)
{
    hibf_gpu_hibf * h = a->h;
    check_order_and_work(a, nq, false);
    cudaStream_t s = a->stream;
    k_init_ctrl<<<1, 32, 0, s>>>(a->ctrl.as<unsigned long long>(), a->stats.as<unsigned long long>(), nq);
    HG_CUDA(cudaGetLastError());
    // One decision for the whole batch.  The queue (persistent or block kernel) waits on empty-slot marks in the
    // task array, so every batch it runs starts from a fully marked array; the level schedule reads only the slots
    // a finished launch wrote.
    bool const blk = nq <= a->tune.block_queries;
    bool const levels = !blk && a->tune.schedule == HIBF_GPU_SCHEDULE_LEVELS && !a->force_queue;
    if (!levels)
        HG_CUDA(cudaMemsetAsync(a->tasks.p, 0xFF, a->cap_tasks * 8, s)); // the queue's empty-slot marks
    HG_CUDA(cudaMemsetAsync(a->qcount.p, 0, std::max<uint64_t>(nq, 1) * 4, s));
    if (a->qwork && nq)
        HG_CUDA(cudaMemsetAsync(a->qwork, 0, nq * 8, s));
    a->last_levels = 0;
    if (nq)
    {
        query_params p = base_params(a, d_values, d_qoff, d_thr, nq, mask_for(mode, width));
        p.decide = mode == HIBF_GPU_QUERY_MEMBERSHIP;
        int const fit = blk ? a->max_blocks_blk : a->max_blocks[a->variant];
        int const per_sm = a->tune.blocks_per_sm ? std::min<int>(fit, static_cast<int>(a->tune.blocks_per_sm)) : fit;
        uint64_t const full = static_cast<uint64_t>(sm_count()) * static_cast<uint64_t>(per_sm);
        // block mode: one block per query at most, so that concurrent batches (a server's slots) find room
        uint64_t const want = blk ? nq : (nq + 7) / 8;
        unsigned const grid = static_cast<unsigned>(std::max<uint64_t>(1, std::min(full, want)));
        // inside a stream capture an event record only orders work unless it is marked external; external records
        // become event-record nodes of the graph, so replays time the kernel too
        cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
        HG_CUDA(cudaStreamIsCapturing(s, &cap));
        unsigned const rec_flags = cap == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : 0u;
        HG_CUDA(cudaEventRecordWithFlags(a->ev_k0, s, rec_flags));
        if (levels)
        {
            // an in-place host batch: the roots stage the values they read, the lower levels read them from there
            p.stage = a->stage_values;
            p.staged = a->stage_counts;
            // one launch per level: the roots, then each level's appended tasks grouped by IBF
            uint64_t const stats_bytes = (h->max_depth + 1) * kStats * 8;
            if (!a->lvl_tasks.p || a->lvl_tasks.bytes < a->cap_tasks * 8 || !a->lvl_hist.p ||
                a->lvl_hist.bytes < h->n_ibfs * 4 || !a->lvl_count.p || a->lvl_stats.bytes < stats_bytes ||
                a->h_lvl_stats.bytes < stats_bytes)
                fail(HIBF_GPU_ERR_LOGIC, "level schedule buffers missing (set the tuning through set_tuning)");
            // each level counts its work into its own kStats words; read_status sums them
            HG_CUDA(cudaMemsetAsync(a->lvl_stats.p, 0, stats_bytes, s));
            unsigned long long * const lvl_stats = a->lvl_stats.as<unsigned long long>();
            while (a->ev_lvl.size() <= h->max_depth)
            {
                cudaEvent_t e{};
                HG_CUDA(cudaEventCreate(&e));
                a->ev_lvl.push_back(e);
            }
            unsigned const grid_full = static_cast<unsigned>(full);
            int const child_variant = a->child_variant;
            int const child_fit = a->max_blocks[child_variant];
            int const child_per_sm =
                a->tune.blocks_per_sm ? std::min<int>(child_fit, static_cast<int>(a->tune.blocks_per_sm)) : child_fit;
            unsigned const grid_child = static_cast<unsigned>(sm_count()) * static_cast<unsigned>(child_per_sm);
            p.level = 1;
            p.stats = lvl_stats;
            query_kernel(h->hash_count, a->variant)<<<grid_full, 256, query_smem(h), s>>>(p);
            HG_CUDA(cudaGetLastError());
            HG_CUDA(cudaEventRecordWithFlags(a->ev_lvl[0], s, rec_flags));
            uint32_t const n_ibfs = static_cast<uint32_t>(h->n_ibfs);
            int const use_smem = n_ibfs <= 12288;
            unsigned const sort_grid = static_cast<unsigned>(sm_count()) * 4u;
            for (uint32_t d = 1; d <= h->max_depth; ++d)
            {
                HG_CUDA(cudaMemsetAsync(a->lvl_hist.p, 0, n_ibfs * 4u, s));
                k_level_hist<<<sort_grid, 256, use_smem ? n_ibfs * 4u : 0u, s>>>(
                    a->tasks.as<unsigned long long>(), a->ctrl.as<unsigned long long>(), a->cap_tasks,
                    a->lvl_hist.as<unsigned int>(), n_ibfs, use_smem);
                HG_CUDA(cudaGetLastError());
                k_level_scan<<<1, 1024, 0, s>>>(a->lvl_hist.as<unsigned int>(), n_ibfs,
                                                a->ctrl.as<unsigned long long>(), a->cap_tasks,
                                                a->lvl_count.as<unsigned long long>());
                HG_CUDA(cudaGetLastError());
                k_level_scatter<<<sort_grid, 256, 0, s>>>(a->tasks.as<unsigned long long>(),
                                                          a->lvl_count.as<unsigned long long>(),
                                                          a->lvl_hist.as<unsigned int>(),
                                                          a->lvl_tasks.as<unsigned long long>(), n_ibfs);
                HG_CUDA(cudaGetLastError());
                p.in_tasks = a->lvl_tasks.as<unsigned long long>();
                p.in_count = a->lvl_count.as<unsigned long long>();
                p.stats = lvl_stats + d * kStats;
                query_kernel(h->hash_count, child_variant)<<<grid_child, 256, query_smem(h), s>>>(p);
                HG_CUDA(cudaGetLastError());
                HG_CUDA(cudaEventRecordWithFlags(a->ev_lvl[d], s, rec_flags));
            }
            a->last_levels = h->max_depth + 1;
        }
        else
        {
            (blk ? query_block_kernel(h->hash_count) : query_kernel(h->hash_count, a->variant))<<<grid, 256,
                                                                                               query_smem(h), s>>>(p);
            HG_CUDA(cudaGetLastError());
        }
        HG_CUDA(cudaEventRecordWithFlags(a->ev_k1, s, rec_flags));
    }
    launch_postprocess(a, nq, mode, width);
}

// Plain form: one single-block launch per query (the block resets its own control words), then one compaction.
void launch_plain(hibf_gpu_agent * a, int mode, uint64_t const * d_values, uint64_t const * h_qoff,
                  uint64_t const * d_qoff, uint64_t const * d_thr, uint64_t nq, int width)
{
    hibf_gpu_hibf * h = a->h;
    check_order_and_work(a, nq, true);
    cudaStream_t s = a->stream;
    k_init_ctrl<<<1, 32, 0, s>>>(a->ctrl.as<unsigned long long>(), a->stats.as<unsigned long long>(), 0);
    HG_CUDA(cudaGetLastError());
    HG_CUDA(cudaMemsetAsync(a->qcount.p, 0, std::max<uint64_t>(nq, 1) * 4, s));
    if (a->qwork && nq)
        HG_CUDA(cudaMemsetAsync(a->qwork, 0, nq * 8, s));
    uint64_t const mask = mask_for(mode, width);
    for (uint64_t q = 0; q < nq; ++q)
    {
        (void)h_qoff;
        query_params p = base_params(a, d_values, d_qoff + q, d_thr + q, 1, mask);
        p.decide = mode == HIBF_GPU_QUERY_MEMBERSHIP;
        p.q_base = q;
        p.order = nullptr;
        p.self_init = 1;
        HG_CUDA(cudaMemsetAsync(a->tasks.p, 0xFF, std::min<uint64_t>(a->cap_tasks, 64u * h->n_ibfs + 64u) * 8, s));
        p.task_cap = std::min<uint64_t>(a->cap_tasks, 64u * h->n_ibfs + 64u);
        (a->tune.block_queries ? query_block_kernel(h->hash_count) : query_kernel(h->hash_count, a->variant))<<<
            1, 256, query_smem(h), s>>>(p);
        HG_CUDA(cudaGetLastError());
    }
    launch_postprocess(a, nq, mode, width);
}

int read_status(hibf_gpu_agent * a)
{
    HG_CUDA(cudaMemcpyAsync(a->h_ctrl.p, a->ctrl.p, C_WORDS * 8, cudaMemcpyDeviceToHost, a->stream));
    HG_CUDA(cudaMemcpyAsync(a->h_stats.p, a->stats.p, kStats * 8, cudaMemcpyDeviceToHost, a->stream));
    uint32_t const levels = a->last_levels;
    if (levels)
        HG_CUDA(cudaMemcpyAsync(a->h_lvl_stats.p, a->lvl_stats.p, levels * kStats * 8, cudaMemcpyDeviceToHost,
                                a->stream));
    HG_CUDA(cudaStreamSynchronize(a->stream));
    unsigned long long const * c = a->h_ctrl.as<unsigned long long>();
    unsigned long long const * st = a->h_stats.as<unsigned long long>();
    a->last_tasks = st[0];
    a->last_visits = st[1];
    a->last_executed = st[2];
    a->last_level_stats.clear();
    if (levels)
    {
        unsigned long long const * ls = a->h_lvl_stats.as<unsigned long long>();
        a->last_level_stats.assign(ls, ls + levels * kStats);
        for (uint32_t d = 0; d < levels; ++d)
        {
            a->last_tasks += ls[d * kStats + 0];
            a->last_visits += ls[d * kStats + 1];
            a->last_executed += ls[d * kStats + 2];
        }
    }
    unsigned long long const e = c[C_ERROR];
    if (e & E_TIMEOUT)
        return HIBF_GPU_ERR_TIMEOUT;
    if (e & E_CYCLE)
        return HIBF_GPU_ERR_CYCLE;
    if (e & E_VARIANT)
        return HIBF_GPU_ERR_LOGIC;
    if (e & E_ORDER)
        return HIBF_GPU_ERR_INVALID_ARG;
    if (e & E_TASK)
        return HIBF_GPU_ERR_LOGIC;
    if (e & (E_OVERFLOW_REC | E_OVERFLOW_TASK))
        return HIBF_GPU_ERR_OVERFLOW;
    return HIBF_GPU_OK;
}

// Runs ok(lo, hi) over [0, n) and returns whether every piece held: one piece below 2^17 entries, else up to eight
// pieces on their own threads (a 1e6-query batch's checks read 16 MB, which one Grace core takes about 0.9 ms for).
template <typename F>
bool holds_everywhere(uint64_t n, F const & ok)
{
    constexpr uint64_t kSerialLimit = 1u << 17;
    if (n < kSerialLimit)
        return ok(uint64_t{0}, n);
    unsigned const pieces = std::max(1u, std::min(8u, std::thread::hardware_concurrency()));
    uint64_t const step = (n + pieces - 1) / pieces;
    std::vector<char> good(pieces, 1);
    auto run = [&](unsigned k) {
        uint64_t const lo = std::min(n, k * step);
        good[k] = ok(lo, std::min(n, lo + step)) ? 1 : 0;
    };
    std::vector<std::thread> threads;
    threads.reserve(pieces - 1);
    unsigned k = 1;
    try
    {
        for (; k < pieces; ++k)
            threads.emplace_back(run, k);
    }
    catch (...) // no more threads: this thread takes the remaining pieces
    {
    }
    run(0);
    for (unsigned r = k; r < pieces; ++r)
        run(r);
    for (auto & t : threads)
        t.join();
    return std::all_of(good.begin(), good.end(), [](char g) { return g != 0; });
}

// Host-side checks of a batch: the mode and counter width, the thresholds (uint16 for membership, > 0 for counts)
// and, when given, the query offsets (non-decreasing).  Branch-free loops over slices, in parallel for large batches.
void check_batch(int mode, int width, uint64_t const * thr, uint64_t nq, uint64_t const * qoff = nullptr)
{
    if (mode != HIBF_GPU_QUERY_MEMBERSHIP && mode != HIBF_GPU_QUERY_COUNT)
        fail(HIBF_GPU_ERR_INVALID_ARG, "mode must be HIBF_GPU_QUERY_MEMBERSHIP or HIBF_GPU_QUERY_COUNT");
    if (mode == HIBF_GPU_QUERY_COUNT && !(width == 1 || width == 2 || width == 4 || width == 8))
        fail(HIBF_GPU_ERR_INVALID_ARG, "width must be 1, 2, 4 or 8");
    bool const membership = mode == HIBF_GPU_QUERY_MEMBERSHIP;
    std::atomic<bool> bad_offsets{false};
    bool const good = holds_everywhere(nq, [&](uint64_t lo, uint64_t hi) {
        uint64_t bad_thr = 0, bad_off = 0;
        if (thr && membership)
            for (uint64_t q = lo; q < hi; ++q)
                bad_thr |= static_cast<uint64_t>(thr[q] > 0xFFFFu);
        else if (thr)
            for (uint64_t q = lo; q < hi; ++q)
                bad_thr |= static_cast<uint64_t>(thr[q] == 0);
        if (qoff)
            for (uint64_t q = lo; q < hi; ++q)
                bad_off |= static_cast<uint64_t>(qoff[q + 1] < qoff[q]);
        if (bad_off)
            bad_offsets.store(true, std::memory_order_relaxed);
        return (bad_thr | bad_off) == 0;
    });
    if (good)
        return;
    if (bad_offsets.load())
        fail(HIBF_GPU_ERR_INVALID_ARG, "query offsets must be non-decreasing");
    fail(HIBF_GPU_ERR_INVALID_ARG, membership ? "membership thresholds are uint16" : "bulk_count thresholds must be > 0");
}

void check_mode(int mode, int width, uint64_t const * thr, uint64_t nq)
{
    check_batch(mode, width, thr, nq);
}

constexpr uint64_t kStreamMinBytes = 64ull << 20;    // smaller host batches are copied whole before the launch
constexpr uint64_t kStreamChunkBytes = 16ull << 20;  // smallest target chunk: up to 64 chunks of at least this
constexpr uint32_t kStreamMaxChunks = 64;

// Chunk boundaries of a streamed host batch: query indices q_0 = 0 < q_1 < ... < q_K = nq, each q_k (0 < k < K) a
// query whose first value starts a 32-byte sector (qoff[q_k] % 4 == 0), so that no sector of the device copy holds
// values of two chunks.  Fewer than two chunks: the batch is not streamed.
std::vector<uint64_t> stream_chunks(uint64_t const * qoff, uint64_t nq)
{
    uint64_t const nv = qoff[nq];
    uint64_t want = std::min<uint64_t>(kStreamMaxChunks, std::max<uint64_t>(2, nv * 8 / kStreamChunkBytes));
    want = std::min(want, nq);
    std::vector<uint64_t> qb{0};
    for (uint64_t k = 1; k < want; ++k)
    {
        uint64_t q = std::max(qb.back() + 1, k * nq / want);
        uint64_t const stop = std::min(nq, q + nq / want);
        while (q < stop && (qoff[q] & 3u) != 0)
            ++q;
        if (q < stop && qoff[q] > qoff[qb.back()])
            qb.push_back(q);
    }
    qb.push_back(nq);
    return qb;
}

// Host-pointer batch with automatic growth on overflow.  Results land in the agent's pinned host buffers.  Large
// batches are streamed: the offsets and thresholds go first, then the values in chunks on a second stream, each
// followed by a copy of the chunk counter (its replicas) that the kernel's root claims wait for, so the kernel
// answers the queries of arrived chunks while later chunks are still being copied.  Every copy is issued before the
// kernel launch: a host call after the launch can block until the kernel ends (the first launch of a lazily loaded
// kernel waits for the device's running work), and the kernel would then wait for chunks nobody issued.
// Position of every user bin in the order membership_for_impl reports it (HIBF.hpp:322-355): the technical bins of
// an IBF in order, a merged bin's subtree in place of the merged bin, a user bin where its run of bins ends.  A user
// bin sits in one place of the hierarchy, so ordering a result by this rank gives the reference's output before
// sort_results().  Computed once per HIBF.
std::vector<uint64_t> const & traversal_rank(hibf_gpu_hibf * h)
{
    std::lock_guard<std::mutex> lk(h->mu);
    if (!h->trav_rank.empty() || h->n_user_bins == 0)
        return h->trav_rank;
    std::vector<uint64_t> off(h->n_ibfs + 1, 0);
    for (uint64_t k = 0; k < h->n_ibfs; ++k)
        off[k + 1] = off[k] + h->bins[k];
    std::vector<uint64_t> rank(h->n_user_bins, UINT64_MAX);
    std::vector<uint8_t> entered(h->n_ibfs, 0);
    uint64_t r = 0;
    std::vector<std::pair<uint64_t, uint64_t>> stack{{0, 0}};
    entered[0] = 1;
    while (!stack.empty())
    {
        auto const [k, b] = stack.back();
        stack.pop_back();
        if (b >= h->bins[k])
            continue;
        stack.emplace_back(k, b + 1);
        uint64_t const i = off[k] + b;
        uint64_t const u = h->user_bin_id[i];
        if (u == HIBF_GPU_BIN_MERGED)
        {
            uint64_t const c = h->next_ibf_id[i];
            if (c != k && c < h->n_ibfs && !entered[c])
            {
                entered[c] = 1;
                stack.emplace_back(c, 0);
            }
        }
        else if (u < h->n_user_bins && (b + 1 == h->bins[k] || h->user_bin_id[i + 1] != u) && rank[u] == UINT64_MAX)
        {
            rank[u] = r++;
        }
    }
    h->trav_rank = std::move(rank);
    return h->trav_rank;
}

void host_batch(hibf_gpu_agent * a, int mode, uint64_t const * values, uint64_t const * qoff, uint64_t nq,
                uint64_t const * thr, int width, bool plain)
{
    check_batch(mode, width, thr, nq, qoff);
    uint64_t const nv = nq ? qoff[nq] : 0;
    // In place: values in mapped page-locked memory are read by the kernel over the host link as it needs them, so
    // no copy precedes (or paces) the launch; only the offsets and thresholds are copied.
    uint64_t const * in_place = nullptr;
    if (a->host_read && !plain && nv)
    {
        cudaPointerAttributes attr{};
        void * dev = nullptr;
        if (cudaPointerGetAttributes(&attr, values) == cudaSuccess && attr.type == cudaMemoryTypeHost &&
            cudaHostGetDevicePointer(&dev, const_cast<uint64_t *>(values), 0) == cudaSuccess)
            in_place = static_cast<uint64_t const *>(dev);
        cudaGetLastError(); // pageable memory: the queries above fail, and the values are copied
    }
    a->last_in_place = in_place != nullptr;
    a->in_values.ensure(nv * 8); // the copy's destination, or where an in-place batch's roots stage the values
    if (in_place)
        a->staged.ensure(std::max<uint64_t>(nq, 1) * 4);
    struct stage_reset
    {
        hibf_gpu_agent * a;
        ~stage_reset()
        {
            a->stage_values = nullptr;
            a->stage_counts = nullptr;
        }
    } const stage_guard{a};
    if (in_place)
    {
        a->stage_values = a->in_values.as<uint64_t>();
        a->stage_counts = a->staged.as<uint32_t>();
    }
    a->in_qoff.ensure((nq + 1) * 8);
    a->in_thr.ensure(std::max<uint64_t>(nq, 1) * 8);
    std::vector<uint64_t> qb;
    if (!in_place && !plain && !a->order && nv * 8 >= kStreamMinBytes)
        qb = stream_chunks(qoff, nq);
    bool const streamed = qb.size() > 2;
    a->last_chunks = streamed ? static_cast<uint32_t>(qb.size() - 1) : 0u;
    struct queue_guard // a streamed batch runs the work queue (children run while later roots are still copied)
    {
        hibf_gpu_agent * a;
        ~queue_guard()
        {
            a->force_queue = false;
        }
    } const queue_reset{a};
    a->force_queue = streamed;
    uint64_t tasks = std::max<uint64_t>(a->cap_tasks, nq * 4 + 1024);
    uint64_t results = std::max<uint64_t>(a->cap_results, nq * 4 + 1024);
    ensure_capacity(a, std::max<uint64_t>(nq, 1), tasks, results); // allocations synchronise: before any copy
    uint32_t const n_tl = streamed ? static_cast<uint32_t>(qb.size() - 1) : 1u;
    if (!a->tl_t0)
    {
        HG_CUDA(cudaEventCreate(&a->tl_t0));
        HG_CUDA(cudaEventCreate(&a->tl_done));
    }
    while (a->tl_chunk.size() < n_tl)
    {
        cudaEvent_t e{};
        HG_CUDA(cudaEventCreate(&e));
        a->tl_chunk.push_back(e);
    }
    a->tl_n = 0;
    HG_CUDA(cudaEventRecord(a->tl_t0, a->stream));
    HG_CUDA(cudaMemcpyAsync(a->in_qoff.p, qoff, (nq + 1) * 8, cudaMemcpyHostToDevice, a->stream));
    if (nq)
        HG_CUDA(cudaMemcpyAsync(a->in_thr.p, thr, nq * 8, cudaMemcpyHostToDevice, a->stream));
    struct arrive_reset
    {
        hibf_gpu_agent * a;
        ~arrive_reset()
        {
            if (a->arrive)
                cudaStreamSynchronize(a->copy_stream); // an error left copies in flight: finish them first
            a->arrive = nullptr;
        }
    } const reset{a};
    if (streamed)
    {
        if (!a->copy_stream)
        {
            HG_CUDA(cudaStreamCreateWithFlags(&a->copy_stream, cudaStreamNonBlocking));
            HG_CUDA(cudaEventCreateWithFlags(&a->ev_ready, cudaEventDisableTiming));
            HG_CUDA(cudaEventCreateWithFlags(&a->ev_copied, cudaEventDisableTiming));
        }
        uint32_t const chunks = static_cast<uint32_t>(qb.size() - 1);
        size_t const counter_bytes = kArrivalReplicas * kArrivalStride * 4;
        a->arrived.ensure(counter_bytes);
        a->arrive_first.ensure(qb.size() * 8);
        a->h_arrive_first.ensure(qb.size() * 8);
        a->h_arrive_counts.ensure(chunks * counter_bytes); // chunk k's source holds k + 1 in every replica
        std::memcpy(a->h_arrive_first.p, qb.data(), qb.size() * 8);
        unsigned int * counts = a->h_arrive_counts.as<unsigned int>();
        std::memset(counts, 0, chunks * counter_bytes);
        for (uint32_t k = 0; k < chunks; ++k)
            for (uint32_t r = 0; r < kArrivalReplicas; ++r)
                counts[(static_cast<size_t>(k) * kArrivalReplicas + r) * kArrivalStride] = k + 1u;
        HG_CUDA(cudaMemcpyAsync(a->arrive_first.p, a->h_arrive_first.p, qb.size() * 8, cudaMemcpyHostToDevice,
                                a->stream));
        HG_CUDA(cudaMemsetAsync(a->arrived.p, 0, counter_bytes, a->stream));
        HG_CUDA(cudaEventRecord(a->ev_ready, a->stream));
        HG_CUDA(cudaStreamWaitEvent(a->copy_stream, a->ev_ready, 0));
        try
        {
            for (uint32_t k = 0; k < chunks; ++k)
            {
                uint64_t const v0 = qoff[qb[k]], v1 = qoff[qb[k + 1]];
                if (v1 > v0)
                    HG_CUDA(cudaMemcpyAsync(a->in_values.as<uint64_t>() + v0, values + v0, (v1 - v0) * 8,
                                            cudaMemcpyHostToDevice, a->copy_stream));
                unsigned int const * src = counts + static_cast<size_t>(k) * kArrivalReplicas * kArrivalStride;
                HG_CUDA(cudaMemcpyAsync(a->arrived.p, src, counter_bytes, cudaMemcpyHostToDevice, a->copy_stream));
                HG_CUDA(cudaEventRecord(a->tl_chunk[k], a->copy_stream));
            }
            a->tl_n = chunks;
            HG_CUDA(cudaEventRecord(a->ev_copied, a->copy_stream));
        }
        catch (...)
        {
            cudaStreamSynchronize(a->copy_stream);
            throw;
        }
        a->arrive = a->arrived.as<unsigned int>();
        a->arrive_chunks = chunks;
        a->arrive_limit_ns = 10ull * 1000 * 1000 * 1000 + nv * 8 / 2; // 10 s + the copy at 2 GB/s
    }
    else
    {
        if (nv && !in_place)
            HG_CUDA(cudaMemcpyAsync(a->in_values.p, values, nv * 8, cudaMemcpyHostToDevice, a->stream));
        HG_CUDA(cudaEventRecord(a->tl_chunk[0], a->stream));
        a->tl_n = 1;
    }
    uint64_t const * const d_values = in_place ? in_place : a->in_values.as<uint64_t>();
    for (int attempt = 0;; ++attempt)
    {
        ensure_capacity(a, std::max<uint64_t>(nq, 1), tasks, results);
        if (plain)
            launch_plain(a, mode, d_values, qoff, a->in_qoff.as<uint64_t>(), a->in_thr.as<uint64_t>(), nq, width);
        else
            launch_batch(a, mode, d_values, a->in_qoff.as<uint64_t>(), a->in_thr.as<uint64_t>(), nq, width);
        if (streamed && attempt == 0)
            HG_CUDA(cudaStreamWaitEvent(a->stream, a->ev_copied, 0)); // later work on the stream follows the copies
        int const st = read_status(a);
        if (st == HIBF_GPU_OK)
            break;
        unsigned long long const * c = a->h_ctrl.as<unsigned long long>();
        if (st != HIBF_GPU_ERR_OVERFLOW || attempt > 8)
            fail(st, st == HIBF_GPU_ERR_TIMEOUT     ? "device wait limit expired" :
                     st == HIBF_GPU_ERR_CYCLE       ? "merged bins form a cycle (descent deeper than the hierarchy)" :
                     st == HIBF_GPU_ERR_INVALID_ARG ? "a claim-order entry is not a query index of the batch" :
                     st == HIBF_GPU_ERR_LOGIC       ? "a tuned kernel variant met an IBF it does not handle, or a "
                                                      "task named a query or IBF out of range" :
                                                      "batch capacity exceeded");
        if (c[C_ERROR] & E_OVERFLOW_TASK)
            tasks *= 4;
        if (c[C_ERROR] & E_OVERFLOW_REC)
            results = std::max<uint64_t>(results * 4, c[C_NREC] + 1024);
    }
    a->h_roff.ensure((nq + 1) * 8);
    HG_CUDA(cudaMemcpyAsync(a->h_roff.p, a->roff.p, (nq + 1) * 8, cudaMemcpyDeviceToHost, a->stream));
    HG_CUDA(cudaStreamSynchronize(a->stream));
    uint64_t const nr = a->h_roff.as<uint64_t>()[nq];
    a->h_ids.ensure(nr * 8);
    a->h_cnt.ensure(nr * 8);
    if (nr)
    {
        HG_CUDA(cudaMemcpyAsync(a->h_ids.p, a->out_ids.p, nr * 8, cudaMemcpyDeviceToHost, a->stream));
        if (mode == HIBF_GPU_QUERY_COUNT)
            HG_CUDA(cudaMemcpyAsync(a->h_cnt.p, width == 8 ? a->out_cnt.p : a->out_cntw.p, nr * width,
                                    cudaMemcpyDeviceToHost, a->stream));
    }
    HG_CUDA(cudaEventRecord(a->tl_done, a->stream));
    HG_CUDA(cudaStreamSynchronize(a->stream));
}

// Whether the tuned kernel variants apply: at most 3 hash functions and rows of at most 4 words.
bool variants_apply(uint32_t hash_count, uint64_t max_row_words)
{
    return hash_count <= 3 && max_row_words <= 4;
}

uint64_t max_bin_words(hibf_gpu_hibf const * h)
{
    uint64_t m = 0;
    for (uint64_t w : h->bin_words)
        m = std::max(m, w);
    return m;
}

// The kernel variant of a schedule (kVariantTable), or -1 when no kernel has that combination.
int variant_of(hibf_gpu_tuning const & t)
{
    for (int v = 0; v < kQueryVariants; ++v)
        if (t.values_per_lane == static_cast<uint32_t>(kVariantTable[v][0]) &&
            t.fetch_bytes == static_cast<uint32_t>(8 * kVariantTable[v][1]) &&
            t.counter_bits == static_cast<uint32_t>(kVariantTable[v][2]))
            return v;
    return -1;
}

// The kernel variant of the levels below the root: values_per_lane replaced by level_values_per_lane when set.
int child_variant_of(hibf_gpu_tuning t)
{
    if (t.level_values_per_lane)
        t.values_per_lane = t.level_values_per_lane;
    return variant_of(t);
}

void check_tuning(hibf_gpu_tuning const & t, hibf_gpu_hibf const * h)
{
    int const cv = child_variant_of(t);
    if (cv < 0 || (cv != 0 && !variants_apply(h->hash_count, max_bin_words(h))))
        fail(HIBF_GPU_ERR_INVALID_ARG, "no query kernel for level_values_per_lane with this fetch_bytes and "
                                       "counter_bits on this hierarchy");
    int const v = variant_of(t);
    if (v < 0)
        fail(HIBF_GPU_ERR_INVALID_ARG, "no query kernel for this (values_per_lane, fetch_bytes, counter_bits)");
    if (v != 0 && !variants_apply(h->hash_count, max_bin_words(h)))
        fail(HIBF_GPU_ERR_INVALID_ARG, "tuned kernel variants need at most 3 hash functions and rows of at most 4 "
                                       "words; this hierarchy takes the default (1, 8, 7)");
    if (t.blocks_per_sm > 32)
        fail(HIBF_GPU_ERR_INVALID_ARG, "blocks_per_sm must be in [0, 32]");
    if (t.schedule != HIBF_GPU_SCHEDULE_QUEUE && t.schedule != HIBF_GPU_SCHEDULE_LEVELS)
        fail(HIBF_GPU_ERR_INVALID_ARG, "schedule must be HIBF_GPU_SCHEDULE_QUEUE or HIBF_GPU_SCHEDULE_LEVELS");
    if (t.early_exit_stages == HIBF_GPU_EARLY_EXIT_ADAPTIVE)
    {
        if (t.early_exit_step == 0)
            fail(HIBF_GPU_ERR_INVALID_ARG, "the adaptive early exit needs early_exit_step >= 1 values between checks");
    }
    else if (t.early_exit_stages)
    {
        uint64_t const last = t.early_exit_first + static_cast<uint64_t>(t.early_exit_stages - 1) * t.early_exit_step;
        if (t.early_exit_first == 0 || last >= 100 || (t.early_exit_stages > 1 && t.early_exit_step == 0))
            fail(HIBF_GPU_ERR_INVALID_ARG, "early-exit checkpoints must be increasing percentages in (0, 100)");
    }
}

hibf_gpu_tuning with_schedule(hibf_gpu_tuning t, uint32_t first, uint32_t step)
{
    t.early_exit_first = first;
    t.early_exit_step = step;
    t.early_exit_stages = first == 0 ? 0u : (step == 0 ? 1u : (90u - first) / step + 1u); // checkpoints up to 90%
    return t;
}

hibf_gpu_tuning with_adaptive(hibf_gpu_tuning t, uint32_t min_values)
{
    t.early_exit_first = 0;
    t.early_exit_step = min_values;
    t.early_exit_stages = HIBF_GPU_EARLY_EXIT_ADAPTIVE;
    return t;
}

hibf_gpu_tuning with_vpl(hibf_gpu_tuning t, uint32_t vpl)
{
    t.values_per_lane = vpl;
    return t;
}

bool same_schedule(hibf_gpu_tuning const & a, hibf_gpu_tuning const & b)
{
    return a.early_exit_stages == b.early_exit_stages &&
           (a.early_exit_stages == 0 || (a.early_exit_first == b.early_exit_first && a.early_exit_step == b.early_exit_step));
}

// Stage 1: every kernel variant at 1 block per SM and at as many as fit; stage 2: the early-exit checkpoints (fixed
// schedules, then the adaptive one at two minimum step sizes) with the fastest kernel; stage 3: the minimum task
// length for early exit.
void tune_search(uint32_t hash_count, uint64_t max_row_words, hibf_gpu_tune_measure_fn measure, void * user,
                 std::vector<hibf_gpu_tune_trial> & trials, hibf_gpu_tuning & best)
{
    hibf_gpu_tuning base{};
    hibf_gpu_tuning_default(&base);
    double best_ms = 0;
    auto run = [&](hibf_gpu_tuning const & t)
    {
        double ms = 0;
        int const st = measure(&t, user, &ms);
        if (st != HIBF_GPU_OK)
            fail(st, "autotune measurement failed");
        if (!(ms >= 0))
            fail(HIBF_GPU_ERR_INVALID_ARG, "autotune measurement returned a negative time");
        trials.push_back(hibf_gpu_tune_trial{t, ms});
        if (trials.size() == 1 || ms < best_ms)
        {
            best_ms = ms;
            best = t;
        }
    };
    for (int v = 0; v < kQueryVariants; ++v)
    {
        if (v != 0 && !variants_apply(hash_count, max_row_words))
            break;
        if (max_row_words < 2 && kVariantTable[v][1] != 1)
            continue; // 16-byte fetches need rows of two or more words
        for (uint32_t bps : {0u, 1u})
        {
            hibf_gpu_tuning t = base;
            t.values_per_lane = static_cast<uint32_t>(kVariantTable[v][0]);
            t.fetch_bytes = static_cast<uint32_t>(8 * kVariantTable[v][1]);
            t.counter_bits = static_cast<uint32_t>(kVariantTable[v][2]);
            t.blocks_per_sm = bps;
            run(t);
        }
    }
    {
        hibf_gpu_tuning t = best;
        t.schedule = HIBF_GPU_SCHEDULE_LEVELS;
        run(t);
        t.level_values_per_lane = 2; // more loads in flight where L2 holds the IBFs
        if (variants_apply(hash_count, max_row_words) && variant_of(with_vpl(t, 2)) >= 0 && t.values_per_lane != 2)
            run(t);
    }
    hibf_gpu_tuning const k = best;
    static constexpr uint32_t schedules[][2] = {{0, 0},   {10, 10}, {20, 10}, {30, 10}, {50, 10},
                                                {30, 20}, {50, 20}, {40, 5},  {50, 5},  {60, 5}};
    for (auto const & sch : schedules)
    {
        hibf_gpu_tuning const t = with_schedule(k, sch[0], sch[1]);
        if (!same_schedule(t, k))
            run(t);
    }
    for (uint32_t m : {32u, 128u})
    {
        hibf_gpu_tuning const t = with_adaptive(k, m);
        if (!same_schedule(t, k))
            run(t);
    }
    hibf_gpu_tuning const e = best;
    if (e.early_exit_stages)
        for (uint32_t m : {64u, 128u, 256u, 512u, 1024u})
            if (m != e.early_exit_min)
            {
                hibf_gpu_tuning t = e;
                t.early_exit_min = m;
                run(t);
            }
}

// Device measurement of one schedule for hibf_gpu_agent_autotune.
struct autotune_ctx
{
    hibf_gpu_agent * a;
    int mode, width, reps;
    uint64_t const *values, *qoff, *thr;
    uint64_t nq;
    std::vector<uint64_t> ref_roff, ref_ids, ref_cnt, roff, ids, cnt;
    bool have_ref{false};
};

void fetch_batch_results(autotune_ctx & c, std::vector<uint64_t> & roff, std::vector<uint64_t> & ids,
                         std::vector<uint64_t> & cnt)
{
    hibf_gpu_agent * a = c.a;
    roff.resize(c.nq + 1);
    HG_CUDA(cudaMemcpyAsync(roff.data(), a->roff.p, (c.nq + 1) * 8, cudaMemcpyDeviceToHost, a->stream));
    HG_CUDA(cudaStreamSynchronize(a->stream));
    uint64_t const nr = roff[c.nq];
    ids.resize(nr);
    cnt.resize(c.mode == HIBF_GPU_QUERY_COUNT ? nr : 0);
    if (nr)
    {
        HG_CUDA(cudaMemcpyAsync(ids.data(), a->out_ids.p, nr * 8, cudaMemcpyDeviceToHost, a->stream));
        if (c.mode == HIBF_GPU_QUERY_COUNT)
            HG_CUDA(cudaMemcpyAsync(cnt.data(), a->out_cnt.p, nr * 8, cudaMemcpyDeviceToHost, a->stream));
    }
    HG_CUDA(cudaStreamSynchronize(a->stream));
}

int autotune_measure(hibf_gpu_tuning const * t, void * user, double * kernel_ms)
{
    return guarded(
        [&]
        {
            autotune_ctx & c = *static_cast<autotune_ctx *>(user);
            hibf_gpu_agent * a = c.a;
            a->tune = *t;
            a->variant = variant_of(*t);
            a->child_variant = child_variant_of(*t);
            ensure_capacity(a, a->cap_queries, a->cap_tasks, a->cap_results); // the level schedule's buffers
            std::vector<double> ms;
            for (int r = -1; r < c.reps; ++r)
            {
                launch_batch(a, c.mode, c.values, c.qoff, c.thr, c.nq, c.width);
                int const st = read_status(a);
                if (st != HIBF_GPU_OK)
                    fail(st, "autotune batch failed (reserve enough tasks and results for the sample)");
                if (r < 0)
                {
                    auto & roff = c.have_ref ? c.roff : c.ref_roff;
                    auto & ids = c.have_ref ? c.ids : c.ref_ids;
                    auto & cnt = c.have_ref ? c.cnt : c.ref_cnt;
                    fetch_batch_results(c, roff, ids, cnt);
                    if (c.have_ref && (roff != c.ref_roff || ids != c.ref_ids || cnt != c.ref_cnt))
                        fail(HIBF_GPU_ERR_LOGIC, "a kernel schedule changed the query results");
                    c.have_ref = true;
                    continue;
                }
                float k = 0;
                HG_CUDA(cudaEventElapsedTime(&k, a->ev_k0, a->ev_k1));
                ms.push_back(k);
            }
            std::sort(ms.begin(), ms.end());
            *kernel_ms = ms.empty() ? 0.0 : ms[ms.size() / 2];
        });
}

} // namespace

extern "C"
{
    void hibf_gpu_tuning_default(hibf_gpu_tuning * t)
    {
        if (!t)
            return;
        t->values_per_lane = 1;
        t->fetch_bytes = 8;
        t->counter_bits = 7;
        t->blocks_per_sm = 0;
        t->early_exit_first = 0;
        t->early_exit_step = 32; // adaptive: checks where the outcome can first change, at least 32 values apart
        t->early_exit_stages = HIBF_GPU_EARLY_EXIT_ADAPTIVE;
        t->early_exit_min = 256;
        t->block_queries = 8192;
        t->schedule = HIBF_GPU_SCHEDULE_QUEUE;
        t->level_values_per_lane = 0;
    }

    int hibf_gpu_agent_set_tuning(hibf_gpu_agent * a, hibf_gpu_tuning const * t)
    {
        return guarded(
            [&]
            {
                if (!a || !t)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                check_tuning(*t, a->h);
                a->tune = *t;
                a->variant = variant_of(*t);
                a->child_variant = child_variant_of(*t);
                ensure_capacity(a, a->cap_queries, a->cap_tasks, a->cap_results); // level buffers, if now needed
                if (a->graph)
                {
                    HG_CUDA(cudaGraphExecDestroy(a->graph));
                    a->graph = nullptr;
                }
            });
    }

    int hibf_gpu_agent_set_order_d(hibf_gpu_agent * a, uint32_t const * d_order, uint64_t n_queries)
    {
        return guarded(
            [&]
            {
                if (!a)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                a->order = n_queries ? d_order : nullptr;
                a->order_n = a->order ? n_queries : 0;
                if (a->graph)
                {
                    HG_CUDA(cudaGraphExecDestroy(a->graph));
                    a->graph = nullptr;
                }
            });
    }

    int hibf_gpu_agent_set_work_out_d(hibf_gpu_agent * a, uint64_t * d_work, uint64_t n_queries)
    {
        return guarded(
            [&]
            {
                if (!a)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                a->qwork = n_queries ? reinterpret_cast<unsigned long long *>(d_work) : nullptr;
                a->qwork_n = a->qwork ? n_queries : 0;
                if (a->graph)
                {
                    HG_CUDA(cudaGraphExecDestroy(a->graph));
                    a->graph = nullptr;
                }
            });
    }

    int hibf_gpu_agent_query_features_d(hibf_gpu_agent * a, uint64_t const * d_values,
                                        uint64_t const * d_query_offsets, uint64_t n_queries,
                                        uint64_t const * d_thresholds, uint32_t probe, float * d_features)
    {
        return guarded(
            [&]
            {
                if (!a || !d_query_offsets || !d_thresholds || (n_queries && !d_features) || probe == 0)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "bad argument");
                if (!n_queries)
                    return;
                query_params p = base_params(a, d_values, d_query_offsets, d_thresholds, n_queries, ~0ull);
                uint64_t const want = (n_queries + 7) / 8;
                unsigned const grid = static_cast<unsigned>(
                    std::max<uint64_t>(1, std::min<uint64_t>(want, static_cast<uint64_t>(sm_count()) * 8u)));
                features_kernel(a->h->hash_count)<<<grid, 256, query_smem(a->h), a->stream>>>(p, probe, d_features);
                HG_CUDA(cudaGetLastError());
            });
    }

    int hibf_gpu_agent_get_tuning(hibf_gpu_agent * a, hibf_gpu_tuning * t)
    {
        if (!a || !t)
            return HIBF_GPU_ERR_INVALID_ARG;
        *t = a->tune;
        return HIBF_GPU_OK;
    }

    int hibf_gpu_tune_search(uint32_t hash_count, uint32_t max_row_words, hibf_gpu_tune_measure_fn measure,
                             void * user, hibf_gpu_tune_trial * trials, uint64_t cap, uint64_t * n_trials,
                             hibf_gpu_tuning * best)
    {
        return guarded(
            [&]
            {
                if (!measure || !best || hash_count == 0 || hash_count > 5)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "bad argument");
                std::vector<hibf_gpu_tune_trial> all;
                tune_search(hash_count, max_row_words, measure, user, all, *best);
                if (n_trials)
                    *n_trials = all.size();
                if (trials)
                    std::copy_n(all.begin(), std::min<uint64_t>(cap, all.size()), trials);
            });
    }

    int hibf_gpu_agent_autotune(hibf_gpu_agent * a, int mode, uint64_t const * d_values,
                                uint64_t const * d_query_offsets, uint64_t n_queries, uint64_t const * d_thresholds,
                                int width, int reps, hibf_gpu_tune_trial * trials, uint64_t cap, uint64_t * n_trials)
    {
        return guarded(
            [&]
            {
                if (!a || !d_query_offsets || !d_thresholds || n_queries == 0 || reps < 1 || reps > 100)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "bad argument");
                check_mode(mode, width, nullptr, n_queries);
                ensure_capacity(a, n_queries, std::max<uint64_t>(a->cap_tasks, n_queries * 4 + 1024),
                                std::max<uint64_t>(a->cap_results, n_queries * 4 + 1024));
                if (a->graph)
                {
                    HG_CUDA(cudaGraphExecDestroy(a->graph));
                    a->graph = nullptr;
                }
                autotune_ctx c{a, mode, width, reps, d_values, d_query_offsets, d_thresholds, n_queries, {}, {}, {},
                               {}, {}, {}};
                hibf_gpu_tuning const before = a->tune;
                std::vector<hibf_gpu_tune_trial> all;
                hibf_gpu_tuning best{};
                try
                {
                    tune_search(a->h->hash_count, max_bin_words(a->h), autotune_measure, &c, all, best);
                }
                catch (...)
                {
                    a->tune = before;
                    a->variant = variant_of(before);
                    a->child_variant = child_variant_of(before);
                    throw;
                }
                a->tune = best;
                a->variant = variant_of(best);
                a->child_variant = child_variant_of(best);
                ensure_capacity(a, a->cap_queries, a->cap_tasks, a->cap_results);
                if (n_trials)
                    *n_trials = all.size();
                if (trials)
                    std::copy_n(all.begin(), std::min<uint64_t>(cap, all.size()), trials);
            });
    }



    int hibf_gpu_hibf_create(uint64_t n_user_bins, uint64_t n_ibfs, uint64_t const * bins,
                             uint64_t const * bin_sizes, uint64_t const * hash_funs, uint64_t const * next_ibf_id,
                             uint64_t const * user_bin_id, hibf_gpu_hibf ** out)
    {
        return guarded(
            [&]
            {
                if (!out || !bins || !bin_sizes || !hash_funs || !next_ibf_id || !user_bin_id)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                *out = nullptr;
                if (n_ibfs == 0 || n_ibfs > kNodeMask)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "number of IBFs must be in [1, 2^26)");
                if (n_user_bins >= 0xFFFFFFFEull)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "number of user bins must be below 2^32 - 2");
                std::vector<uint64_t> off(n_ibfs + 1, 0);
                for (uint64_t k = 0; k < n_ibfs; ++k)
                {
                    if (bins[k] == 0)
                        fail(HIBF_GPU_ERR_LOGIC, "The number of bins must be > 0.");
                    if (hash_funs[k] == 0 || hash_funs[k] > 5)
                        fail(HIBF_GPU_ERR_LOGIC, "The number of hash functions must be > 0 and <= 5.");
                    if (bin_sizes[k] == 0)
                        fail(HIBF_GPU_ERR_LOGIC, "The size of a bin must be > 0.");
                    off[k + 1] = off[k] + bins[k];
                }
                for (uint64_t k = 1; k < n_ibfs; ++k)
                    if (hash_funs[k] != hash_funs[0])
                        fail(HIBF_GPU_ERR_INVALID_ARG,
                             "all IBFs of a hierarchy must use the same number of hash functions");
                if (off[n_ibfs] >= 0xFFFFFFFFull)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "too many technical bins in total");
                // per-bin descriptors
                std::vector<uint2> descs(off[n_ibfs]);
                for (uint64_t k = 0; k < n_ibfs; ++k)
                {
                    for (uint64_t b = 0; b < bins[k]; ++b)
                    {
                        uint64_t const i = off[k] + b;
                        uint64_t const ub = user_bin_id[i];
                        uint32_t flags = 0;
                        uint32_t id = 0;
                        if (ub == HIBF_GPU_BIN_MERGED)
                        {
                            flags |= F_MERGED;
                            if (next_ibf_id[i] >= n_ibfs)
                                fail(HIBF_GPU_ERR_INVALID_ARG, "next_ibf_id out of range");
                            id = static_cast<uint32_t>(next_ibf_id[i]);
                        }
                        else if (ub == HIBF_GPU_BIN_DELETED)
                        {
                            flags |= F_DELETED;
                        }
                        else
                        {
                            if (ub >= n_user_bins)
                                fail(HIBF_GPU_ERR_INVALID_ARG, "user bin id out of range");
                            id = static_cast<uint32_t>(ub);
                            // last bin || end of split bin (HIBF.hpp:345)
                            if (b + 1 == bins[k] || ub != user_bin_id[i + 1])
                                flags |= F_RUN_END;
                        }
                        if (b == 0)
                            flags |= F_HEAD;
                        else
                        {
                            uint64_t const pu = user_bin_id[i - 1];
                            bool const prev_merged = pu == HIBF_GPU_BIN_MERGED;
                            bool const prev_end = pu != HIBF_GPU_BIN_MERGED && pu != HIBF_GPU_BIN_DELETED &&
                                                  pu != ub;
                            if (prev_merged || prev_end)
                                flags |= F_HEAD;
                        }
                        descs[i] = make_uint2(id, flags);
                    }
                }
                // depth of the hierarchy (longest merged-bin path from the root); a cycle makes it unbounded
                std::vector<uint32_t> depth(n_ibfs, 0xFFFFFFFFu);
                std::vector<uint64_t> stack{0};
                depth[0] = 0;
                uint32_t max_depth = 0;
                uint64_t visited = 0;
                while (!stack.empty())
                {
                    uint64_t const k = stack.back();
                    stack.pop_back();
                    if (++visited > n_ibfs)
                        break;
                    for (uint64_t b = 0; b < bins[k]; ++b)
                    {
                        uint64_t const i = off[k] + b;
                        if (user_bin_id[i] != HIBF_GPU_BIN_MERGED)
                            continue;
                        uint64_t const c = next_ibf_id[i];
                        if (depth[c] != 0xFFFFFFFFu)
                            continue; // already reached (or a cycle); the device enforces the depth bound
                        depth[c] = depth[k] + 1;
                        max_depth = std::max(max_depth, depth[c]);
                        stack.push_back(c);
                    }
                }
                if (max_depth > 60)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "hierarchy deeper than 60 levels");
                require_device();
                auto h = new hibf_gpu_hibf{};
                try
                {
                    h->n_user_bins = n_user_bins;
                    h->n_ibfs = n_ibfs;
                    h->next_ibf_id.assign(next_ibf_id, next_ibf_id + off[n_ibfs]);
                    h->user_bin_id.assign(user_bin_id, user_bin_id + off[n_ibfs]);
                    // parents: every merged bin's child IBF gets (IBF, bin); the root keeps (0, 0)
                    h->prev_ibf.assign(n_ibfs, 0);
                    h->prev_bin.assign(n_ibfs, 0);
                    for (uint64_t k = 0; k < n_ibfs; ++k)
                        for (uint64_t b = 0; b < bins[k]; ++b)
                        {
                            uint64_t const i = off[k] + b;
                            if (user_bin_id[i] == HIBF_GPU_BIN_MERGED && next_ibf_id[i] != k)
                            {
                                h->prev_ibf[next_ibf_id[i]] = k;
                                h->prev_bin[next_ibf_id[i]] = b;
                            }
                        }
                    h->occupancy.resize(n_ibfs);
                    for (uint64_t k = 0; k < n_ibfs; ++k)
                        h->occupancy[k].assign(((bins[k] + 63) / 64) * 64, 0);
                    h->track_occupancy.assign(n_ibfs, 0);
                    h->max_depth = max_depth;
                    HG_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
                    uint32_t cpw = 64;
                    for (uint64_t k = 0; k < n_ibfs; ++k)
                    {
                        uint64_t const bw = (bins[k] + 63u) / 64u;
                        uint64_t const rw = padded_row_words(bw);
                        h->bins.push_back(bins[k]);
                        h->bin_size.push_back(bin_sizes[k]);
                        h->hash_funs.push_back(hash_funs[k]);
                        h->bin_words.push_back(bw);
                        h->row_words.push_back(rw);
                        auto st = std::make_unique<dbuf>();
                        size_t const bytes = bin_sizes[k] * rw * 8;
                        st->ensure(bytes);
                        HG_CUDA(cudaMemsetAsync(st->p, 0, bytes, h->stream));
                        h->total_bytes += bytes;
                        dev_node nd{};
                        nd.words = st->as<uint64_t>();
                        nd.bin_size = bin_sizes[k];
                        nd.bins = static_cast<uint32_t>(bins[k]);
                        nd.bin_words = static_cast<uint32_t>(bw);
                        nd.row_words = static_cast<uint32_t>(rw);
                        nd.hash_shift = static_cast<uint32_t>(__builtin_clzll(bin_sizes[k]));
                        nd.hash_funs = static_cast<uint32_t>(hash_funs[k]);
                        nd.desc_offset = static_cast<uint32_t>(off[k]);
                        nd.lpv_log2 = lanes_per_value_log2(bw);
                        uint32_t const need = bw > 32 ? static_cast<uint32_t>(64 * bw) : (64u << nd.lpv_log2);
                        cpw = std::max(cpw, need);
                        h->nodes.push_back(nd);
                        h->stores.push_back(std::move(st));
                    }
                    h->counters_per_warp = cpw;
                    h->hash_count = static_cast<uint32_t>(hash_funs[0]);
                    if (static_cast<size_t>(8) * cpw * 4 > 200 * 1024)
                        fail(HIBF_GPU_ERR_INVALID_ARG, "an IBF is too wide for the query kernel's shared counters");
                    h->d_nodes.ensure(n_ibfs * sizeof(dev_node));
                    HG_CUDA(cudaMemcpyAsync(h->d_nodes.p, h->nodes.data(), n_ibfs * sizeof(dev_node),
                                            cudaMemcpyHostToDevice, h->stream));
                    h->d_descs.ensure(descs.size() * sizeof(uint2));
                    HG_CUDA(cudaMemcpyAsync(h->d_descs.p, descs.data(), descs.size() * sizeof(uint2),
                                            cudaMemcpyHostToDevice, h->stream));
                    HG_CUDA(cudaStreamSynchronize(h->stream));
                    size_t const smem = query_smem(h);
                    for (int v = 0; v < kQueryVariants; ++v)
                        HG_CUDA(cudaFuncSetAttribute(query_kernel(h->hash_count, v),
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     static_cast<int>(std::max<size_t>(smem, 48 * 1024))));
                    HG_CUDA(cudaFuncSetAttribute(features_kernel(h->hash_count),
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 static_cast<int>(std::max<size_t>(smem, 48 * 1024))));
                    HG_CUDA(cudaFuncSetAttribute(query_block_kernel(h->hash_count),
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 static_cast<int>(std::max<size_t>(smem, 48 * 1024))));
                }
                catch (...)
                {
                    if (h->stream)
                        cudaStreamDestroy(h->stream);
                    delete h;
                    throw;
                }
                *out = h;
            });
    }

    int hibf_gpu_hibf_destroy(hibf_gpu_hibf * h)
    {
        return guarded(
            [&]
            {
                if (!h)
                    return;
                cudaStreamSynchronize(h->stream);
                cudaStreamDestroy(h->stream);
                delete h;
            });
    }

    int hibf_gpu_hibf_info(hibf_gpu_hibf const * h, uint64_t out[4])
    {
        return guarded(
            [&]
            {
                if (!h || !out)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                out[0] = h->n_user_bins;
                out[1] = h->n_ibfs;
                out[2] = h->max_depth;
                out[3] = h->total_bytes;
            });
    }

    int hibf_gpu_hibf_get_tables(hibf_gpu_hibf const * h, uint64_t * bins, uint64_t * bin_sizes, uint64_t * hash_funs,
                                 uint64_t * next_ibf_id, uint64_t * user_bin_id)
    {
        return guarded(
            [&]
            {
                if (!h)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                if (bins)
                    std::copy(h->bins.begin(), h->bins.end(), bins);
                if (bin_sizes)
                    std::copy(h->bin_size.begin(), h->bin_size.end(), bin_sizes);
                if (hash_funs)
                    std::copy(h->hash_funs.begin(), h->hash_funs.end(), hash_funs);
                if (next_ibf_id)
                    std::copy(h->next_ibf_id.begin(), h->next_ibf_id.end(), next_ibf_id);
                if (user_bin_id)
                    std::copy(h->user_bin_id.begin(), h->user_bin_id.end(), user_bin_id);
            });
    }

    int hibf_gpu_hibf_ibf_info(hibf_gpu_hibf const * h, uint64_t k, uint64_t out[5])
    {
        return guarded(
            [&]
            {
                if (!h || !out || k >= h->n_ibfs)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "bad argument");
                out[0] = h->bins[k];
                out[1] = h->bin_words[k] * 64;
                out[2] = h->bin_size[k];
                out[3] = h->hash_funs[k];
                out[4] = h->row_words[k] * 8;
            });
    }

    int hibf_gpu_hibf_emplace_d(hibf_gpu_hibf * h, uint64_t k, uint64_t const * d_values, uint64_t const * d_bins,
                                uint64_t n, uint64_t bin, void * stream)
    {
        return guarded(
            [&]
            {
                if (!h || k >= h->n_ibfs || (n && !d_values))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "bad argument");
                if (!d_bins && bin >= h->bins[k])
                    fail(HIBF_GPU_ERR_INVALID_ARG, "bin index out of range");
                if (!n)
                    return;
                cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : h->stream;
                dev_node const & nd = h->nodes[k];
                k_hibf_emplace<<<grid_cap(n, 256), 256, 0, s>>>(const_cast<uint64_t *>(nd.words), nd.bin_size,
                                                                nd.row_words, nd.hash_shift, nd.hash_funs, d_values,
                                                                d_bins, n, bin, h->bins[k]);
                HG_CUDA(cudaGetLastError());
            });
    }

    int hibf_gpu_hibf_emplace(hibf_gpu_hibf * h, uint64_t k, uint64_t const * values, uint64_t n, uint64_t bin)
    {
        return guarded(
            [&]
            {
                if (!h || k >= h->n_ibfs || (n && !values))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "bad argument");
                if (bin >= h->bins[k])
                    fail(HIBF_GPU_ERR_INVALID_ARG, "bin index out of range");
                if (!n)
                    return;
                std::lock_guard<std::mutex> lk(h->mu);
                h->io.ensure(n * 8);
                HG_CUDA(cudaMemcpyAsync(h->io.p, values, n * 8, cudaMemcpyHostToDevice, h->stream));
                dev_node const & nd = h->nodes[k];
                k_hibf_emplace<<<grid_cap(n, 256), 256, 0, h->stream>>>(
                    const_cast<uint64_t *>(nd.words), nd.bin_size, nd.row_words, nd.hash_shift, nd.hash_funs,
                    h->io.as<uint64_t>(), nullptr, n, bin, h->bins[k]);
                HG_CUDA(cudaGetLastError());
                HG_CUDA(cudaStreamSynchronize(h->stream));
            });
    }

    int hibf_gpu_hibf_set_prev(hibf_gpu_hibf * h, uint64_t const * prev_ibf, uint64_t const * prev_bin)
    {
        return guarded(
            [&]
            {
                if (!h || !prev_ibf || !prev_bin)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                for (uint64_t k = 0; k < h->n_ibfs; ++k)
                    if (prev_ibf[k] >= h->n_ibfs || prev_bin[k] >= h->bins[prev_ibf[k]])
                        fail(HIBF_GPU_ERR_INVALID_ARG, "prev_ibf_id out of range");
                std::lock_guard<std::mutex> lk(h->mu);
                h->prev_ibf.assign(prev_ibf, prev_ibf + h->n_ibfs);
                h->prev_bin.assign(prev_bin, prev_bin + h->n_ibfs);
            });
    }

    int hibf_gpu_hibf_get_prev(hibf_gpu_hibf const * h, uint64_t * prev_ibf, uint64_t * prev_bin)
    {
        return guarded(
            [&]
            {
                if (!h)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                std::lock_guard<std::mutex> lk(const_cast<hibf_gpu_hibf *>(h)->mu); // against a concurrent set_prev
                if (prev_ibf)
                    std::copy(h->prev_ibf.begin(), h->prev_ibf.end(), prev_ibf);
                if (prev_bin)
                    std::copy(h->prev_bin.begin(), h->prev_bin.end(), prev_bin);
            });
    }

    int hibf_gpu_hibf_save(hibf_gpu_hibf * h, char const * path)
    {
        return guarded(
            [&]
            {
                if (!h || !path)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                std::lock_guard<std::mutex> lk(h->mu);
                HG_CUDA(cudaStreamSynchronize(h->stream));
                file_writer w(path);
                w.u32(kArchiveVersion);
                w.u64(h->n_user_bins);
                w.u64(h->n_ibfs);
                for (uint64_t k = 0; k < h->n_ibfs; ++k)
                {
                    write_ibf_header(w, h->bins[k], h->bin_size[k], h->hash_funs[k]);
                    write_rows(w, h->stores[k]->as<uint64_t>(), h->bin_size[k], h->bin_words[k], h->row_words[k],
                               h->stream);
                    w.u64s(h->occupancy[k]);
                    w.u8(h->track_occupancy[k]);
                }
                uint64_t off = 0;
                auto per_ibf = [&](std::vector<uint64_t> const & flat)
                {
                    w.u64(h->n_ibfs);
                    off = 0;
                    for (uint64_t k = 0; k < h->n_ibfs; ++k)
                    {
                        w.u64(h->bins[k]);
                        w.raw(flat.data() + off, h->bins[k] * 8);
                        off += h->bins[k];
                    }
                };
                per_ibf(h->next_ibf_id);
                w.u64(h->n_ibfs);
                for (uint64_t k = 0; k < h->n_ibfs; ++k)
                {
                    w.u64(h->prev_ibf[k]);
                    w.u64(h->prev_bin[k]);
                }
                per_ibf(h->user_bin_id);
                w.close();
            });
    }

    int hibf_gpu_hibf_load(char const * path, hibf_gpu_hibf ** out)
    {
        return guarded(
            [&]
            {
                if (!path || !out)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                *out = nullptr;
                file_reader r(path);
                if (r.u32() != kArchiveVersion)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "archive: unsupported hierarchical_interleaved_bloom_filter version");
                uint64_t const nub = r.u64();
                uint64_t const n = r.u64();
                if (n == 0 || n > kNodeMask)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "archive: implausible number of IBFs");
                std::vector<uint64_t> bins(n), sizes(n), funs(n);
                std::vector<long> words_at(n);
                std::vector<std::vector<uint64_t>> occ(n);
                std::vector<uint8_t> track(n);
                for (uint64_t k = 0; k < n; ++k)
                {
                    ibf_header const hd = read_ibf_header(r);
                    bins[k] = hd.bins;
                    sizes[k] = hd.bin_size;
                    funs[k] = hd.hash_funs;
                    words_at[k] = r.tell();
                    r.skip(hd.bin_size * hd.bin_words * 8);
                    occ[k] = r.u64s(hd.technical_bins);
                    track[k] = r.u8();
                }
                auto per_ibf = [&]()
                {
                    if (r.u64() != n)
                        fail(HIBF_GPU_ERR_INVALID_ARG, "archive: table length differs from the IBF count");
                    std::vector<uint64_t> flat;
                    for (uint64_t k = 0; k < n; ++k)
                    {
                        std::vector<uint64_t> const v = r.u64s(bins[k]);
                        if (v.size() != bins[k])
                            fail(HIBF_GPU_ERR_INVALID_ARG, "archive: table row length differs from the IBF's bins");
                        flat.insert(flat.end(), v.begin(), v.end());
                    }
                    return flat;
                };
                std::vector<uint64_t> const next = per_ibf();
                if (r.u64() != n)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "archive: prev_ibf_id length differs from the IBF count");
                std::vector<uint64_t> prev_ibf(n), prev_bin(n);
                for (uint64_t k = 0; k < n; ++k)
                {
                    prev_ibf[k] = r.u64();
                    prev_bin[k] = r.u64();
                }
                std::vector<uint64_t> const ub = per_ibf();
                if (!r.at_end())
                    fail(HIBF_GPU_ERR_INVALID_ARG, "archive: trailing bytes");
                hibf_gpu_hibf * h = nullptr;
                int st = hibf_gpu_hibf_create(nub, n, bins.data(), sizes.data(), funs.data(), next.data(), ub.data(), &h);
                if (st != HIBF_GPU_OK)
                    fail(st, std::string(hibf_gpu_last_error()));
                try
                {
                    for (uint64_t k = 0; k < n; ++k)
                    {
                        r.seek(words_at[k]);
                        read_rows(r, h->stores[k]->as<uint64_t>(), h->bin_size[k], h->bin_words[k], h->row_words[k],
                                  h->stream);
                    }
                    st = hibf_gpu_hibf_set_prev(h, prev_ibf.data(), prev_bin.data());
                    if (st != HIBF_GPU_OK)
                        fail(st, std::string(hibf_gpu_last_error()));
                    h->occupancy = std::move(occ);
                    h->track_occupancy = std::move(track);
                }
                catch (...)
                {
                    hibf_gpu_hibf_destroy(h);
                    throw;
                }
                *out = h;
            });
    }

    int hibf_gpu_hibf_upload_words(hibf_gpu_hibf * h, uint64_t k, uint64_t const * words, uint64_t n_words)
    {
        return guarded(
            [&]
            {
                if (!h || k >= h->n_ibfs || !words)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "bad argument");
                if (n_words != h->bin_words[k] * h->bin_size[k])
                    fail(HIBF_GPU_ERR_INVALID_ARG, "word count does not match the IBF");
                std::lock_guard<std::mutex> lk(h->mu);
                HG_CUDA(cudaMemcpy2DAsync(h->stores[k]->p, h->row_words[k] * 8, words, h->bin_words[k] * 8,
                                          h->bin_words[k] * 8, h->bin_size[k], cudaMemcpyHostToDevice, h->stream));
                HG_CUDA(cudaStreamSynchronize(h->stream));
            });
    }

    int hibf_gpu_hibf_download_words(hibf_gpu_hibf * h, uint64_t k, uint64_t * words, uint64_t n_words)
    {
        return guarded(
            [&]
            {
                if (!h || k >= h->n_ibfs || !words)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "bad argument");
                if (n_words != h->bin_words[k] * h->bin_size[k])
                    fail(HIBF_GPU_ERR_INVALID_ARG, "word count does not match the IBF");
                std::lock_guard<std::mutex> lk(h->mu);
                HG_CUDA(cudaDeviceSynchronize());
                HG_CUDA(cudaMemcpy2DAsync(words, h->bin_words[k] * 8, h->stores[k]->p, h->row_words[k] * 8,
                                          h->bin_words[k] * 8, h->bin_size[k], cudaMemcpyDeviceToHost, h->stream));
                HG_CUDA(cudaStreamSynchronize(h->stream));
            });
    }

    int hibf_gpu_hibf_digests(hibf_gpu_hibf * h, uint64_t * out, uint32_t threads)
    {
        return guarded(
            [&]
            {
                if (!h || !out)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                std::lock_guard<std::mutex> lk(h->mu);
                HG_CUDA(cudaDeviceSynchronize());
                int dev = 0;
                HG_CUDA(cudaGetDevice(&dev));
                // IBFs largest first over the host threads; each thread folds its IBF's rows in order through a
                // pinned chunk of whole rows
                std::vector<uint64_t> order(h->n_ibfs);
                for (uint64_t k = 0; k < h->n_ibfs; ++k)
                    order[k] = k;
                std::sort(order.begin(), order.end(), [&](uint64_t a, uint64_t b)
                          { return h->bin_words[a] * h->bin_size[a] > h->bin_words[b] * h->bin_size[b]; });
                std::atomic<uint64_t> next{0};
                std::exception_ptr error;
                std::mutex error_lock;
                auto worker = [&]
                {
                    try
                    {
                        HG_CUDA(cudaSetDevice(dev));
                        cudaStream_t st{};
                        HG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
                        uint64_t const chunk_bytes = 64ull << 20;
                        void * buf = nullptr;
                        if (cudaHostAlloc(&buf, chunk_bytes, cudaHostAllocDefault) != cudaSuccess)
                        {
                            cudaStreamDestroy(st);
                            fail(HIBF_GPU_ERR_OUT_OF_MEMORY, "pinned staging buffer");
                        }
                        for (uint64_t i; (i = next.fetch_add(1)) < h->n_ibfs;)
                        {
                            uint64_t const k = order[i];
                            uint64_t const bw = h->bin_words[k], rows = h->bin_size[k];
                            uint64_t const per = std::max<uint64_t>(1, chunk_bytes / (bw * 8));
                            uint64_t d = HG_DIGEST_INIT;
                            for (uint64_t r = 0; r < rows; r += per)
                            {
                                uint64_t const n = std::min(per, rows - r);
                                auto const * src = static_cast<char const *>(h->stores[k]->p) + r * h->row_words[k] * 8;
                                HG_CUDA(cudaMemcpy2DAsync(buf, bw * 8, src, h->row_words[k] * 8, bw * 8, n,
                                                          cudaMemcpyDeviceToHost, st));
                                HG_CUDA(cudaStreamSynchronize(st));
                                auto const * w = static_cast<uint64_t const *>(buf);
                                for (uint64_t j = 0; j < n * bw; ++j)
                                    d = hg_digest_step(d, w[j]);
                            }
                            out[k] = d;
                        }
                        cudaFreeHost(buf);
                        cudaStreamDestroy(st);
                    }
                    catch (...)
                    {
                        std::lock_guard<std::mutex> g(error_lock);
                        if (!error)
                            error = std::current_exception();
                    }
                };
                unsigned const nt = static_cast<unsigned>(std::min<uint64_t>(
                    h->n_ibfs, threads ? threads : std::max(1u, std::thread::hardware_concurrency())));
                std::vector<std::thread> pool;
                for (unsigned t = 1; t < nt; ++t)
                    pool.emplace_back(worker);
                worker();
                for (std::thread & t : pool)
                    t.join();
                if (error)
                    std::rethrow_exception(error);
            });
    }

    int hibf_gpu_agent_create(hibf_gpu_hibf * h, hibf_gpu_agent ** out)
    {
        return guarded(
            [&]
            {
                if (!h || !out)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                *out = nullptr;
                auto a = new hibf_gpu_agent{};
                try
                {
                    a->h = h;
                    HG_CUDA(cudaStreamCreateWithFlags(&a->own, cudaStreamNonBlocking));
                    a->stream = a->own;
                    HG_CUDA(cudaEventCreate(&a->ev_k0));
                    HG_CUDA(cudaEventCreate(&a->ev_k1));
                    a->ctrl.ensure(C_WORDS * 8);
                    a->stats.ensure(kStats * 8);
                    a->h_ctrl.ensure(C_WORDS * 8);
                    a->h_stats.ensure(kStats * 8);
                    for (int v = 0; v < kQueryVariants; ++v)
                    {
                        int nb = 0;
                        HG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, query_kernel(h->hash_count, v), 256,
                                                                              query_smem(h)));
                        a->max_blocks[v] = std::max(1, nb);
                    }
                    {
                        int nb = 0;
                        HG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, query_block_kernel(h->hash_count),
                                                                              256, query_smem(h)));
                        a->max_blocks_blk = std::max(1, nb);
                    }
                    hibf_gpu_tuning_default(&a->tune);
                    ensure_capacity(a, 1024, 4096, 4096);
                }
                catch (...)
                {
                    if (a->own)
                        cudaStreamDestroy(a->own);
                    delete a;
                    throw;
                }
                *out = a;
            });
    }

    int hibf_gpu_agent_destroy(hibf_gpu_agent * a)
    {
        return guarded(
            [&]
            {
                if (!a)
                    return;
                cudaStreamSynchronize(a->stream);
                if (a->graph)
                    cudaGraphExecDestroy(a->graph);
                cudaEventDestroy(a->ev_k0);
                cudaEventDestroy(a->ev_k1);
                if (a->tl_t0)
                {
                    cudaEventDestroy(a->tl_t0);
                    cudaEventDestroy(a->tl_done);
                }
                for (cudaEvent_t e : a->tl_chunk)
                    cudaEventDestroy(e);
                for (cudaEvent_t e : a->ev_lvl)
                    cudaEventDestroy(e);
                if (a->copy_stream)
                {
                    cudaStreamSynchronize(a->copy_stream);
                    cudaEventDestroy(a->ev_ready);
                    cudaEventDestroy(a->ev_copied);
                    cudaStreamDestroy(a->copy_stream);
                }
                cudaStreamDestroy(a->own);
                delete a;
            });
    }

    int hibf_gpu_agent_set_stream(hibf_gpu_agent * a, void * stream)
    {
        return guarded(
            [&]
            {
                if (!a)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                a->stream = stream ? static_cast<cudaStream_t>(stream) : a->own;
            });
    }

    int hibf_gpu_agent_reserve(hibf_gpu_agent * a, uint64_t max_queries, uint64_t max_values, uint64_t max_tasks,
                               uint64_t max_results)
    {
        return guarded(
            [&]
            {
                if (!a)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                ensure_capacity(a, std::max<uint64_t>(max_queries, 1), std::max<uint64_t>(max_tasks, 1),
                                std::max<uint64_t>(max_results, 1));
                a->in_values.ensure(max_values * 8);
                a->in_qoff.ensure((max_queries + 1) * 8);
                a->in_thr.ensure(std::max<uint64_t>(max_queries, 1) * 8);
            });
    }

    int hibf_gpu_agent_membership_for(hibf_gpu_agent * a, uint64_t const * values, uint64_t n, uint16_t threshold,
                                      uint64_t const ** ids, uint64_t * n_ids)
    {
        return guarded(
            [&]
            {
                if (!a || (n && !values) || !ids || !n_ids)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                uint64_t const qoff[2] = {0, n};
                uint64_t const thr = threshold;
                host_batch(a, HIBF_GPU_QUERY_MEMBERSHIP, values, qoff, 1, &thr, 2, true);
                uint64_t const nr = a->h_roff.as<uint64_t>()[1];
                a->single_ids.assign(a->h_ids.as<uint64_t>(), a->h_ids.as<uint64_t>() + nr);
                *ids = a->single_ids.data();
                *n_ids = nr;
            });
    }

    int hibf_gpu_agent_membership_for_unsorted(hibf_gpu_agent * a, uint64_t const * values, uint64_t n,
                                               uint16_t threshold, uint64_t const ** ids, uint64_t * n_ids)
    {
        return guarded(
            [&]
            {
                if (!a || (n && !values) || !ids || !n_ids)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                uint64_t const qoff[2] = {0, n};
                uint64_t const thr = threshold;
                host_batch(a, HIBF_GPU_QUERY_MEMBERSHIP, values, qoff, 1, &thr, 2, true);
                uint64_t const nr = a->h_roff.as<uint64_t>()[1];
                a->single_ids.assign(a->h_ids.as<uint64_t>(), a->h_ids.as<uint64_t>() + nr);
                std::vector<uint64_t> const & rank = traversal_rank(a->h);
                std::sort(a->single_ids.begin(), a->single_ids.end(),
                          [&](uint64_t x, uint64_t y) { return rank[x] < rank[y]; });
                *ids = a->single_ids.data();
                *n_ids = nr;
            });
    }

    int hibf_gpu_agent_bulk_count(hibf_gpu_agent * a, uint64_t const * values, uint64_t n, uint64_t threshold,
                                  int width, void const ** counts)
    {
        return guarded(
            [&]
            {
                if (!a || (n && !values) || !counts)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                uint64_t const qoff[2] = {0, n};
                host_batch(a, HIBF_GPU_QUERY_COUNT, values, qoff, 1, &threshold, width, true);
                uint64_t const nr = a->h_roff.as<uint64_t>()[1];
                a->dense.assign(a->h->n_user_bins * static_cast<size_t>(width), 0);
                uint8_t const * src = a->h_cnt.as<uint8_t>();
                uint64_t const * ids = a->h_ids.as<uint64_t>();
                for (uint64_t i = 0; i < nr; ++i)
                    std::memcpy(a->dense.data() + ids[i] * width, src + i * width, width);
                *counts = a->dense.data();
            });
    }

    int hibf_gpu_agent_query_batch(hibf_gpu_agent * a, int mode, uint64_t const * values,
                                   uint64_t const * query_offsets, uint64_t n_queries, uint64_t const * thresholds,
                                   int width, uint64_t const ** result_offsets, uint64_t const ** result_ids,
                                   void const ** result_counts)
    {
        return guarded(
            [&]
            {
                if (!a || !query_offsets || (n_queries && !thresholds) || !result_offsets || !result_ids)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                if (n_queries >= 0xFFFFFFFFull)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "at most 2^32 - 1 queries per batch");
                if (n_queries && query_offsets[n_queries] && !values)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null values");
                host_batch(a, mode, values, query_offsets, n_queries, thresholds, width, false);
                *result_offsets = a->h_roff.as<uint64_t>();
                *result_ids = a->h_ids.as<uint64_t>();
                if (result_counts)
                    *result_counts = mode == HIBF_GPU_QUERY_COUNT ? a->h_cnt.p : nullptr;
            });
    }

    int hibf_gpu_agent_query_batch_d(hibf_gpu_agent * a, int mode, uint64_t const * d_values,
                                     uint64_t const * d_query_offsets, uint64_t n_queries,
                                     uint64_t const * d_thresholds, int width, uint64_t const ** d_result_offsets,
                                     uint64_t const ** d_result_ids, void const ** d_result_counts)
    {
        return guarded(
            [&]
            {
                if (!a || !d_query_offsets || (n_queries && (!d_thresholds || !d_values)))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                if (n_queries >= 0xFFFFFFFFull)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "at most 2^32 - 1 queries per batch");
                check_mode(mode, width, nullptr, 0);
                ensure_capacity(a, std::max<uint64_t>(n_queries, 1), std::max<uint64_t>(a->cap_tasks, 1024),
                                std::max<uint64_t>(a->cap_results, 1024));
                launch_batch(a, mode, d_values, d_query_offsets, d_thresholds, n_queries, width);
                if (d_result_offsets)
                    *d_result_offsets = a->roff.as<uint64_t>();
                if (d_result_ids)
                    *d_result_ids = a->out_ids.as<uint64_t>();
                if (d_result_counts)
                    *d_result_counts = mode == HIBF_GPU_QUERY_COUNT ? (width == 8 ? a->out_cnt.p : a->out_cntw.p)
                                                                   : nullptr;
            });
    }

    int hibf_gpu_agent_query_plain_d(hibf_gpu_agent * a, int mode, uint64_t const * d_values,
                                     uint64_t const * h_query_offsets, uint64_t n_queries,
                                     uint64_t const * h_thresholds, int width)
    {
        return guarded(
            [&]
            {
                if (!a || !h_query_offsets || (n_queries && (!h_thresholds || !d_values)))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                check_mode(mode, width, h_thresholds, n_queries);
                ensure_capacity(a, std::max<uint64_t>(n_queries, 1), std::max<uint64_t>(a->cap_tasks, 1024),
                                std::max<uint64_t>(a->cap_results, 1024));
                a->in_qoff.ensure((n_queries + 1) * 8);
                a->in_thr.ensure(std::max<uint64_t>(n_queries, 1) * 8);
                HG_CUDA(cudaMemcpyAsync(a->in_qoff.p, h_query_offsets, (n_queries + 1) * 8, cudaMemcpyHostToDevice,
                                        a->stream));
                if (n_queries)
                    HG_CUDA(cudaMemcpyAsync(a->in_thr.p, h_thresholds, n_queries * 8, cudaMemcpyHostToDevice,
                                            a->stream));
                launch_plain(a, mode, d_values, h_query_offsets, a->in_qoff.as<uint64_t>(), a->in_thr.as<uint64_t>(),
                             n_queries, width);
            });
    }

    int hibf_gpu_agent_fetch_results(hibf_gpu_agent * a, uint64_t n_queries, int mode, int width,
                                     uint64_t const ** result_offsets, uint64_t const ** result_ids,
                                     void const ** result_counts)
    {
        return guarded(
            [&]
            {
                if (!a || !result_offsets || !result_ids)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                if (n_queries > a->cap_queries)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "more queries than the agent's last batch can hold");
                check_mode(mode, width, nullptr, 0);
                int const st = read_status(a);
                if (st != HIBF_GPU_OK)
                    fail(st, "device-side failure in the last batch");
                a->h_roff.ensure((n_queries + 1) * 8);
                HG_CUDA(cudaMemcpyAsync(a->h_roff.p, a->roff.p, (n_queries + 1) * 8, cudaMemcpyDeviceToHost,
                                        a->stream));
                HG_CUDA(cudaStreamSynchronize(a->stream));
                uint64_t const nr = a->h_roff.as<uint64_t>()[n_queries];
                a->h_ids.ensure(nr * 8);
                a->h_cnt.ensure(nr * 8);
                if (nr)
                {
                    HG_CUDA(cudaMemcpyAsync(a->h_ids.p, a->out_ids.p, nr * 8, cudaMemcpyDeviceToHost, a->stream));
                    if (mode == HIBF_GPU_QUERY_COUNT)
                        HG_CUDA(cudaMemcpyAsync(a->h_cnt.p, width == 8 ? a->out_cnt.p : a->out_cntw.p, nr * width,
                                                cudaMemcpyDeviceToHost, a->stream));
                }
                HG_CUDA(cudaStreamSynchronize(a->stream));
                *result_offsets = a->h_roff.as<uint64_t>();
                *result_ids = a->h_ids.as<uint64_t>();
                if (result_counts)
                    *result_counts = mode == HIBF_GPU_QUERY_COUNT ? a->h_cnt.p : nullptr;
            });
    }

    int hibf_gpu_agent_capture_batch_d(hibf_gpu_agent * a, int mode, uint64_t const * d_values,
                                       uint64_t const * d_query_offsets, uint64_t n_queries,
                                       uint64_t const * d_thresholds, int width)
    {
        return guarded(
            [&]
            {
                if (!a || !d_query_offsets || (n_queries && (!d_thresholds || !d_values)))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                if (n_queries >= 0xFFFFFFFFull)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "at most 2^32 - 1 queries per batch");
                check_mode(mode, width, nullptr, 0);
                ensure_capacity(a, std::max<uint64_t>(n_queries, 1), std::max<uint64_t>(a->cap_tasks, 1024),
                                std::max<uint64_t>(a->cap_results, 1024));
                HG_CUDA(cudaStreamSynchronize(a->stream));
                if (a->graph)
                {
                    HG_CUDA(cudaGraphExecDestroy(a->graph));
                    a->graph = nullptr;
                }
                (void)sm_count();
                cudaGraph_t g = nullptr;
                HG_CUDA(cudaStreamBeginCapture(a->stream, cudaStreamCaptureModeThreadLocal));
                try
                {
                    launch_batch(a, mode, d_values, d_query_offsets, d_thresholds, n_queries, width);
                }
                catch (...)
                {
                    cudaStreamEndCapture(a->stream, &g);
                    if (g)
                        cudaGraphDestroy(g);
                    throw;
                }
                HG_CUDA(cudaStreamEndCapture(a->stream, &g));
                cudaError_t const e = cudaGraphInstantiate(&a->graph, g, 0);
                cudaGraphDestroy(g);
                HG_CUDA(e);
            });
    }

    int hibf_gpu_agent_replay(hibf_gpu_agent * a)
    {
        return guarded(
            [&]
            {
                if (!a || !a->graph)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "no captured batch");
                HG_CUDA(cudaGraphLaunch(a->graph, a->stream));
            });
    }

    int hibf_gpu_agent_kernel_ms(hibf_gpu_agent * a, float * ms)
    {
        return guarded(
            [&]
            {
                if (!a || !ms)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                HG_CUDA(cudaEventSynchronize(a->ev_k1));
                HG_CUDA(cudaEventElapsedTime(ms, a->ev_k0, a->ev_k1));
            });
    }

    int hibf_gpu_stream_plan(uint64_t const * query_offsets, uint64_t n_queries, uint64_t * first_queries,
                             uint64_t cap, uint64_t * n)
    {
        return guarded(
            [&]
            {
                if (!query_offsets || !n || (cap && !first_queries))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                for (uint64_t q = 0; q < n_queries; ++q)
                    if (query_offsets[q + 1] < query_offsets[q])
                        fail(HIBF_GPU_ERR_INVALID_ARG, "query offsets must be non-decreasing");
                std::vector<uint64_t> qb;
                if (n_queries && query_offsets[n_queries] * 8 >= kStreamMinBytes)
                    qb = stream_chunks(query_offsets, n_queries);
                *n = qb.size();
                std::copy(qb.begin(), qb.begin() + static_cast<std::ptrdiff_t>(std::min<uint64_t>(cap, qb.size())),
                          first_queries);
            });
    }

    int hibf_gpu_agent_level_ms(hibf_gpu_agent * a, float * ms, uint32_t cap, uint32_t * n)
    {
        return guarded(
            [&]
            {
                if (!a || !n || (cap && !ms))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                *n = a->last_levels;
                if (a->last_levels == 0)
                    return;
                HG_CUDA(cudaEventSynchronize(a->ev_lvl[a->last_levels - 1]));
                for (uint32_t d = 0; d < std::min(cap, a->last_levels); ++d)
                    HG_CUDA(cudaEventElapsedTime(ms + d, d ? a->ev_lvl[d - 1] : a->ev_k0, a->ev_lvl[d]));
            });
    }

    int hibf_gpu_agent_set_host_read(hibf_gpu_agent * a, int in_place)
    {
        return guarded(
            [&]
            {
                if (!a)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                a->host_read = in_place != 0;
            });
    }

    int hibf_gpu_agent_last_in_place(hibf_gpu_agent const * a, int * in_place)
    {
        return guarded(
            [&]
            {
                if (!a || !in_place)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                *in_place = a->last_in_place ? 1 : 0;
            });
    }

    int hibf_gpu_agent_level_work(hibf_gpu_agent * a, uint64_t * tasks, uint64_t * value_visits,
                                  uint64_t * value_visits_executed, uint32_t cap, uint32_t * n)
    {
        return guarded(
            [&]
            {
                if (!a || !n || (cap && (!tasks || !value_visits || !value_visits_executed)))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                (void)read_status(a);
                uint32_t const levels = static_cast<uint32_t>(a->last_level_stats.size() / kStats);
                *n = levels;
                for (uint32_t d = 0; d < std::min(cap, levels); ++d)
                {
                    tasks[d] = a->last_level_stats[d * kStats + 0];
                    value_visits[d] = a->last_level_stats[d * kStats + 1];
                    value_visits_executed[d] = a->last_level_stats[d * kStats + 2];
                }
            });
    }

    int hibf_gpu_agent_last_timeline(hibf_gpu_agent const * a, double * out_ms, uint32_t cap, uint32_t * n)
    {
        return guarded(
            [&]
            {
                if (!a || !n || (cap && !out_ms))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                if (!a->tl_t0 || a->tl_n == 0)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "the agent has not answered a host batch");
                *n = a->tl_n + 3;
                auto since = [&](cudaEvent_t e)
                {
                    float ms = 0;
                    HG_CUDA(cudaEventElapsedTime(&ms, a->tl_t0, e));
                    return static_cast<double>(ms);
                };
                std::vector<double> t;
                for (uint32_t k = 0; k < a->tl_n; ++k)
                    t.push_back(since(a->tl_chunk[k]));
                t.push_back(since(a->ev_k0));
                t.push_back(since(a->ev_k1));
                t.push_back(since(a->tl_done));
                for (uint32_t i = 0; i < std::min<uint32_t>(cap, *n); ++i)
                    out_ms[i] = t[i];
            });
    }

    int hibf_gpu_agent_input_chunks(hibf_gpu_agent const * a, uint32_t * chunks)
    {
        return guarded(
            [&]
            {
                if (!a || !chunks)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                *chunks = a->last_chunks;
            });
    }

    int hibf_gpu_agent_selftest_wait_limit(hibf_gpu_agent * a, double limit_ms)
    {
        return guarded(
            [&]
            {
                if (!a || !(limit_ms > 0) || limit_ms > 10000)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "limit must be in (0, 10000] ms");
                cudaStream_t s = a->stream;
                ensure_capacity(a, 1, std::max<uint64_t>(a->cap_tasks, 1024), std::max<uint64_t>(a->cap_results, 1024));
                a->in_values.ensure(8);
                a->in_qoff.ensure(16);
                a->in_thr.ensure(8);
                HG_CUDA(cudaMemsetAsync(a->in_qoff.p, 0, 16, s));
                // no query, but one task announced that nobody will ever push: every worker's wait must expire
                k_init_ctrl<<<1, 32, 0, s>>>(a->ctrl.as<unsigned long long>(), a->stats.as<unsigned long long>(), 1);
                HG_CUDA(cudaGetLastError());
                HG_CUDA(cudaMemsetAsync(a->tasks.p, 0xFF, a->cap_tasks * 8, s));
                query_params p = base_params(a, a->in_values.as<uint64_t>(), a->in_qoff.as<uint64_t>(),
                                             a->in_thr.as<uint64_t>(), 0, 0xFFFFu);
                p.wait_limit_ns = static_cast<uint64_t>(limit_ms * 1e6);
                query_kernel(a->h->hash_count, a->variant)<<<1, 256, query_smem(a->h), s>>>(p);
                HG_CUDA(cudaGetLastError());
                int const st = read_status(a);
                if (st != HIBF_GPU_ERR_TIMEOUT)
                    fail(HIBF_GPU_ERR_CUDA, "the bounded wait did not report a timeout");
            });
    }

    int hibf_gpu_set_l2_fetch_granularity(int bytes)
    {
        return guarded(
            [&]
            {
                if (bytes < 0 || bytes > 128)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "L2 fetch granularity must be in [0, 128] bytes");
                require_device();
                HG_CUDA(cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, static_cast<size_t>(bytes)));
            });
    }

    int hibf_gpu_agent_status(hibf_gpu_agent * a)
    {
        if (!a)
            return HIBF_GPU_ERR_INVALID_ARG;
        return guarded(
            [&]
            {
                int const st = read_status(a);
                if (st != HIBF_GPU_OK)
                    fail(st, "device-side failure in the last batch");
            });
    }

    int hibf_gpu_agent_last_work_executed(hibf_gpu_agent * a, uint64_t * value_visits_executed)
    {
        return guarded(
            [&]
            {
                if (!a || !value_visits_executed)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                (void)read_status(a);
                *value_visits_executed = a->last_executed;
            });
    }

    int hibf_gpu_agent_last_work(hibf_gpu_agent * a, uint64_t * tasks, uint64_t * value_visits)
    {
        return guarded(
            [&]
            {
                if (!a)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                (void)read_status(a);
                if (tasks)
                    *tasks = a->last_tasks;
                if (value_visits)
                    *value_visits = a->last_visits;
            });
    }

} // extern "C"
