// hibf_internal.cuh -- the HIBF object shared by the query (hibf.cu) and build (build.cu) translation units.
#pragma once

#include <cstdint>
#include <memory>
#include <mutex>
#include <vector>

#include "common.hpp"

namespace hibf_gb300
{

// One IBF of the hierarchy as the query kernel sees it.
struct alignas(16) dev_node
{
    uint64_t const * words;
    uint64_t bin_size;
    uint32_t bins;
    uint32_t bin_words;
    uint32_t row_words;
    uint32_t hash_shift;
    uint32_t hash_funs;
    uint32_t desc_offset;
    uint32_t lpv_log2;
    uint32_t pad;
};


int sm_count();

// One build phase's time, kept like the reference's concurrent_timer (include/hibf/misc/timer.hpp): the seconds of
// all intervals, the longest interval and the number of intervals.
struct phase_timer
{
    double seconds{};
    double max_seconds{};
    uint64_t count{};
    void add(double s)
    {
        seconds += s;
        max_seconds = s > max_seconds ? s : max_seconds;
        ++count;
    }
};
enum : int
{
    timer_index_allocation,
    timer_user_bin_io,
    timer_merge_kmers,
    timer_fill_ibf,
    n_timers
};

} // namespace hibf_gb300

struct hibf_gpu_hibf
{
    uint64_t n_user_bins{};
    uint64_t n_ibfs{};
    uint32_t max_depth{};
    uint32_t hash_count{}; // number of hash functions, the same for every IBF
    uint32_t counters_per_warp{};
    uint64_t total_bytes{};
    std::vector<hibf_gb300::dev_node> nodes;           // host copy
    std::vector<std::unique_ptr<hibf_gb300::dbuf>> stores;
    std::vector<uint64_t> bins, bin_size, hash_funs, bin_words, row_words;
    hibf_gb300::dbuf d_nodes;
    hibf_gb300::dbuf d_descs;
    hibf_gb300::dbuf io;
    // the tables as given (reference conventions), for hibf_gpu_hibf_get_tables
    std::vector<uint64_t> next_ibf_id, user_bin_id;
    // prev_ibf_id (parent IBF and bin of every IBF) and each IBF's occupancy / track_occupancy, kept on the host for
    // serialisation only (queries use neither)
    std::vector<uint64_t> prev_ibf, prev_bin;
    std::vector<std::vector<uint64_t>> occupancy;
    std::vector<uint8_t> track_occupancy;
    // every user bin's position in membership_for's traversal order (computed on first use, under `mu`)
    std::vector<uint64_t> trav_rank;
    // the build's phase timers (zero unless built by hibf_gpu_hibf_build / _build_synthetic)
    hibf_gb300::phase_timer timers[hibf_gb300::n_timers];
    cudaStream_t stream{};
    std::mutex mu;
};

