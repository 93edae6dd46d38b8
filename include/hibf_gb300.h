/* hibf_gb300.h -- C ABI of the GB300-native HIBF build/query path.
 *
 * This is the drop-in boundary: plain pointers, sizes and status codes, no C++ or torch types.  A seqan::hibf
 * build keeps its host-side config, layout DP, HyperLogLog sketching and serialization; it hands the device the
 * interleaved bit store and the per-IBF tables, routes emplace() through the batched insert entry points, and
 * replaces its agents' query calls with the entry points below.  Each declaration names the reference interface it
 * replaces (file:line inside the seqan/hibf tree).
 *
 * Conventions
 *   - Functions without a suffix take HOST pointers and are synchronous, like the reference's member functions.
 *   - Functions ending in _d take DEVICE pointers and a cudaStream_t passed as void*; they are asynchronous and
 *     report device-side failures (result overflow, a bounded wait that expired) through the owning object's
 *     status, read with hibf_gpu_agent_status / hibf_gpu_ibf_status after the stream has been synchronised.
 *   - Every function returns an int status (enum hibf_gpu_status).  hibf_gpu_last_error() describes the last
 *     failure of the calling thread.
 *   - Counter widths are given in bytes (1, 2, 4, 8) and select counting_agent<uint8_t .. uint64_t>; counts wrap
 *     modulo 2^(8*width) exactly as the reference's counting_vector does.
 *   - The library never falls back to a CPU path: without a usable CUDA device every call that needs one fails
 *     with HIBF_GPU_ERR_NO_DEVICE.
 */
#ifndef HIBF_GB300_H
#define HIBF_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HIBF_GPU_ABI_VERSION 1

enum hibf_gpu_status
{
    HIBF_GPU_OK = 0,
    HIBF_GPU_ERR_INVALID_ARG = 1,   /* std::invalid_argument in the reference (config.cpp:66-129, IBF.cpp:165) */
    HIBF_GPU_ERR_LOGIC = 2,         /* std::logic_error in the reference (IBF.cpp:41-46)                       */
    HIBF_GPU_ERR_OUT_OF_MEMORY = 3, /* device or pinned-host allocation failed                                */
    HIBF_GPU_ERR_NO_DEVICE = 4,     /* no CUDA device / driver                                                 */
    HIBF_GPU_ERR_CUDA = 5,          /* any other CUDA runtime error                                            */
    HIBF_GPU_ERR_OVERFLOW = 6,      /* result or task capacity of a batch exceeded; nothing was lost silently */
    HIBF_GPU_ERR_TIMEOUT = 7,       /* a bounded device-side wait expired; the context stays usable           */
    HIBF_GPU_ERR_ADMISSION = 8,     /* request rejected by the serving loop's memory admission cap            */
    HIBF_GPU_ERR_CYCLE = 9          /* a merged bin leads back into its own subtree (descent depth exceeded)  */
};

/* Sentinels of ibf_bin_to_user_bin_id (include/hibf/hierarchical_interleaved_bloom_filter.hpp:32-40). */
#define HIBF_GPU_BIN_MERGED UINT64_MAX
#define HIBF_GPU_BIN_DELETED (UINT64_MAX - 1u)

const char * hibf_gpu_last_error(void);
int hibf_gpu_abi_version(void);
/* Number of usable CUDA devices (0 when none); selects nothing. */
int hibf_gpu_device_count(int * count);

/* ============================================================================================================ */
/* Single-level interleaved Bloom filter: seqan::hibf::interleaved_bloom_filter                                  */
/* ============================================================================================================ */
typedef struct hibf_gpu_ibf hibf_gpu_ibf;

/* interleaved_bloom_filter(bin_count, bin_size, hash_function_count, track_occupancy)
 * (include/hibf/interleaved_bloom_filter.hpp:225-228, src/interleaved_bloom_filter.cpp:32-53).
 * Zeroed device bit store of bin_size rows x technical_bins bits, technical_bins = 64 * ceil(bins / 64).
 * HIBF_GPU_ERR_LOGIC for bins == 0, hash_funs not in [1,5] or bin_size == 0. */
int hibf_gpu_ibf_create(uint64_t bins, uint64_t bin_size, uint64_t hash_funs, int track_occupancy,
                        hibf_gpu_ibf ** out);
int hibf_gpu_ibf_destroy(hibf_gpu_ibf * ibf);

/* bin_count(), bin_size(), hash_function_count(), bit_size() (interleaved_bloom_filter.hpp:395-425);
 * out[4] = device row stride in bytes (rows are padded so that none straddles a 32-byte sector). */
int hibf_gpu_ibf_info(hibf_gpu_ibf const * ibf, uint64_t out[5]);

/* emplace(value, bin) for n values into one bin (src/interleaved_bloom_filter.cpp:119-140; the insert_iterator IBF
 * branch, include/hibf/misc/insert_iterator.hpp:60-81).  Bits are set with atomicOr, so the result does not depend
 * on the order of the values. */
int hibf_gpu_ibf_emplace(hibf_gpu_ibf * ibf, uint64_t const * values, uint64_t n, uint64_t bin);
/* emplace(values[i], bins[i]) for i < n. */
int hibf_gpu_ibf_emplace_binned(hibf_gpu_ibf * ibf, uint64_t const * values, uint64_t const * bins, uint64_t n);
/* Device-pointer form; d_bins == NULL means every value goes to `bin`. */
int hibf_gpu_ibf_emplace_d(hibf_gpu_ibf * ibf, uint64_t const * d_values, uint64_t const * d_bins, uint64_t n,
                           uint64_t bin, void * stream);

/* clear(bin_index) (src/interleaved_bloom_filter.cpp:142-148) and clear(range) (interleaved_bloom_filter.hpp:283-297). */
int hibf_gpu_ibf_clear(hibf_gpu_ibf * ibf, uint64_t bin);
int hibf_gpu_ibf_clear_range(hibf_gpu_ibf * ibf, uint64_t const * bins, uint64_t n);

/* try_increase_bin_number_to / increase_bin_number_to (src/interleaved_bloom_filter.cpp:150-202). */
int hibf_gpu_ibf_try_increase_bin_number_to(hibf_gpu_ibf * ibf, uint64_t new_bins, int * increased);
int hibf_gpu_ibf_increase_bin_number_to(hibf_gpu_ibf * ibf, uint64_t new_bins);

/* containment_agent_type::bulk_contains (src/interleaved_bloom_filter.cpp:204-291) for n values:
 * out receives n * ceil(bins/64) words, the bit_vector words of each value's result. */
int hibf_gpu_ibf_bulk_contains(hibf_gpu_ibf * ibf, uint64_t const * values, uint64_t n, uint64_t * out);
int hibf_gpu_ibf_bulk_contains_d(hibf_gpu_ibf * ibf, uint64_t const * d_values, uint64_t n, uint64_t * d_out,
                                 void * stream);

/* counting_agent_type<value_t>::bulk_count (include/hibf/interleaved_bloom_filter.hpp:652-665): one counting vector
 * of `bins` counters of `width` bytes over all n values. */
int hibf_gpu_ibf_bulk_count(hibf_gpu_ibf * ibf, uint64_t const * values, uint64_t n, int width, void * out);
int hibf_gpu_ibf_bulk_count_d(hibf_gpu_ibf * ibf, uint64_t const * d_values, uint64_t n, int width, void * d_out,
                              void * stream);

/* No counterpart in the reference.  hibf_gpu_ibf_bulk_count_d for callers that cannot allocate device memory:
 * a process whose device memory is all held by its own pool (a framework's caching allocator), or a loop where
 * cudaMalloc's implicit device-wide synchronisation is not acceptable.  The counting scratch is a fixed static
 * device array of HIBF_GPU_NOALLOC_MAX_BINS 64-bit totals (128 KiB, held by every device that loads the library
 * until exit); filters with more bins are rejected with HIBF_GPU_ERR_INVALID_ARG.  The call allocates nothing.
 * Its first call on a device looks the array's address up and keeps it for the life of the process (make that call
 * before any stream capture; resetting the device afterwards, e.g. cudaDeviceReset, is not supported).  It counts
 * exactly like hibf_gpu_ibf_bulk_count_d (the same launch, with the static array as its scratch).  All calls share
 * the array: calls that overlap on the GPU race; each call clears the totals it uses first. */
#define HIBF_GPU_NOALLOC_MAX_BINS 16384
int hibf_gpu_ibf_bulk_count_noalloc_d(hibf_gpu_ibf * ibf, uint64_t const * d_values, uint64_t n, int width,
                                      void * d_out, void * stream);

/* membership_agent_type::membership_for (include/hibf/interleaved_bloom_filter.hpp:744-764): ascending bin ids whose
 * uint16 count reaches `threshold`.  out_ids needs room for `bins` ids; *n_out receives the count. */
int hibf_gpu_ibf_membership_for(hibf_gpu_ibf * ibf, uint64_t const * values, uint64_t n, uint16_t threshold,
                                uint64_t * out_ids, uint64_t * n_out);

/* The bit store in the reference's bit_vector word layout (row r = words [r*ceil(bins/64), ...)), for
 * serialization through the host (interleaved_bloom_filter.hpp:471-485, bit_vector.hpp:885-925). */
int hibf_gpu_ibf_upload_words(hibf_gpu_ibf * ibf, uint64_t const * words, uint64_t n_words);
int hibf_gpu_ibf_download_words(hibf_gpu_ibf * ibf, uint64_t * words, uint64_t n_words);
/* occupancy vector (interleaved_bloom_filter.hpp:433-437): technical_bins counters. */
int hibf_gpu_ibf_download_occupancy(hibf_gpu_ibf * ibf, uint64_t * out, uint64_t n);
/* track_occupancy (interleaved_bloom_filter.hpp:457-458): 1 when emplace counts newly set bits, else 0. */
int hibf_gpu_ibf_track_occupancy(hibf_gpu_ibf const * ibf, int * out);
/* Status of the last asynchronous (_d) call on this filter. */
int hibf_gpu_ibf_status(hibf_gpu_ibf * ibf);

/* ============================================================================================================ */
/* Hierarchical interleaved Bloom filter: seqan::hibf::hierarchical_interleaved_bloom_filter                     */
/* ============================================================================================================ */
typedef struct hibf_gpu_hibf hibf_gpu_hibf;

/* The HIBF's tables (hierarchical_interleaved_bloom_filter.hpp:208-238) plus one empty IBF per entry of ibf_vector,
 * sized like construct_ibf does (src/build/construct_ibf.cpp:52-55):
 *   bins[k], bin_sizes[k], hash_funs[k]       interleaved_bloom_filter(bin_count, bin_size, hash_function_count)
 *   next_ibf_id / user_bin_id                 next_ibf_id[k][b] and ibf_bin_to_user_bin_id[k][b], flattened in IBF
 *                                             order, sum(bins) entries each; HIBF_GPU_BIN_MERGED / _DELETED sentinels
 * IBF 0 is the root.  n_user_bins must be below 2^32 - 2. */
int hibf_gpu_hibf_create(uint64_t n_user_bins, uint64_t n_ibfs, uint64_t const * bins, uint64_t const * bin_sizes,
                         uint64_t const * hash_funs, uint64_t const * next_ibf_id, uint64_t const * user_bin_id,
                         hibf_gpu_hibf ** out);
int hibf_gpu_hibf_destroy(hibf_gpu_hibf * h);
/* out: n_user_bins, n_ibfs, max depth, total device bytes of the bit stores. */
int hibf_gpu_hibf_info(hibf_gpu_hibf const * h, uint64_t out[4]);
/* Per IBF: bins, technical bins, bin_size, hash_funs, device row stride in bytes. */
int hibf_gpu_hibf_ibf_info(hibf_gpu_hibf const * h, uint64_t ibf, uint64_t out[5]);

/* emplace into IBF `ibf` (insert_into_ibf, src/build/insert_into_ibf.cpp:28-84): host values into one bin, or
 * device values with per-value bins (d_bins) or one bin. */
int hibf_gpu_hibf_emplace(hibf_gpu_hibf * h, uint64_t ibf, uint64_t const * values, uint64_t n, uint64_t bin);
int hibf_gpu_hibf_emplace_d(hibf_gpu_hibf * h, uint64_t ibf, uint64_t const * d_values, uint64_t const * d_bins,
                            uint64_t n, uint64_t bin, void * stream);
/* The tables as given at creation (reference conventions): bins / bin_sizes / hash_funs have n_ibfs entries,
 * next_ibf_id / user_bin_id sum(bins) entries.  Any pointer may be NULL. */
int hibf_gpu_hibf_get_tables(hibf_gpu_hibf const * h, uint64_t * bins, uint64_t * bin_sizes, uint64_t * hash_funs,
                             uint64_t * next_ibf_id, uint64_t * user_bin_id);
/* Words of IBF `ibf` in the reference's bit_vector layout (for serialization or a host-built HIBF). */
int hibf_gpu_hibf_upload_words(hibf_gpu_hibf * h, uint64_t ibf, uint64_t const * words, uint64_t n_words);
/* prev_ibf_id (hierarchical_interleaved_bloom_filter.hpp:222-229): parent IBF and bin of every IBF.  Created
 * hierarchies give every merged bin's child its parent and the root (0, 0); the build leaves the reference's
 * convention ((0, 0) also for favourite children); set it to carry a host-built HIBF's table through serialisation. */
int hibf_gpu_hibf_set_prev(hibf_gpu_hibf * h, uint64_t const * prev_ibf, uint64_t const * prev_bin);
/* The same table read back: n_ibfs entries each; either pointer may be NULL. */
int hibf_gpu_hibf_get_prev(hibf_gpu_hibf const * h, uint64_t * prev_ibf, uint64_t * prev_bin);
/* Serialisation in the reference's byte layout (cereal binary archive encoding of the serialize functions of
 * interleaved_bloom_filter.hpp:471-485 with bit_vector.hpp:885-925, and hierarchical_interleaved_bloom_filter.hpp:
 * 267-277): save streams the device stores to `path`, load reads one into new device stores.  Invalid or
 * inconsistent archives fail with HIBF_GPU_ERR_INVALID_ARG. */
int hibf_gpu_ibf_save(hibf_gpu_ibf * ibf, char const * path);
int hibf_gpu_ibf_load(char const * path, hibf_gpu_ibf ** out);
int hibf_gpu_hibf_save(hibf_gpu_hibf * h, char const * path);
int hibf_gpu_hibf_load(char const * path, hibf_gpu_hibf ** out);
int hibf_gpu_hibf_download_words(hibf_gpu_hibf * h, uint64_t ibf, uint64_t * words, uint64_t n_words);
/* Checksum of every IBF's bit store in the reference's word order (the words of ibf_vector[k]'s bit_vector,
 * interleaved_bloom_filter.hpp:146): out[k] = fold of hg_digest_step over the words from HG_DIGEST_INIT
 * (include/hibf_gb300_synthetic.h), for comparing a device index with a reference build without moving it.  IBFs are
 * folded on `threads` host threads (0: all). */
int hibf_gpu_hibf_digests(hibf_gpu_hibf * h, uint64_t * out, uint32_t threads);

/* ------------------------------------------------------------------------------------------------------------ */
/* Build from a layout (hierarchical_interleaved_bloom_filter(config&, layout::layout const&),                   */
/* hierarchical_interleaved_bloom_filter.hpp:205; src/hierarchical_interleaved_bloom_filter.cpp:40-253).         */
/* The host parses the layout file text (src/layout/layout.cpp:60-145), builds the IBF graph                      */
/* (src/layout/graph.cpp:19-125), sizes every IBF like construct_ibf (src/build/construct_ibf.cpp:26-64) and      */
/* fills the tables; every insert runs on the device.  IBFs are numbered depth-first in layout order.              */
/* ------------------------------------------------------------------------------------------------------------ */
typedef struct hibf_gpu_build_config
{
    uint64_t number_of_user_bins;      /* config::number_of_user_bins      */
    uint64_t number_of_hash_functions; /* config::number_of_hash_functions */
    double maximum_fpr;                /* config::maximum_fpr              */
    double relaxed_fpr;                /* config::relaxed_fpr              */
    uint64_t threads;                  /* config::threads (host work)      */
    int user_bins_disjoint;            /* user bins share no value: unions are sized by sums, no host set union */
} hibf_gpu_build_config;

/* config::input_fn (config.hpp:111): for user bin `user_bin` the callback pushes its values into the sink,
 * the insert_iterator of the reference (include/hibf/misc/insert_iterator.hpp:24-111). */
typedef struct hibf_gpu_sink hibf_gpu_sink;
typedef void (*hibf_gpu_input_fn)(void * user, uint64_t user_bin, hibf_gpu_sink * sink);
int hibf_gpu_sink_push(hibf_gpu_sink * sink, uint64_t const * values, uint64_t n);

int hibf_gpu_hibf_build(hibf_gpu_build_config const * cfg, char const * layout_text, hibf_gpu_input_fn input_fn,
                        void * user, hibf_gpu_hibf ** out);
/* Split tables.  The reference splits a user bin over k technical bins in chunks of ceil(n / k) values taken in its
 * hash set's iteration order (src/build/insert_into_ibf.cpp:28-47; robin_hood::unordered_flat_set, whose order
 * depends on the set's whole history in hierarchical_build, src/hierarchical_interleaved_bloom_filter.cpp:39-171).
 * That order visits values in non-decreasing home slot of the set's table, so a split table keeps, per split user
 * bin, only the set's hash multiplier and slot mask and, per chunk boundary, the home slot of the value at the
 * boundary and the values of that slot ranked before it; the device places every value from it.  A table is
 * computed by replaying the reference's set history on the host (config::threads threads; every split user bin's
 * values and every set that can affect one are inserted, nothing else), or imported from arrays exported earlier:
 *   user_bin[n_split] ascending, n_values[n_split], mult[n_split], mask[n_split], bnd_off[n_split + 1] (boundaries
 *   of entry i: [bnd_off[i], bnd_off[i+1])), bnd_home[n_boundaries], before_off[n_boundaries + 1], before[n_before].
 * A table belongs to one layout and one set of user bin sizes; builds check both. */
typedef struct hibf_gpu_split_table hibf_gpu_split_table;
int hibf_gpu_split_table_synthetic(hibf_gpu_build_config const * cfg, char const * layout_text, uint64_t seed,
                                   uint64_t const * user_bin_offsets, hibf_gpu_split_table ** out);
/* The table of an input_fn build (hibf_gpu_hibf_build's inputs: user bins read once, split user bins in input order). */
int hibf_gpu_split_table_inputs(hibf_gpu_build_config const * cfg, char const * layout_text, hibf_gpu_input_fn input_fn,
                                void * user, hibf_gpu_split_table ** out);
int hibf_gpu_split_table_sizes(hibf_gpu_split_table const * t, uint64_t * n_split, uint64_t * n_boundaries,
                               uint64_t * n_before);
int hibf_gpu_split_table_export(hibf_gpu_split_table const * t, uint64_t * user_bin, uint64_t * n_values,
                                uint64_t * mult, uint64_t * mask, uint64_t * bnd_off, uint64_t * bnd_home,
                                uint64_t * before_off, uint64_t * before);
int hibf_gpu_split_table_import(uint64_t n_split, uint64_t n_boundaries, uint64_t n_before, uint64_t const * user_bin,
                                uint64_t const * n_values, uint64_t const * mult, uint64_t const * mask,
                                uint64_t const * bnd_off, uint64_t const * bnd_home, uint64_t const * before_off,
                                uint64_t const * before, hibf_gpu_split_table ** out);
/* Host lookup: chunks[j] = the technical bin offset (from the user bin's storage bin) of values[j] of a split user bin. */
int hibf_gpu_split_table_chunks(hibf_gpu_split_table const * t, uint64_t user_bin, uint64_t const * values, uint64_t n,
                                uint64_t * chunks);
void hibf_gpu_split_table_destroy(hibf_gpu_split_table * t);
/* The same build for the seeded synthetic workloads of include/hibf_gb300_synthetic.h: user bin u holds stream
 * positions [user_bin_offsets[u], user_bin_offsets[u+1]) of the splitmix64 stream `seed`, generated on the device.
 * Split user bins are chunked by `table` (NULL: computed first, as hibf_gpu_split_table_synthetic does), so every
 * IBF's bit store is the reference's. */
int hibf_gpu_hibf_build_synthetic(hibf_gpu_build_config const * cfg, char const * layout_text, uint64_t seed,
                                  uint64_t const * user_bin_offsets, hibf_gpu_split_table const * table,
                                  hibf_gpu_hibf ** out);
/* The build's phase timers (hierarchical_interleaved_bloom_filter.hpp:283-290, each a concurrent_timer,
 * include/hibf/misc/timer.hpp): the seconds of all intervals, the longest interval and the interval count of
 *   [0] index_allocation: allocating and zeroing the bit stores (src/build/construct_ibf.cpp:49-57);
 *   [1] user_bin_io: the input_fn calls, one interval per user bin (src/build/compute_kmers.cpp:27-31), and the
 *       upload of the distinct values; no interval in a synthetic build, whose fill kernel generates the values;
 *   [2] merge_kmers: the set work that stands in for the reference's parent merges (update_parent_kmers): distinct
 *       sets, union sizes and the split-order replay, one interval each;
 *   [3] fill_ibf: the device inserts into every IBF, one interval (src/build/insert_into_ibf.cpp:37-68).
 * All zero for an HIBF that was loaded or created from tables: the reference's timers hold values only after a
 * build.  The reference's layout_* timers time the layout computation, which stays with seqan::hibf. */
typedef struct hibf_gpu_timer
{
    double seconds;     /* concurrent_timer::in_seconds()     */
    double max_seconds; /* concurrent_timer::max_in_seconds() */
    uint64_t count;     /* intervals added                    */
} hibf_gpu_timer;
#define HIBF_GPU_TIMER_INDEX_ALLOCATION 0
#define HIBF_GPU_TIMER_USER_BIN_IO 1
#define HIBF_GPU_TIMER_MERGE_KMERS 2
#define HIBF_GPU_TIMER_FILL_IBF 3
#define HIBF_GPU_TIMER_COUNT 4
int hibf_gpu_hibf_build_timers(hibf_gpu_hibf const * h, hibf_gpu_timer * timers /* [HIBF_GPU_TIMER_COUNT] */);
/* interleaved_bloom_filter(config&, max_bin_elements) (interleaved_bloom_filter.hpp:241, src/interleaved_bloom_filter.cpp:
 * 55-117): bin count = number_of_user_bins; bin size from max_bin_elements, or -- when 0 -- from the exact distinct
 * count of the user bin with the largest HyperLogLog estimate (sketch_bits), the first such bin on ties; then user
 * bin u's values go to bin u.  input_fn is called once per user bin for the sketches, once for the exact count and
 * once for the inserts, as in the reference. */
int hibf_gpu_ibf_build(hibf_gpu_build_config const * cfg, uint64_t max_bin_elements, uint32_t sketch_bits,
                       int track_occupancy, hibf_gpu_input_fn input_fn, void * user, hibf_gpu_ibf ** out);
/* The host part of that constructor alone (no device): the bin size in bits and the user bin it was taken from. */
int hibf_gpu_ibf_plan(hibf_gpu_build_config const * cfg, uint64_t max_bin_elements, uint32_t sketch_bits,
                      hibf_gpu_input_fn input_fn, void * user, uint64_t * bin_size, uint64_t * biggest_user_bin);
/* HyperLogLog sketches (seqan::hibf::sketch::hyperloglog, src/sketch/hyperloglog.cpp): registers of 2^bits bytes.
 * Host: hyperloglog(bits) + add(values[i]) for i < n (hyperloglog.cpp:55-70); estimate() (hyperloglog.cpp:72-128).
 * Device: compute_sketches (src/sketch/compute_sketches.cpp:27-43) for n_user_bins user bins at once, user bin u =
 * d_values[offsets[u] .. offsets[u+1]) (host offsets), or, when d_values is NULL, those positions of the splitmix64
 * stream `seed`; d_registers receives n_user_bins * 2^bits bytes, the same registers as the host.  bits in [5, 16]
 * on the device.  Synchronous. */
int hibf_gpu_hll_sketch(uint64_t const * values, uint64_t n, uint32_t bits, uint8_t * registers);
int hibf_gpu_hll_estimate(uint8_t const * registers, uint32_t bits, double * estimate);
int hibf_gpu_hll_sketch_d(uint64_t const * d_values, uint64_t seed, uint64_t const * offsets, uint64_t n_user_bins,
                          uint32_t bits, uint8_t * d_registers, void * stream);
/* Host part of hibf_gpu_hibf_build alone (no device): every user bin's distinct values in the order the build
 * inserts them, user bin u = values[offsets[u] .. offsets[u+1]).  Split user bins come in the reference's chunk
 * order (its hash set's iteration order, src/build/insert_into_ibf.cpp:28-47, replayed through the history of
 * hierarchical_build, src/hierarchical_interleaved_bloom_filter.cpp:39-171); chunk k of ceil(n / tbs) values goes
 * to technical bin storage + k.  First call with values == NULL for the offsets (n_user_bins + 1 entries). */
int hibf_gpu_hibf_build_inputs(hibf_gpu_build_config const * cfg, char const * layout_text,
                               hibf_gpu_input_fn input_fn, void * user, uint64_t * offsets, uint64_t * values);
/* Host-only planning for pairwise disjoint user bins of the given distinct sizes: the IBF count and total bins
 * (first call with NULL arrays), then sizes, tables and each IBF's parent (IBF, bin).  No device needed. */
int hibf_gpu_plan_disjoint(hibf_gpu_build_config const * cfg, char const * layout_text,
                           uint64_t const * user_bin_sizes, uint64_t * n_ibfs, uint64_t * total_bins, uint64_t * bins,
                           uint64_t * bin_sizes, uint64_t * next_ibf_id, uint64_t * user_bin_id,
                           uint64_t * parent_ibf, uint64_t * parent_bin);

/* ------------------------------------------------------------------------------------------------------------ */
/* Agents (hierarchical_interleaved_bloom_filter.hpp:241-247).  An agent owns its device workspace, result       */
/* buffers and stream; like the reference's agents, use one per thread.  Results returned by pointer stay valid   */
/* until the agent's next call, as the reference's `const &` results do.                                          */
/* ------------------------------------------------------------------------------------------------------------ */
typedef struct hibf_gpu_agent hibf_gpu_agent;

int hibf_gpu_agent_create(hibf_gpu_hibf * h, hibf_gpu_agent ** out);
int hibf_gpu_agent_destroy(hibf_gpu_agent * a);
/* Run the agent's work on this stream (cudaStream_t as void*); NULL restores the agent's own stream. */
int hibf_gpu_agent_set_stream(hibf_gpu_agent * a, void * stream);
/* Capacities of the device workspace; calls that need more grow it (host calls) or fail with OVERFLOW (_d). */
int hibf_gpu_agent_reserve(hibf_gpu_agent * a, uint64_t max_queries, uint64_t max_values, uint64_t max_tasks,
                           uint64_t max_results);

/* membership_agent_type::membership_for + sort_results (hierarchical_interleaved_bloom_filter.hpp:322-439) for one
 * query: the plain form, one device launch per call.  *ids points at the agent's sorted result buffer. */
int hibf_gpu_agent_membership_for(hibf_gpu_agent * a, uint64_t const * values, uint64_t n, uint16_t threshold,
                                  uint64_t const ** ids, uint64_t * n_ids);
/* membership_agent_type::membership_for alone (hierarchical_interleaved_bloom_filter.hpp:322-355, 424-439): the same
 * user bins in the order the reference reports them before sort_results() -- depth-first, a merged bin's subtree in
 * place of the merged bin. */
int hibf_gpu_agent_membership_for_unsorted(hibf_gpu_agent * a, uint64_t const * values, uint64_t n,
                                           uint16_t threshold, uint64_t const ** ids, uint64_t * n_ids);
/* counting_agent_type<value_t>::bulk_count (hierarchical_interleaved_bloom_filter.hpp:463-566) for one query:
 * *counts points at the agent's dense vector of n_user_bins counters of `width` bytes.  threshold must be > 0. */
int hibf_gpu_agent_bulk_count(hibf_gpu_agent * a, uint64_t const * values, uint64_t n, uint64_t threshold,
                              int width, void const ** counts);

/* Batched queries, one persistent launch for all of them.  Queries are CSR: values[query_offsets[q] ..
 * query_offsets[q+1]).  mode HIBF_GPU_QUERY_MEMBERSHIP uses the uint16 thresholds of membership_for;
 * HIBF_GPU_QUERY_COUNT the size_t thresholds of bulk_count with counters of `width` bytes (thresholds > 0).
 * Results are CSR per query, ascending user-bin ids, and for COUNT the count of each listed user bin (the
 * dense counting vector's non-zero entries; every other entry is 0).  Host form: *result_offsets (n_queries+1),
 * *result_ids and *result_counts (width bytes each; NULL for MEMBERSHIP) point into agent-owned host memory.
 * A host batch of at least 64 MiB of values is streamed: its values are copied in chunks on a second stream while
 * the kernel answers the queries of chunks already copied (results are the same either way). */
#define HIBF_GPU_QUERY_MEMBERSHIP 1
#define HIBF_GPU_QUERY_COUNT 2
int hibf_gpu_agent_query_batch(hibf_gpu_agent * a, int mode, uint64_t const * values,
                               uint64_t const * query_offsets, uint64_t n_queries, uint64_t const * thresholds,
                               int width, uint64_t const ** result_offsets, uint64_t const ** result_ids,
                               void const ** result_counts);
/* Device form: inputs already in HBM; results stay in the agent's device buffers (returned as device pointers).
 * Asynchronous on the agent's stream; hibf_gpu_agent_status() after synchronising gives OVERFLOW / TIMEOUT. */
int hibf_gpu_agent_query_batch_d(hibf_gpu_agent * a, int mode, uint64_t const * d_values,
                                 uint64_t const * d_query_offsets, uint64_t n_queries, uint64_t const * d_thresholds,
                                 int width, uint64_t const ** d_result_offsets, uint64_t const ** d_result_ids,
                                 void const ** d_result_counts);
/* Plain form of the batch: one launch per query (the baseline the persistent launch is measured against). */
int hibf_gpu_agent_query_plain_d(hibf_gpu_agent * a, int mode, uint64_t const * d_values,
                                 uint64_t const * h_query_offsets, uint64_t n_queries, uint64_t const * h_thresholds,
                                 int width);
/* Copies the results of the agent's last batch (_d or plain) into agent-owned host memory; synchronises. */
int hibf_gpu_agent_fetch_results(hibf_gpu_agent * a, uint64_t n_queries, int mode, int width,
                                 uint64_t const ** result_offsets, uint64_t const ** result_ids,
                                 void const ** result_counts);
int hibf_gpu_agent_status(hibf_gpu_agent * a);
/* Failure-detection self-test of the work queue's bounded wait: runs the persistent kernel with one announced task
 * that is never pushed, so every worker's wait must expire after limit_ms and the batch must report
 * HIBF_GPU_ERR_TIMEOUT through the device status word.  Returns OK when it did; the context stays usable. */
int hibf_gpu_agent_selftest_wait_limit(hibf_gpu_agent * a, double limit_ms);
/* Captures one batch's launch sequence (control reset, persistent kernel, compaction) on fixed device buffers into
 * a CUDA graph owned by the agent; hibf_gpu_agent_replay launches it on the agent's stream. */
int hibf_gpu_agent_capture_batch_d(hibf_gpu_agent * a, int mode, uint64_t const * d_values,
                                   uint64_t const * d_query_offsets, uint64_t n_queries, uint64_t const * d_thresholds,
                                   int width);
int hibf_gpu_agent_replay(hibf_gpu_agent * a);
/* Device time of the persistent query kernel of the agent's last batch (CUDA events on the agent's stream). */
int hibf_gpu_agent_kernel_ms(hibf_gpu_agent * a, float * ms);
/* Under HIBF_GPU_SCHEDULE_LEVELS: device time of each level of the agent's last batch (the root first; a level's time
 * includes grouping its tasks by IBF).  *n receives the level count (0 for a batch run by the queue); at most `cap`
 * are written. */
int hibf_gpu_agent_level_ms(hibf_gpu_agent * a, float * ms, uint32_t cap, uint32_t * n);
/* Per level of the last level-scheduled batch: tasks, value visits and executed value visits (the early exit's
 * saving per level; their sums are hibf_gpu_agent_last_work / _last_work_executed).  *n receives the level count (0
 * for a batch run by the queue); at most `cap` entries of each array are written.  Synchronises the agent's stream. */
int hibf_gpu_agent_level_work(hibf_gpu_agent * a, uint64_t * tasks, uint64_t * value_visits,
                              uint64_t * value_visits_executed, uint32_t cap, uint32_t * n);
/* In place (on by default): host batches (hibf_gpu_agent_query_batch) whose values lie in mapped page-locked memory
 * (cudaHostAlloc, cudaHostRegister) are not copied: the kernel reads the values over the host link as it needs them,
 * and the batch runs its configured schedule from the first root.  in_place == 0 copies them first (a batch of 64 MiB
 * or more is then streamed in chunks and runs the work queue).  Pageable values are always copied.  Results are the
 * same either way; on the 8,192-bin batch (8.1 GB of values) in place took 50.3 ms per call, every call, where the
 * copy's rate varied with the host link (47-344 ms). */
int hibf_gpu_agent_set_host_read(hibf_gpu_agent * a, int in_place);
/* Whether the agent's last host batch was read in place (1) or copied (0). */
int hibf_gpu_agent_last_in_place(hibf_gpu_agent const * a, int * in_place);
/* Number of chunks in which the agent's last host batch streamed its values (0: copied whole before the launch). */
int hibf_gpu_agent_input_chunks(hibf_gpu_agent const * a, uint32_t * chunks);
/* Timeline of the agent's last host batch (hibf_gpu_agent_query_batch), in ms from the call's first device work:
 * the time each value chunk's copy completed (one entry when the values were copied whole), then the persistent
 * kernel's start and end, then the time the results were back in host memory.  *n receives the entry count
 * (chunks + 3); at most `cap` entries are written. */
int hibf_gpu_agent_last_timeline(hibf_gpu_agent const * a, double * out_ms, uint32_t cap, uint32_t * n);
/* (diagnostic, no device needed) The chunk boundaries a host batch with these query offsets would stream in: the
 * first query of every chunk, then n_queries; every boundary but 0 and n_queries starts a 32-byte sector
 * (query_offsets[q] % 4 == 0).  *n receives the count (2 or fewer: not streamed); at most cap entries are written. */
int hibf_gpu_stream_plan(uint64_t const * query_offsets, uint64_t n_queries, uint64_t * first_queries, uint64_t cap,
                         uint64_t * n);
/* Number of (query, IBF) tasks the last batch processed and the number of query values they covered
 * (sum over tasks of the query length): the work the roofline is computed from. */
int hibf_gpu_agent_last_work(hibf_gpu_agent * a, uint64_t * tasks, uint64_t * value_visits);
/* The query values the last batch actually read: a (query, IBF) task stops reading once no bin segment of the IBF
 * can reach the threshold any more (its result is then already fixed), so this is at most value_visits. */
int hibf_gpu_agent_last_work_executed(hibf_gpu_agent * a, uint64_t * value_visits_executed);

/* ============================================================================================================ */
/* Schedule of the persistent query kernel and its autotuner (no counterpart in the reference).  Every schedule     */
/* computes the same exact counts, so results do not depend on it; only the time does.                              */
/* ============================================================================================================ */
#define HIBF_GPU_EARLY_EXIT_ADAPTIVE 0xFFFFFFFFu
typedef struct hibf_gpu_tuning
{
    uint32_t values_per_lane;   /* 1 or 2: values each lane hashes per pass, times max(1, 4 / lanes per row) */
    uint32_t fetch_bytes;       /* 8 or 16: bytes each lane loads of a row (16: one 128-bit load; rows of >= 2 words) */
    uint32_t counter_bits;      /* 5 or 7: width of the per-lane bit-sliced counters between shared-memory flushes */
    uint32_t blocks_per_sm;     /* persistent blocks of 256 threads per SM; 0 = as many as fit */
    uint32_t early_exit_first;  /* percent of a task's values counted before its first early-exit check */
    uint32_t early_exit_step;   /* percent between later checks (adaptive: the fewest values between checks) */
    uint32_t early_exit_stages; /* number of checks (0: none; first + (stages - 1) * step must stay below 100), or
                                   HIBF_GPU_EARLY_EXIT_ADAPTIVE: check where the outcome can first change, computed
                                   from the bin sums at every check (early_exit_first unused) */
    uint32_t early_exit_min;    /* tasks with fewer values are counted in one stage */
    uint32_t block_queries;     /* batches of at most this many queries run one task per block of 8 warps (latency
                                   mode: each task's values split over the warps, no early exit); 0: never */
    uint32_t schedule;          /* HIBF_GPU_SCHEDULE_QUEUE: one persistent launch, child tasks run as they appear;
                                   HIBF_GPU_SCHEDULE_LEVELS: one launch per level of the hierarchy, each level's tasks
                                   grouped by IBF first, so the warps running at any moment read a few IBFs, which
                                   L2 holds (the root level as in the queue).  A streamed host batch always runs
                                   the queue: its roots arrive over the copy and children run in between */
    uint32_t level_values_per_lane; /* HIBF_GPU_SCHEDULE_LEVELS: values_per_lane of the levels below the root, whose
                                       IBFs L2 mostly holds (more loads in flight per lane); 0: values_per_lane */
} hibf_gpu_tuning;
#define HIBF_GPU_SCHEDULE_QUEUE 0u
#define HIBF_GPU_SCHEDULE_LEVELS 1u
/* (values_per_lane, fetch_bytes, counter_bits) in {(1,8,7) (2,8,7) (1,8,5) (2,8,5) (1,16,7) (1,16,5)}; hierarchies
 * with more than 3 hash functions or rows of more than 4 words (over 256 technical bins) take (1,8,7) only. */
void hibf_gpu_tuning_default(hibf_gpu_tuning * t);
/* Sets the agent's schedule for later batches (a captured graph is dropped: capture again). */
int hibf_gpu_agent_set_tuning(hibf_gpu_agent * a, hibf_gpu_tuning const * t);
int hibf_gpu_agent_get_tuning(hibf_gpu_agent * a, hibf_gpu_tuning * t);
typedef struct hibf_gpu_tune_trial
{
    hibf_gpu_tuning tuning;
    double kernel_ms; /* median device time of the persistent kernel over the repetitions */
} hibf_gpu_tune_trial;
/* Measures `tuning` (writes *kernel_ms); returns a status. */
typedef int (*hibf_gpu_tune_measure_fn)(hibf_gpu_tuning const * tuning, void * user, double * kernel_ms);
/* The autotuner's search, independent of the device: every kernel variant the hierarchy admits (given its hash
 * function count and its widest row in 64-bit words; the 16-byte fetch only for rows of >= 2 words) at 1 and at the
 * maximum blocks per SM, then the early-exit schedule and its minimum task length by coordinate descent.  Writes up
 * to cap trials in measurement order, *n_trials (all of them) and *best (the fastest). */
int hibf_gpu_tune_search(uint32_t hash_count, uint32_t max_row_words, hibf_gpu_tune_measure_fn measure, void * user,
                         hibf_gpu_tune_trial * trials, uint64_t cap, uint64_t * n_trials, hibf_gpu_tuning * best);
/* Autotunes the agent on a sample batch in HBM (as hibf_gpu_agent_query_batch_d): each trial is one warm-up and
 * `reps` timed launches; every trial's results must equal the first's (else HIBF_GPU_ERR_LOGIC).  Leaves the best
 * schedule set on the agent. */
int hibf_gpu_agent_autotune(hibf_gpu_agent * a, int mode, uint64_t const * d_values, uint64_t const * d_query_offsets,
                            uint64_t n_queries, uint64_t const * d_thresholds, int width, int reps,
                            hibf_gpu_tune_trial * trials, uint64_t cap, uint64_t * n_trials);

/* ============================================================================================================ */
/* Learned scheduler (no counterpart in the reference): a small MLP predicts each query's work from cheap features  */
/* and the persistent kernel claims root tasks largest-first.  Only the order of tasks changes; results are exact.  */
/* ============================================================================================================ */
#define HIBF_GPU_COST_FEATURES 6
#define HIBF_GPU_COST_PARAMS 1313
/* Claim order of the root tasks for the agent's later batches: a device permutation of 0..n_queries-1 (NULL or
 * n_queries == 0: query order).  Later batches must have exactly n_queries queries (else INVALID_ARG); an entry that
 * is not a query index is skipped and reported as INVALID_ARG by the batch status.  The pointer is used as given by
 * every later batch (a captured graph is dropped: capture again).  Ignored by the plain form. */
int hibf_gpu_agent_set_order_d(hibf_gpu_agent * a, uint32_t const * d_order, uint64_t n_queries);
/* Records each query's executed value visits (summed over its tasks) into d_work[0..n) during later batches of at
 * most n_queries queries (zeroed at each batch start; NULL: off).  The training target of the cost model. */
int hibf_gpu_agent_set_work_out_d(hibf_gpu_agent * a, uint64_t * d_work, uint64_t n_queries);
/* Features of each query, HIBF_GPU_COST_FEATURES floats per query: log2(1+n)/16, min(t/n, 2), and from the root
 * IBF's counts over the first `probe` values: the best segment's count / probe values, the number of segments and
 * of merged bins that reach t/n of the probe (/ 8, at most 1), probe values / probe.  Asynchronous on the agent's
 * stream. */
int hibf_gpu_agent_query_features_d(hibf_gpu_agent * a, uint64_t const * d_values, uint64_t const * d_query_offsets,
                                    uint64_t n_queries, uint64_t const * d_thresholds, uint32_t probe,
                                    float * d_features);
typedef struct hibf_gpu_cost_model hibf_gpu_cost_model;
/* 6 -> 32 -> 32 -> 1 ReLU network, He-uniform initial weights from a seeded splitmix64 stream. */
int hibf_gpu_cost_model_create(uint64_t seed, hibf_gpu_cost_model ** out);
int hibf_gpu_cost_model_destroy(hibf_gpu_cost_model * m);
/* HIBF_GPU_COST_PARAMS floats: W1[32][6], b1[32], W2[32][32], b2[32], w3[32], b3 (set resets the optimiser). */
int hibf_gpu_cost_model_get_params(hibf_gpu_cost_model * m, float * out);
int hibf_gpu_cost_model_set_params(hibf_gpu_cost_model * m, float const * in);
/* Mean squared error of the prediction against log(1 + d_work[i]) over n samples and its gradient (host array of
 * HIBF_GPU_COST_PARAMS floats, may be NULL), computed by the device's backward kernel.  Synchronous. */
int hibf_gpu_cost_model_loss_grad_d(hibf_gpu_cost_model * m, float const * d_features, uint64_t const * d_work,
                                    uint64_t n, float * grads, double * loss);
/* `steps` full-batch Adam steps (learning rate lr) on the device; *loss = the final mean squared error. */
int hibf_gpu_cost_model_train_d(hibf_gpu_cost_model * m, float const * d_features, uint64_t const * d_work,
                                uint64_t n, uint32_t steps, float lr, double * loss);
/* Predicted log(1 + work) per query. */
int hibf_gpu_cost_model_predict_d(hibf_gpu_cost_model * m, float const * d_features, uint64_t n, float * d_pred,
                                  void * stream);
/* Claim order by predicted work, largest first (ties in query order): predict, then a stable descending sort. */
int hibf_gpu_cost_model_order_d(hibf_gpu_cost_model * m, float const * d_features, uint64_t n, uint32_t * d_order,
                                void * stream);
/* The same stable descending sort for caller-supplied keys (e.g. a heuristic's), using the model's scratch. */
int hibf_gpu_sort_desc_d(hibf_gpu_cost_model * m, float const * d_keys, uint64_t n, uint32_t * d_order,
                         void * stream);

/* ============================================================================================================ */
/* Continuous-batching server over a resident HIBF (no counterpart in the reference, whose agents answer one query   */
/* per call).  A loop thread owns n_slots agents with their own streams; waiting requests are coalesced oldest-first */
/* into one batch per free slot, bounded by the slot capacity (queries, values) and by admission_bytes, the device   */
/* memory of inputs, task queues, records and result lists of all batches in flight.  Batches on different slots    */
/* overlap on the device.  A request that cannot run even alone in a slot is rejected with HIBF_GPU_ERR_ADMISSION.   */
/* Results are membership_for + sort_results per query, identical to the request answered alone.                    */
/* ============================================================================================================ */
typedef struct hibf_gpu_server hibf_gpu_server;
int hibf_gpu_server_create(hibf_gpu_hibf * h, int n_slots, uint64_t max_batch_queries, uint64_t max_batch_values,
                           uint64_t admission_bytes, hibf_gpu_server ** out);
int hibf_gpu_server_destroy(hibf_gpu_server * s);
/* copy != 0: inputs copied; copy == 0: the caller keeps them alive until hibf_gpu_server_release (offsets from 0);
 * borrowed values inside a range registered with hibf_gpu_server_register_host are copied to the device directly,
 * other memory is staged through the slot's pinned buffer.
 * arrival_s: arrival time on hibf_gpu_server_now's clock (< 0: now); latencies are measured from it. */
int hibf_gpu_server_submit(hibf_gpu_server * s, uint64_t const * values, uint64_t const * query_offsets,
                           uint64_t n_queries, uint64_t const * thresholds, double arrival_s, int copy, uint64_t * id);
/* Registers [ptr, ptr + bytes) as page-locked request memory: borrowed requests whose values lie inside a registered
 * range are read in place or copied to the device directly (no staging).  already_pinned == 0: the server page-locks
 * and maps the range (cudaHostRegister, mapped) and unlocks it on unregister or destroy; != 0: the caller allocated it
 * page-locked.  The device
 * reads the range once on registration (synchronous): a page-locked page's first device read is several times slower
 * than later ones, so requests from a registered range start warm. */
int hibf_gpu_server_register_host(hibf_gpu_server * s, void const * ptr, uint64_t bytes, int already_pinned);
/* Zero copy (on by default): a batch whose borrowed requests lie back to back in one registered range that the
 * device can address (mapped page-locked memory) is answered without copying its values: the kernel reads them in
 * place over the host link as it needs them.  Other batches copy their values first.  Results are the same. */
int hibf_gpu_server_set_zero_copy(hibf_gpu_server * s, int on);
int hibf_gpu_server_unregister_host(hibf_gpu_server * s, void const * ptr);
/* Waits up to timeout_ms (< 0: forever); *status is the request's status; results valid until release. */
int hibf_gpu_server_wait(hibf_gpu_server * s, uint64_t id, double timeout_ms, int * status,
                         uint64_t const ** result_offsets, uint64_t const ** result_ids, double * latency_s);
int hibf_gpu_server_release(hibf_gpu_server * s, uint64_t id);
double hibf_gpu_server_now(void);
/* out: batches launched, queries in them, requests rejected, device bytes admitted in flight. */
/* Mean seconds per batch since creation: queueing of the batch's oldest request, staging + launch, device work,
 * result fetch, per-request split. */
int hibf_gpu_server_phase_times(hibf_gpu_server * s, double out[5]);
/* Per batch, in the order batches finished (at most 2^20 are kept): 12 doubles -- the arrival of its oldest request,
 * the slot's start, the launch, device work done, results fetched, requests finished (seconds on the server's
 * clock, hibf_gpu_server_now), its queries and values, the device time (s, CUDA events) of its input copies and of
 * its query kernel, the values it staged through the slot's pinned buffer (requests outside a registered range), and
 * 1 if the kernel read its values in place (zero copy), else 0.  *n receives the batch count; at most `cap` are
 * written. */
int hibf_gpu_server_batch_log(hibf_gpu_server * s, double * out, uint64_t cap, uint64_t * n);
int hibf_gpu_server_stats(hibf_gpu_server * s, uint64_t out[4]);
/* Open-loop Poisson load from a pool of queries (host CSR): request sizes log-uniform in [1, max_request_queries],
 * per-request thresholds ceil(f * length), f uniform in [thr_lo, thr_hi].  out: achieved queries/s, p50, p99, p99.9
 * latency (seconds), requests, queries, rejected requests, mean queries per batch. */
int hibf_gpu_server_open_loop(hibf_gpu_server * s, uint64_t const * pool_values, uint64_t const * pool_offsets,
                              uint64_t pool_queries, double offered_qps, double duration_s,
                              uint64_t max_request_queries, double thr_lo, double thr_hi, uint64_t seed,
                              double out[8]);
/* The last open-loop run's load generator (seconds): the largest and the 99.9th-percentile lateness of a submission
 * behind its scheduled arrival, the number of submissions more than 1 ms late, and the p99 and p99.9 latency measured
 * from the actual submission (the open-loop figures above count from the scheduled arrival). */
int hibf_gpu_server_open_loop_detail(hibf_gpu_server * s, double out[5]);


/* ============================================================================================================ */
/* Seeded synthetic workloads (include/hibf_gb300_synthetic.h), for benchmarks and tests                        */
/* ============================================================================================================ */
/* offsets[0..n_user_bins]: prefix sums of the user bin sizes (law: HG_SIZES_LOG_UNIFORM / _LOG_NORMAL). */
int hibf_gpu_synth_user_bin_offsets(uint64_t seed, int law, double p0, double p1, uint64_t lo, uint64_t hi,
                                    uint64_t n_user_bins, uint64_t * offsets);
/* query_offsets[0..n_queries] and thresholds[0..n_queries) of queries first_query .. first_query+n_queries-1. */
int hibf_gpu_synth_query_offsets(uint64_t seed, int law, uint64_t len_lo, uint64_t len_hi, uint32_t mix_pct,
                                 uint32_t noise_pct, uint32_t thr_num, uint32_t thr_den, uint64_t n_user_bins,
                                 uint64_t first_query, uint64_t n_queries, uint64_t * query_offsets,
                                 uint64_t * thresholds);
/* Query values on the host, or on the device (one thread per query). */
int hibf_gpu_synth_queries(uint64_t seed, int law, uint64_t len_lo, uint64_t len_hi, uint32_t mix_pct,
                           uint32_t noise_pct, uint32_t thr_num, uint32_t thr_den, uint64_t n_user_bins,
                           uint64_t const * user_bin_offsets, uint64_t first_query, uint64_t n_queries,
                           uint64_t const * query_offsets, uint64_t * values);
int hibf_gpu_synth_queries_d(uint64_t seed, int law, uint64_t len_lo, uint64_t len_hi, uint32_t mix_pct,
                             uint32_t noise_pct, uint32_t thr_num, uint32_t thr_den, uint64_t n_user_bins,
                             uint64_t const * d_user_bin_offsets, uint64_t first_query, uint64_t n_queries,
                             uint64_t const * d_query_offsets, uint64_t * d_values, void * stream);
/* Single-level IBF workload (hg_ibf_bin_value / hg_ibf_query_value): emplace of bins [first_bin, first_bin +
 * n_bins), bin b receiving its values_per_bin values generated on the device (asynchronous on `stream`; the same
 * bits as hibf_gpu_ibf_emplace with those values). */
int hibf_gpu_synth_ibf_emplace(hibf_gpu_ibf * ibf, uint64_t seed, uint64_t values_per_bin, uint64_t first_bin,
                               uint64_t n_bins, void * stream);
/* Query values first .. first+n-1 of that workload over n_bins bins, on the host or on the device. */
int hibf_gpu_synth_ibf_queries(uint64_t seed, uint64_t n_bins, uint64_t values_per_bin, uint64_t first, uint64_t n,
                               uint64_t * values);
int hibf_gpu_synth_ibf_queries_d(uint64_t seed, uint64_t n_bins, uint64_t values_per_bin, uint64_t first, uint64_t n,
                                 uint64_t * d_values, void * stream);

#ifdef __cplusplus
}
#endif

#endif /* HIBF_GB300_H */
