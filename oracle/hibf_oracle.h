/* hibf_oracle.h -- CPU restatement of seqan::hibf's IBF/HIBF build-and-query path, in plain C.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the GPU path is compared against (tests/), the CPU baseline that
 * bench.py times beside the GPU, and the fallback "reference" arm on hosts where the reference itself cannot be
 * compiled.  The product never links, loads or calls it.
 *
 * Parity of this restatement is pinned against the reference itself: tests/golden holds vectors produced by the
 * reference's own code (oracle/ref_driver.cpp over the reference's sources, see tests/golden/make_golden.py), and
 * tests/test_oracle_golden.py checks this file against them.
 *
 * Each function cites the reference file:line it restates (paths inside the seqan/hibf tree).
 */
#ifndef HIBF_ORACLE_H
#define HIBF_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One interleaved Bloom filter (include/hibf/interleaved_bloom_filter.hpp:146-195). */
typedef struct orc_ibf
{
    uint64_t bins;           /* user-visible bins                                  */
    uint64_t technical_bins; /* bins rounded up to a multiple of 64 (IBF.cpp:49-50) */
    uint64_t bin_size;       /* rows                                                */
    uint64_t hash_shift;     /* countl_zero(bin_size) (IBF.cpp:48)                  */
    uint64_t bin_words;      /* technical_bins / 64                                 */
    uint64_t hash_funs;      /* 1..5                                                */
    uint64_t nwords;         /* technical_bins * bin_size / 64                      */
    uint64_t * data;         /* row-major bit matrix, bin b of row r = bit r*tb + b */
    uint64_t * occupancy;    /* technical_bins counters                             */
    int track_occupancy;
} orc_ibf;

/* Hierarchy of IBFs (include/hibf/hierarchical_interleaved_bloom_filter.hpp:208-238). */
typedef struct orc_hibf
{
    uint64_t n_ibfs;
    uint64_t n_user_bins;
    orc_ibf * ibfs;
    uint64_t * tb_offsets; /* n_ibfs + 1 prefix sums of the per-IBF bin counts      */
    uint64_t * next_ibf;   /* next_ibf_id, flattened with tb_offsets                 */
    uint64_t * user_bin;   /* ibf_bin_to_user_bin_id, flattened with tb_offsets      */
} orc_hibf;

#define ORC_MERGED UINT64_MAX
#define ORC_DELETED (UINT64_MAX - 1u)

uint64_t orc_hash_and_fit(orc_ibf const * ibf, uint64_t h, uint64_t seed);

/* 0 on success; -1 for the reference's std::logic_error cases (IBF.cpp:41-46); -2 out of memory. */
int orc_ibf_init(orc_ibf * ibf, uint64_t bins, uint64_t bin_size, uint64_t hash_funs, int track_occupancy);
void orc_ibf_free(orc_ibf * ibf);
orc_ibf * orc_ibf_new(uint64_t bins, uint64_t bin_size, uint64_t hash_funs, int track_occupancy);
void orc_ibf_delete(orc_ibf * ibf);
uint64_t * orc_ibf_data(orc_ibf * ibf);
uint64_t orc_ibf_nwords(orc_ibf const * ibf);
uint64_t const * orc_ibf_occupancy(orc_ibf const * ibf);

void orc_ibf_emplace(orc_ibf * ibf, uint64_t value, uint64_t bin);
void orc_ibf_emplace_many(orc_ibf * ibf, uint64_t const * values, uint64_t const * bins, uint64_t n);
void orc_ibf_emplace_one_bin(orc_ibf * ibf, uint64_t const * values, uint64_t n, uint64_t bin);
void orc_ibf_clear(orc_ibf * ibf, uint64_t bin);
void orc_ibf_clear_range(orc_ibf * ibf, uint64_t const * bins, uint64_t n);
int orc_ibf_try_increase_bin_number_to(orc_ibf * ibf, uint64_t new_bins);
int orc_ibf_increase_bin_number_to(orc_ibf * ibf, uint64_t new_bins);

void orc_ibf_bulk_contains(orc_ibf const * ibf, uint64_t value, uint64_t * out_words);
void orc_ibf_bulk_contains_many(orc_ibf const * ibf, uint64_t const * values, uint64_t n, uint64_t * out_words);
/* width = sizeof(value_t) in bytes: 1, 2, 4 or 8.  `out` holds `bins` counters of that width. */
void orc_ibf_bulk_count(orc_ibf const * ibf, uint64_t const * values, uint64_t n, int width, void * out);
void orc_ibf_bulk_count_mt(orc_ibf const * ibf, uint64_t const * values, uint64_t n, int width, void * out,
                           int threads);
void orc_ibf_bulk_contains_many_mt(orc_ibf const * ibf, uint64_t const * values, uint64_t n, uint64_t * out,
                                   int threads);
uint64_t orc_ibf_membership(orc_ibf const * ibf, uint64_t const * values, uint64_t n, uint16_t threshold,
                            uint64_t * out);

/* HIBF from flat tables; every IBF starts zeroed. */
orc_hibf * orc_hibf_new(uint64_t n_ibfs, uint64_t n_user_bins, uint64_t const * bins, uint64_t const * bin_sizes,
                        uint64_t const * hash_funs, uint64_t const * next_ibf, uint64_t const * user_bin);
void orc_hibf_delete(orc_hibf * h);
orc_ibf * orc_hibf_ibf(orc_hibf * h, uint64_t k);

uint64_t orc_hibf_membership(orc_hibf const * h, uint64_t const * values, uint64_t n, uint16_t threshold, int sort,
                             uint64_t * out);
void orc_hibf_count(orc_hibf const * h, uint64_t const * values, uint64_t n, uint64_t threshold, int width,
                    void * out);

/* Batched: per query the sorted membership list and the uint16 count vector, reduced to
 *   mem_len[q], mem_digest[q]: length and digest of the sorted user-bin list,
 *   cnt_nnz[q], cnt_digest[q]: number and digest of the (user bin, count) pairs with count != 0, ascending.
 * `threads` OpenMP threads, dynamic schedule over queries, one private agent state per thread.
 * visits (optional) receives per query the number of IBF visits (nodes whose counts were computed). */
void orc_hibf_query_batch(orc_hibf const * h, uint64_t const * values, uint64_t const * qoffsets, uint64_t nq,
                          uint16_t const * mem_thresholds, uint64_t const * cnt_thresholds, int threads,
                          uint64_t * mem_len, uint64_t * mem_digest, uint64_t * cnt_nnz, uint64_t * cnt_digest,
                          uint64_t * visits);

/* Same traversal as orc_hibf_query_batch restricted to membership (one pass), writing the sorted lists into a
 * caller-provided CSR: first call with ids == NULL to get lengths, then with ids sized sum(lengths). */
void orc_hibf_membership_batch(orc_hibf const * h, uint64_t const * values, uint64_t const * qoffsets, uint64_t nq,
                               uint16_t const * thresholds, int threads, uint64_t * lengths,
                               uint64_t const * ids_offsets, uint64_t * ids);

/* Timed CPU baseline.  mode bit 0: membership_for + sort_results; bit 1: counting bulk_count (uint16);
 * each selected operation runs as its own traversal, as the reference's two agents do.  Returns the number of
 * (value, visited IBF) pairs processed; *checksum receives a digest of all outputs (sum over queries). */
uint64_t orc_hibf_run_queries(orc_hibf const * h, uint64_t const * values, uint64_t const * qoffsets, uint64_t nq,
                              uint16_t const * mem_thresholds, uint64_t const * cnt_thresholds, int mode,
                              int threads, uint64_t * checksum);

/* Fills the HIBF (tables already set) with the seeded synthetic user bins: user bin u = positions
 * [offsets[u], offsets[u+1]) of the splitmix64 stream `seed`, inserted into its own technical bins and the merged bin
 * of every ancestor IBF, as the reference's build inserts them (src/hierarchical_interleaved_bloom_filter.cpp:40-171,
 * src/build/insert_into_ibf.cpp:28-84).  A user bin over several technical bins is chunked by its split-table entry
 * (the layout of include/hibf_gb300.h, hibf_gpu_split_table_*).  0 on success, -1 when the tables and the split
 * table do not fit together, -2 out of memory. */
int orc_hibf_fill_synthetic(orc_hibf * h, uint64_t seed, uint64_t const * offsets, uint64_t n_split,
                            uint64_t const * split_user_bin, uint64_t const * split_mult,
                            uint64_t const * split_mask, uint64_t const * bnd_off, uint64_t const * bnd_home,
                            uint64_t const * before_off, uint64_t const * before, int threads);
/* out[k] = hg_digest_step fold over IBF k's words from HG_DIGEST_INIT. */
void orc_hibf_digests(orc_hibf const * h, uint64_t * out, int threads);

/* The synthetic workloads' generators on the host: offsets[0..n] of the user bins (hg_user_bin_size), and queries
 * first .. first+n-1 -- with values == NULL their offsets (n + 1) and thresholds, else their values
 * (hg_query_values). */
struct hg_query_spec;
void orc_synth_user_bin_offsets(uint64_t seed, int law, double p0, double p1, uint64_t lo, uint64_t hi, uint64_t n,
                                uint64_t * offsets);
void orc_synth_queries(struct hg_query_spec const * q, uint64_t const * ub_offsets, uint64_t first, uint64_t n,
                       uint64_t * qoffsets, uint64_t * thresholds, uint64_t * values, int threads);

#ifdef __cplusplus
}
#endif

#endif /* HIBF_ORACLE_H */
