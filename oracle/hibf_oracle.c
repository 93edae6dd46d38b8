/* hibf_oracle.c -- CPU restatement of seqan::hibf's IBF/HIBF emplace and query path (TEST INFRASTRUCTURE ONLY).
 *
 * The checker and CPU baseline for the GPU path; never linked by the product.  See hibf_oracle.h.
 * Citations are file:line inside the seqan/hibf tree:
 *   IBF.hpp  = include/hibf/interleaved_bloom_filter.hpp      IBF.cpp  = src/interleaved_bloom_filter.cpp
 *   HIBF.hpp = include/hibf/hierarchical_interleaved_bloom_filter.hpp
 *   CV.hpp   = include/hibf/misc/counting_vector.hpp
 */
#define _POSIX_C_SOURCE 200809L
#include "hibf_oracle.h"

#include <omp.h>
#include <stdlib.h>
#include <string.h>

#include "../include/hibf_gb300_synthetic.h"

/* The five multiplicative hashing seeds of IBF.hpp:172-176.  They define the bit positions of every filter, so a
 * bit-exact implementation must use the same values. */
static uint64_t const orc_seeds[5] = {13572355802537770549ULL,
                                      13043817825332782213ULL,
                                      10650232656628343401ULL,
                                      16499269484942379435ULL,
                                      4893150838803335377ULL};

/* IBF.hpp:185-195: multiply by the seed, fold the high bits down by hash_shift, multiply by 2^64/phi, map into
 * [0, bin_size) with a 64x64->128 multiply-high (fastrange), scale to the row's first bit. */
uint64_t orc_hash_and_fit(orc_ibf const * ibf, uint64_t h, uint64_t seed)
{
    h *= seed;
    h ^= h >> ibf->hash_shift;
    h *= 11400714819323198485ULL;
    h = (uint64_t)(((unsigned __int128)h * (unsigned __int128)ibf->bin_size) >> 64);
    return h * ibf->technical_bins;
}

/* IBF.cpp:32-53. */
int orc_ibf_init(orc_ibf * ibf, uint64_t bins, uint64_t bin_size, uint64_t hash_funs, int track_occupancy)
{
    memset(ibf, 0, sizeof(*ibf));
    if (bins == 0u || hash_funs == 0u || hash_funs > 5u || bin_size == 0u)
        return -1;
    ibf->bins = bins;
    ibf->bin_size = bin_size;
    ibf->hash_funs = hash_funs;
    ibf->track_occupancy = track_occupancy;
    ibf->hash_shift = (uint64_t)__builtin_clzll(bin_size);
    ibf->bin_words = (bins + 63u) / 64u;
    ibf->technical_bins = ibf->bin_words * 64u;
    ibf->nwords = ibf->bin_words * bin_size;
    ibf->data = (uint64_t *)calloc(ibf->nwords, sizeof(uint64_t));
    ibf->occupancy = (uint64_t *)calloc(ibf->technical_bins, sizeof(uint64_t));
    if (!ibf->data || !ibf->occupancy)
    {
        orc_ibf_free(ibf);
        return -2;
    }
    return 0;
}

void orc_ibf_free(orc_ibf * ibf)
{
    free(ibf->data);
    free(ibf->occupancy);
    ibf->data = NULL;
    ibf->occupancy = NULL;
}

orc_ibf * orc_ibf_new(uint64_t bins, uint64_t bin_size, uint64_t hash_funs, int track_occupancy)
{
    orc_ibf * ibf = (orc_ibf *)malloc(sizeof(orc_ibf));
    if (!ibf)
        return NULL;
    if (orc_ibf_init(ibf, bins, bin_size, hash_funs, track_occupancy) != 0)
    {
        free(ibf);
        return NULL;
    }
    return ibf;
}

void orc_ibf_delete(orc_ibf * ibf)
{
    if (!ibf)
        return;
    orc_ibf_free(ibf);
    free(ibf);
}

uint64_t * orc_ibf_data(orc_ibf * ibf)
{
    return ibf->data;
}

uint64_t orc_ibf_nwords(orc_ibf const * ibf)
{
    return ibf->nwords;
}

/* occupancy counters, technical_bins of them (IBF.cpp:123-139: counted in insertion order) */
uint64_t const * orc_ibf_occupancy(orc_ibf const * ibf)
{
    return ibf->occupancy;
}

/* IBF.cpp:119-140: set bit hash_and_fit(value, seed_i) + bin for every hash function; with occupancy tracking,
 * count the bin once if any of the bits was newly set. */
void orc_ibf_emplace(orc_ibf * ibf, uint64_t value, uint64_t bin)
{
    int exists = ibf->track_occupancy;
    for (uint64_t i = 0; i < ibf->hash_funs; ++i)
    {
        uint64_t const idx = orc_hash_and_fit(ibf, value, orc_seeds[i]) + bin;
        uint64_t const mask = 1ULL << (idx & 63u);
        if (ibf->track_occupancy)
            exists &= (ibf->data[idx >> 6] & mask) != 0u;
        ibf->data[idx >> 6] |= mask;
    }
    if (ibf->track_occupancy && !exists)
        ++ibf->occupancy[bin];
}

void orc_ibf_emplace_many(orc_ibf * ibf, uint64_t const * values, uint64_t const * bins, uint64_t n)
{
    for (uint64_t i = 0; i < n; ++i)
        orc_ibf_emplace(ibf, values[i], bins[i]);
}

void orc_ibf_emplace_one_bin(orc_ibf * ibf, uint64_t const * values, uint64_t n, uint64_t bin)
{
    for (uint64_t i = 0; i < n; ++i)
        orc_ibf_emplace(ibf, values[i], bin);
}

/* IBF.cpp:142-148: reset the occupancy and clear bit `bin` of every row. */
void orc_ibf_clear(orc_ibf * ibf, uint64_t bin)
{
    ibf->occupancy[bin] = 0u;
    for (uint64_t r = 0, idx = bin; r < ibf->bin_size; ++r, idx += ibf->technical_bins)
        ibf->data[idx >> 6] &= ~(1ULL << (idx & 63u));
}

/* IBF.hpp:283-297: clear the bits of every listed bin in every row (occupancy is left as is). */
void orc_ibf_clear_range(orc_ibf * ibf, uint64_t const * bins, uint64_t n)
{
    for (uint64_t r = 0, off = 0; r < ibf->bin_size; ++r, off += ibf->technical_bins)
        for (uint64_t i = 0; i < n; ++i)
        {
            uint64_t const idx = off + bins[i];
            ibf->data[idx >> 6] &= ~(1ULL << (idx & 63u));
        }
}

/* IBF.cpp:150-161. */
int orc_ibf_try_increase_bin_number_to(orc_ibf * ibf, uint64_t new_bins)
{
    uint64_t const new_bin_words = (new_bins + 63u) / 64u;
    if (new_bins < ibf->bins || new_bin_words > ibf->bin_words)
        return 0;
    ibf->bins = new_bins;
    return 1;
}

/* IBF.cpp:163-202: widen every row to the new technical bin count; old row r keeps its words at the start of new
 * row r, the new words are zero.  Returns -1 for the reference's std::invalid_argument, -2 out of memory. */
int orc_ibf_increase_bin_number_to(orc_ibf * ibf, uint64_t new_bins)
{
    if (new_bins < ibf->bins)
        return -1;
    if (orc_ibf_try_increase_bin_number_to(ibf, new_bins))
        return 0;
    uint64_t const new_bin_words = (new_bins + 63u) / 64u;
    uint64_t const new_nwords = new_bin_words * ibf->bin_size;
    uint64_t * nd = (uint64_t *)calloc(new_nwords, sizeof(uint64_t));
    uint64_t * no = (uint64_t *)calloc(new_bin_words * 64u, sizeof(uint64_t));
    if (!nd || !no)
    {
        free(nd);
        free(no);
        return -2;
    }
    for (uint64_t r = 0; r < ibf->bin_size; ++r)
        memcpy(nd + r * new_bin_words, ibf->data + r * ibf->bin_words, ibf->bin_words * sizeof(uint64_t));
    memcpy(no, ibf->occupancy, ibf->technical_bins * sizeof(uint64_t));
    free(ibf->data);
    free(ibf->occupancy);
    ibf->data = nd;
    ibf->occupancy = no;
    ibf->bins = new_bins;
    ibf->bin_words = new_bin_words;
    ibf->technical_bins = new_bin_words * 64u;
    ibf->nwords = new_nwords;
    return 0;
}

/* IBF.cpp:204-291: AND of the h rows addressed by hash_and_fit(value, seed_i) / 64. */
void orc_ibf_bulk_contains(orc_ibf const * ibf, uint64_t value, uint64_t * out)
{
    uint64_t const bw = ibf->bin_words;
    uint64_t const * row = ibf->data + orc_hash_and_fit(ibf, value, orc_seeds[0]) / 64u;
    memcpy(out, row, bw * sizeof(uint64_t));
    for (uint64_t i = 1; i < ibf->hash_funs; ++i)
    {
        row = ibf->data + orc_hash_and_fit(ibf, value, orc_seeds[i]) / 64u;
        for (uint64_t j = 0; j < bw; ++j)
            out[j] &= row[j];
    }
}

void orc_ibf_bulk_contains_many(orc_ibf const * ibf, uint64_t const * values, uint64_t n, uint64_t * out)
{
    for (uint64_t i = 0; i < n; ++i)
        orc_ibf_bulk_contains(ibf, values[i], out + i * ibf->bin_words);
}

/* counting_agent::bulk_count (IBF.hpp:652-665) + counting_vector::operator+= (CV.hpp:171-175, scalar path
 * CV.hpp:279-312): for every value add 1 to the counter of each set bit of bulk_contains.  Counters are kept in 64
 * bits here and reduced modulo 2^(8*width) by the caller, which equals counting in value_t with wraparound. */
static void orc_count_raw(orc_ibf const * ibf, uint64_t const * values, uint64_t n, uint64_t * counts,
                          uint64_t * scratch_words)
{
    memset(counts, 0, ibf->bins * sizeof(uint64_t));
    uint64_t const bw = ibf->bin_words;
    for (uint64_t i = 0; i < n; ++i)
    {
        orc_ibf_bulk_contains(ibf, values[i], scratch_words);
        for (uint64_t w = 0; w < bw; ++w)
        {
            uint64_t word = scratch_words[w];
            while (word)
            {
                uint64_t const b = w * 64u + (uint64_t)__builtin_ctzll(word);
                word &= word - 1u;
                if (b < ibf->bins)
                    ++counts[b];
            }
        }
    }
}

static uint64_t width_mask(int width)
{
    return width >= 8 ? UINT64_MAX : ((1ULL << (8 * width)) - 1u);
}

static void store_width(void * out, uint64_t i, uint64_t v, int width)
{
    switch (width)
    {
    case 1:
        ((uint8_t *)out)[i] = (uint8_t)v;
        break;
    case 2:
        ((uint16_t *)out)[i] = (uint16_t)v;
        break;
    case 4:
        ((uint32_t *)out)[i] = (uint32_t)v;
        break;
    default:
        ((uint64_t *)out)[i] = v;
    }
}

void orc_ibf_bulk_count(orc_ibf const * ibf, uint64_t const * values, uint64_t n, int width, void * out)
{
    uint64_t * counts = (uint64_t *)malloc(ibf->bins * sizeof(uint64_t));
    uint64_t * scratch = (uint64_t *)malloc(ibf->bin_words * sizeof(uint64_t));
    orc_count_raw(ibf, values, n, counts, scratch);
    for (uint64_t b = 0; b < ibf->bins; ++b)
        store_width(out, b, counts[b], width);
    free(counts);
    free(scratch);
}

/* The same count over `threads` disjoint slices of the values with one counting vector each, summed at the end:
 * addition modulo 2^(8*width) is associative, so this equals one counting_agent over all values. */
void orc_ibf_bulk_count_mt(orc_ibf const * ibf, uint64_t const * values, uint64_t n, int width, void * out,
                           int threads)
{
    if (threads < 1)
        threads = 1;
    uint64_t * total = (uint64_t *)calloc(ibf->bins, sizeof(uint64_t));
#pragma omp parallel num_threads(threads)
    {
        uint64_t * counts = (uint64_t *)malloc(ibf->bins * sizeof(uint64_t));
        uint64_t * scratch = (uint64_t *)malloc(ibf->bin_words * sizeof(uint64_t));
        int const t = omp_get_thread_num();
        int const nt = omp_get_num_threads();
        uint64_t const lo = n * (uint64_t)t / (uint64_t)nt;
        uint64_t const hi = n * (uint64_t)(t + 1) / (uint64_t)nt;
        orc_count_raw(ibf, values + lo, hi - lo, counts, scratch);
#pragma omp critical
        for (uint64_t b = 0; b < ibf->bins; ++b)
            total[b] += counts[b];
        free(counts);
        free(scratch);
    }
    for (uint64_t b = 0; b < ibf->bins; ++b)
        store_width(out, b, total[b], width);
    free(total);
}

void orc_ibf_bulk_contains_many_mt(orc_ibf const * ibf, uint64_t const * values, uint64_t n, uint64_t * out,
                                   int threads)
{
#pragma omp parallel for num_threads(threads < 1 ? 1 : threads) schedule(static)
    for (uint64_t i = 0; i < n; ++i)
        orc_ibf_bulk_contains(ibf, values[i], out + i * ibf->bin_words);
}

/* IBF.hpp:744-764: uint16 bulk_count, then the ascending bin ids whose count reaches the threshold. */
uint64_t orc_ibf_membership(orc_ibf const * ibf, uint64_t const * values, uint64_t n, uint16_t threshold,
                            uint64_t * out)
{
    uint64_t * counts = (uint64_t *)malloc(ibf->bins * sizeof(uint64_t));
    uint64_t * scratch = (uint64_t *)malloc(ibf->bin_words * sizeof(uint64_t));
    orc_count_raw(ibf, values, n, counts, scratch);
    uint64_t m = 0;
    for (uint64_t b = 0; b < ibf->bins; ++b)
        if ((uint16_t)counts[b] >= threshold)
            out[m++] = b;
    free(counts);
    free(scratch);
    return m;
}

/* ---------------------------------------------------------------------------------------------------------- */
/* HIBF                                                                                                         */
/* ---------------------------------------------------------------------------------------------------------- */

orc_hibf * orc_hibf_new(uint64_t n_ibfs, uint64_t n_user_bins, uint64_t const * bins, uint64_t const * bin_sizes,
                        uint64_t const * hash_funs, uint64_t const * next_ibf, uint64_t const * user_bin)
{
    orc_hibf * h = (orc_hibf *)calloc(1, sizeof(orc_hibf));
    if (!h)
        return NULL;
    h->n_ibfs = n_ibfs;
    h->n_user_bins = n_user_bins;
    h->ibfs = (orc_ibf *)calloc(n_ibfs, sizeof(orc_ibf));
    h->tb_offsets = (uint64_t *)calloc(n_ibfs + 1u, sizeof(uint64_t));
    if (!h->ibfs || !h->tb_offsets)
    {
        orc_hibf_delete(h);
        return NULL;
    }
    for (uint64_t k = 0; k < n_ibfs; ++k)
    {
        if (orc_ibf_init(&h->ibfs[k], bins[k], bin_sizes[k], hash_funs[k], 0) != 0)
        {
            orc_hibf_delete(h);
            return NULL;
        }
        h->tb_offsets[k + 1] = h->tb_offsets[k] + bins[k];
    }
    uint64_t const total = h->tb_offsets[n_ibfs];
    h->next_ibf = (uint64_t *)malloc(total * sizeof(uint64_t) + 8u);
    h->user_bin = (uint64_t *)malloc(total * sizeof(uint64_t) + 8u);
    if (!h->next_ibf || !h->user_bin)
    {
        orc_hibf_delete(h);
        return NULL;
    }
    memcpy(h->next_ibf, next_ibf, total * sizeof(uint64_t));
    memcpy(h->user_bin, user_bin, total * sizeof(uint64_t));
    return h;
}

void orc_hibf_delete(orc_hibf * h)
{
    if (!h)
        return;
    if (h->ibfs)
        for (uint64_t k = 0; k < h->n_ibfs; ++k)
            orc_ibf_free(&h->ibfs[k]);
    free(h->ibfs);
    free(h->tb_offsets);
    free(h->next_ibf);
    free(h->user_bin);
    free(h);
}

orc_ibf * orc_hibf_ibf(orc_hibf * h, uint64_t k)
{
    return &h->ibfs[k];
}

/* Per-thread traversal state: one counter array per recursion depth (the scan of a parent resumes after a child
 * has been visited, HIBF.hpp:341-344), a word buffer for bulk_contains, and the result sink. */
typedef struct orc_walk
{
    uint64_t ** counts; /* [depth][max_bins] */
    uint64_t * words;
    uint64_t max_depth;
    uint64_t visits;
    uint64_t * out_ids; /* membership: ids in DFS order; counting: unused */
    uint64_t n_out;
    uint64_t cap_out;
    uint64_t * count_out; /* counting: dense [n_user_bins], modulo 2^(8*width) */
    uint64_t threshold;
    int width;       /* counting width; membership uses 2 */
    int membership;  /* 1: membership_for; 0: bulk_count */
    int overflow;
} orc_walk;

static int orc_walk_init(orc_walk * w, orc_hibf const * h)
{
    memset(w, 0, sizeof(*w));
    uint64_t max_bins = 1, max_words = 1;
    for (uint64_t k = 0; k < h->n_ibfs; ++k)
    {
        if (h->ibfs[k].bins > max_bins)
            max_bins = h->ibfs[k].bins;
        if (h->ibfs[k].bin_words > max_words)
            max_words = h->ibfs[k].bin_words;
    }
    /* A valid hierarchy is a tree, so no path is longer than the number of IBFs; the depth cap also stops the
     * self-recursion of unassigned merged bins (HIBF.cpp:51-55), which the reference would not survive. */
    w->max_depth = h->n_ibfs < 64u ? h->n_ibfs : 64u;
    w->counts = (uint64_t **)calloc(w->max_depth, sizeof(uint64_t *));
    w->words = (uint64_t *)malloc(max_words * sizeof(uint64_t));
    if (!w->counts || !w->words)
        return -1;
    for (uint64_t d = 0; d < w->max_depth; ++d)
    {
        w->counts[d] = (uint64_t *)malloc(max_bins * sizeof(uint64_t));
        if (!w->counts[d])
            return -1;
    }
    return 0;
}

static void orc_walk_free(orc_walk * w)
{
    if (w->counts)
        for (uint64_t d = 0; d < w->max_depth; ++d)
            free(w->counts[d]);
    free(w->counts);
    free(w->words);
}

/* membership_for_impl (HIBF.hpp:322-355) and bulk_count_impl (HIBF.hpp:463-496): count the values in IBF k, then
 * scan its bins in order with a running sum in the counter type:
 *   deleted bin        -> skip, the sum is kept;
 *   merged bin         -> descend into next_ibf_id if sum >= threshold, then reset the sum;
 *   end of a user bin  -> (last bin, or the next bin belongs to another user bin) report it if sum >= threshold,
 *                         then reset the sum.  A split user bin spans consecutive bins and is reported once. */
static void orc_walk_ibf(orc_hibf const * h, orc_walk * w, uint64_t const * values, uint64_t n, uint64_t k,
                         uint64_t depth)
{
    if (depth >= w->max_depth)
    {
        w->overflow = 1;
        return;
    }
    orc_ibf const * ibf = &h->ibfs[k];
    uint64_t * counts = w->counts[depth];
    orc_count_raw(ibf, values, n, counts, w->words);
    ++w->visits;
    uint64_t const * ub = h->user_bin + h->tb_offsets[k];
    uint64_t const * next = h->next_ibf + h->tb_offsets[k];
    uint64_t const mask = width_mask(w->membership ? 2 : w->width);
    uint64_t sum = 0;
    for (uint64_t bin = 0; bin < ibf->bins; ++bin)
    {
        sum = (sum + counts[bin]) & mask;
        uint64_t const id = ub[bin];
        if (id == ORC_DELETED)
            continue;
        if (id == ORC_MERGED)
        {
            if (sum >= w->threshold)
                orc_walk_ibf(h, w, values, n, next[bin], depth + 1u);
            sum = 0;
            continue;
        }
        if (bin + 1u == ibf->bins || id != ub[bin + 1u])
        {
            if (sum >= w->threshold)
            {
                if (w->membership)
                {
                    if (w->n_out < w->cap_out)
                        w->out_ids[w->n_out] = id;
                    ++w->n_out;
                }
                else
                {
                    w->count_out[id] = sum;
                }
            }
            sum = 0;
        }
    }
}

static int cmp_u64(void const * a, void const * b)
{
    uint64_t const x = *(uint64_t const *)a, y = *(uint64_t const *)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

/* hierarchical_interleaved_bloom_filter::membership_agent_type::membership_for (HIBF.hpp:424-439); sort_results
 * (HIBF.hpp:380-383) when `sort`.  `out` needs room for n_user_bins ids. */
uint64_t orc_hibf_membership(orc_hibf const * h, uint64_t const * values, uint64_t n, uint16_t threshold, int sort,
                             uint64_t * out)
{
    orc_walk w;
    if (orc_walk_init(&w, h) != 0)
    {
        orc_walk_free(&w);
        return 0;
    }
    w.membership = 1;
    w.threshold = threshold;
    w.out_ids = out;
    w.cap_out = h->n_user_bins;
    orc_walk_ibf(h, &w, values, n, 0u, 0u);
    if (sort)
        qsort(out, w.n_out < w.cap_out ? w.n_out : w.cap_out, sizeof(uint64_t), cmp_u64);
    orc_walk_free(&w);
    return w.n_out;
}

/* counting_agent_type<value_t>::bulk_count (HIBF.hpp:549-566). */
void orc_hibf_count(orc_hibf const * h, uint64_t const * values, uint64_t n, uint64_t threshold, int width,
                    void * out)
{
    orc_walk w;
    uint64_t * dense = (uint64_t *)calloc(h->n_user_bins, sizeof(uint64_t));
    if (!dense || orc_walk_init(&w, h) != 0)
    {
        free(dense);
        return;
    }
    w.membership = 0;
    w.width = width;
    w.threshold = threshold;
    w.count_out = dense;
    orc_walk_ibf(h, &w, values, n, 0u, 0u);
    for (uint64_t i = 0; i < h->n_user_bins; ++i)
        store_width(out, i, dense[i], width);
    free(dense);
    orc_walk_free(&w);
}

void orc_hibf_query_batch(orc_hibf const * h, uint64_t const * values, uint64_t const * qoffsets, uint64_t nq,
                          uint16_t const * mem_thresholds, uint64_t const * cnt_thresholds, int threads,
                          uint64_t * mem_len, uint64_t * mem_digest, uint64_t * cnt_nnz, uint64_t * cnt_digest,
                          uint64_t * visits)
{
#pragma omp parallel num_threads(threads)
    {
        orc_walk w;
        int ok = orc_walk_init(&w, h) == 0;
        uint64_t * ids = (uint64_t *)malloc((h->n_user_bins + 1u) * sizeof(uint64_t));
        uint64_t * dense = (uint64_t *)calloc(h->n_user_bins + 1u, sizeof(uint64_t));
        ok = ok && ids && dense;
#pragma omp for schedule(dynamic, 16)
        for (uint64_t q = 0; q < nq; ++q)
        {
            if (!ok)
                continue;
            uint64_t const * v = values + qoffsets[q];
            uint64_t const n = qoffsets[q + 1] - qoffsets[q];
            /* membership_for + sort_results */
            w.membership = 1;
            w.threshold = mem_thresholds[q];
            w.out_ids = ids;
            w.cap_out = h->n_user_bins;
            w.n_out = 0;
            w.visits = 0;
            orc_walk_ibf(h, &w, v, n, 0u, 0u);
            if (visits)
                visits[q] = w.visits;
            qsort(ids, w.n_out, sizeof(uint64_t), cmp_u64);
            uint64_t d = HG_DIGEST_INIT;
            for (uint64_t i = 0; i < w.n_out; ++i)
                d = hg_digest_step(d, ids[i]);
            mem_len[q] = w.n_out;
            mem_digest[q] = d;
            /* counting_agent<uint16_t>::bulk_count */
            w.membership = 0;
            w.width = 2;
            w.threshold = cnt_thresholds[q];
            w.count_out = dense;
            orc_walk_ibf(h, &w, v, n, 0u, 0u);
            uint64_t nnz = 0, cd = HG_DIGEST_INIT;
            for (uint64_t ub = 0; ub < h->n_user_bins; ++ub)
                if (dense[ub] != 0u)
                {
                    ++nnz;
                    cd = hg_digest_step(hg_digest_step(cd, ub), dense[ub]);
                    dense[ub] = 0u;
                }
            cnt_nnz[q] = nnz;
            cnt_digest[q] = cd;
        }
        free(ids);
        free(dense);
        orc_walk_free(&w);
    }
}

void orc_hibf_membership_batch(orc_hibf const * h, uint64_t const * values, uint64_t const * qoffsets, uint64_t nq,
                               uint16_t const * thresholds, int threads, uint64_t * lengths,
                               uint64_t const * ids_offsets, uint64_t * ids)
{
#pragma omp parallel num_threads(threads)
    {
        orc_walk w;
        int ok = orc_walk_init(&w, h) == 0;
        uint64_t * buf = (uint64_t *)malloc((h->n_user_bins + 1u) * sizeof(uint64_t));
        ok = ok && buf;
#pragma omp for schedule(dynamic, 16)
        for (uint64_t q = 0; q < nq; ++q)
        {
            if (!ok)
                continue;
            w.membership = 1;
            w.threshold = thresholds[q];
            w.out_ids = buf;
            w.cap_out = h->n_user_bins;
            w.n_out = 0;
            orc_walk_ibf(h, &w, values + qoffsets[q], qoffsets[q + 1] - qoffsets[q], 0u, 0u);
            qsort(buf, w.n_out, sizeof(uint64_t), cmp_u64);
            lengths[q] = w.n_out;
            if (ids)
                memcpy(ids + ids_offsets[q], buf, w.n_out * sizeof(uint64_t));
        }
        free(buf);
        orc_walk_free(&w);
    }
}

uint64_t orc_hibf_run_queries(orc_hibf const * h, uint64_t const * values, uint64_t const * qoffsets, uint64_t nq,
                              uint16_t const * mem_thresholds, uint64_t const * cnt_thresholds, int mode,
                              int threads, uint64_t * checksum)
{
    uint64_t pairs = 0, sum = 0;
#pragma omp parallel num_threads(threads) reduction(+ : pairs, sum)
    {
        orc_walk w;
        int ok = orc_walk_init(&w, h) == 0;
        uint64_t * ids = (uint64_t *)malloc((h->n_user_bins + 1u) * sizeof(uint64_t));
        uint64_t * dense = (uint64_t *)calloc(h->n_user_bins + 1u, sizeof(uint64_t));
        ok = ok && ids && dense;
#pragma omp for schedule(dynamic, 16)
        for (uint64_t q = 0; q < nq; ++q)
        {
            if (!ok)
                continue;
            uint64_t const * v = values + qoffsets[q];
            uint64_t const n = qoffsets[q + 1] - qoffsets[q];
            if (mode & 1)
            {
                w.membership = 1;
                w.threshold = mem_thresholds[q];
                w.out_ids = ids;
                w.cap_out = h->n_user_bins;
                w.n_out = 0;
                w.visits = 0;
                orc_walk_ibf(h, &w, v, n, 0u, 0u);
                qsort(ids, w.n_out, sizeof(uint64_t), cmp_u64);
                uint64_t d = HG_DIGEST_INIT;
                for (uint64_t i = 0; i < w.n_out; ++i)
                    d = hg_digest_step(d, ids[i]);
                sum += d;
                pairs += w.visits * n;
            }
            if (mode & 2)
            {
                w.membership = 0;
                w.width = 2;
                w.threshold = cnt_thresholds[q];
                w.count_out = dense;
                w.visits = 0;
                orc_walk_ibf(h, &w, v, n, 0u, 0u);
                uint64_t cd = HG_DIGEST_INIT;
                for (uint64_t ub = 0; ub < h->n_user_bins; ++ub)
                    if (dense[ub] != 0u)
                    {
                        cd = hg_digest_step(hg_digest_step(cd, ub), dense[ub]);
                        dense[ub] = 0u;
                    }
                sum += cd;
                pairs += w.visits * n;
            }
        }
        free(ids);
        free(dense);
        orc_walk_free(&w);
    }
    if (checksum)
        *checksum = sum;
    return pairs;
}

/* ---------------------------------------------------------------------------------------------------------- */
/* Filling an HIBF with the seeded synthetic user bins (include/hibf_gb300_synthetic.h).                       */
/* ---------------------------------------------------------------------------------------------------------- */

/* Home slot of `key` in a robin_hood::unordered_flat_set<uint64_t> table with hash multiplier `mult` and slot mask
 * `mask` (include/hibf/contrib/robin_hood.hpp: hash_int then the keyToIdx multiply-shift). */
static uint64_t orc_rh_home(uint64_t key, uint64_t mult, uint64_t mask)
{
    uint64_t h = key;
    h ^= h >> 33;
    h *= 0xff51afd7ed558ccdULL;
    h ^= h >> 33;
    h *= mult;
    h ^= h >> 33;
    return (h >> 5) & mask;
}

/* The chunk of value v of a split user bin: the number of chunk boundaries of its split table entry that v lies at
 * or after.  The reference's chunks (src/build/insert_into_ibf.cpp:34-47) take its set's iteration order, which
 * visits keys in non-decreasing home slot; a boundary is the home slot of the key at its rank and the keys of that
 * slot ranked before it. */
static uint64_t orc_split_chunk(uint64_t v, uint64_t mult, uint64_t mask, uint64_t const * home, uint64_t n_bnd,
                                uint64_t const * before_off, uint64_t const * before)
{
    uint64_t const h = orc_rh_home(v, mult, mask);
    uint64_t lo = 0, hi = n_bnd;
    while (lo < hi)
    {
        uint64_t const mid = (lo + hi) / 2u;
        if (home[mid] < h)
            lo = mid + 1u;
        else
            hi = mid;
    }
    uint64_t c = lo;
    for (; c < n_bnd && home[c] == h; ++c)
    {
        int in = 0;
        for (uint64_t j = before_off[c]; j < before_off[c + 1u]; ++j)
            in |= before[j] == v;
        if (in)
            break;
    }
    return c;
}

static void orc_ibf_emplace_atomic(orc_ibf * ibf, uint64_t value, uint64_t bin)
{
    for (uint64_t i = 0; i < ibf->hash_funs; ++i)
    {
        uint64_t const idx = orc_hash_and_fit(ibf, value, orc_seeds[i]) + bin;
        __atomic_fetch_or(&ibf->data[idx >> 6], 1ULL << (idx & 63u), __ATOMIC_RELAXED);
    }
}

int orc_hibf_fill_synthetic(orc_hibf * h, uint64_t seed, uint64_t const * offsets, uint64_t n_split,
                            uint64_t const * split_user_bin, uint64_t const * split_mult,
                            uint64_t const * split_mask, uint64_t const * bnd_off, uint64_t const * bnd_home,
                            uint64_t const * before_off, uint64_t const * before, int threads)
{
    uint64_t const nub = h->n_user_bins;
    uint64_t * leaf = malloc(nub * sizeof(uint64_t));
    uint64_t * first = malloc(nub * sizeof(uint64_t));
    uint64_t * ntb = calloc(nub, sizeof(uint64_t));
    int64_t * split = malloc(nub * sizeof(int64_t));
    uint64_t * up_ibf = malloc(h->n_ibfs * sizeof(uint64_t));
    uint64_t * up_bin = malloc(h->n_ibfs * sizeof(uint64_t));
    int rc = 0;
    if (!leaf || !first || !ntb || !split || !up_ibf || !up_bin)
    {
        rc = -2;
        goto done;
    }
    for (uint64_t k = 0; k < h->n_ibfs; ++k)
        up_ibf[k] = UINT64_MAX;
    for (uint64_t u = 0; u < nub; ++u)
        split[u] = -1;
    /* placements from the tables: a user bin's technical bins, and every child IBF's parent merged bin */
    for (uint64_t k = 0; k < h->n_ibfs; ++k)
        for (uint64_t b = 0; b < h->ibfs[k].bins; ++b)
        {
            uint64_t const i = h->tb_offsets[k] + b;
            uint64_t const u = h->user_bin[i];
            if (u == ORC_MERGED)
            {
                if (h->next_ibf[i] != k && h->next_ibf[i] < h->n_ibfs)
                {
                    up_ibf[h->next_ibf[i]] = k;
                    up_bin[h->next_ibf[i]] = b;
                }
            }
            else if (u < nub)
            {
                if (ntb[u] == 0)
                {
                    leaf[u] = k;
                    first[u] = b;
                }
                ++ntb[u];
            }
        }
    for (uint64_t i = 0; i < n_split; ++i)
    {
        if (split_user_bin[i] >= nub)
        {
            rc = -1;
            goto done;
        }
        split[split_user_bin[i]] = (int64_t)i;
    }
    for (uint64_t u = 0; u < nub; ++u)
        if (ntb[u] == 0 || (ntb[u] > 1 && split[u] < 0))
        {
            rc = -1; /* a user bin without bins, or split without a table entry */
            goto done;
        }
    {
        uint64_t const total = offsets[nub];
        uint64_t const block = 1u << 16;
        uint64_t const nblocks = (total + block - 1u) / block;
#pragma omp parallel for schedule(dynamic, 4) num_threads(threads > 0 ? threads : omp_get_max_threads())
        for (uint64_t blk = 0; blk < nblocks; ++blk)
        {
            uint64_t p = blk * block;
            uint64_t const end = p + block < total ? p + block : total;
            /* the user bin holding position p: last u with offsets[u] <= p */
            uint64_t lo = 0, hi = nub;
            while (hi - lo > 1u)
            {
                uint64_t const mid = (lo + hi) / 2u;
                if (offsets[mid] <= p)
                    lo = mid;
                else
                    hi = mid;
            }
            uint64_t u = lo;
            for (; p < end; ++p)
            {
                while (offsets[u + 1u] <= p)
                    ++u;
                uint64_t const v = hg_stream_at(seed, p);
                uint64_t c = 0;
                if (split[u] >= 0)
                {
                    uint64_t const s = (uint64_t)split[u];
                    c = orc_split_chunk(v, split_mult[s], split_mask[s], bnd_home + bnd_off[s],
                                        bnd_off[s + 1u] - bnd_off[s], before_off + bnd_off[s], before);
                }
                uint64_t k = leaf[u];
                orc_ibf_emplace_atomic(&h->ibfs[k], v, first[u] + c);
                while (up_ibf[k] != UINT64_MAX)
                {
                    uint64_t const b = up_bin[k];
                    k = up_ibf[k];
                    orc_ibf_emplace_atomic(&h->ibfs[k], v, b);
                }
            }
        }
    }
done:
    free(leaf);
    free(first);
    free(ntb);
    free(split);
    free(up_ibf);
    free(up_bin);
    return rc;
}

void orc_hibf_digests(orc_hibf const * h, uint64_t * out, int threads)
{
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads > 0 ? threads : omp_get_max_threads())
    for (uint64_t k = 0; k < h->n_ibfs; ++k)
    {
        uint64_t d = HG_DIGEST_INIT;
        for (uint64_t i = 0; i < h->ibfs[k].nwords; ++i)
            d = hg_digest_step(d, h->ibfs[k].data[i]);
        out[k] = d;
    }
}

/* The seeded synthetic workloads' user bin offsets and queries (include/hibf_gb300_synthetic.h), generated on the
 * host so that the CPU arm of the benchmark needs nothing but this file. */
void orc_synth_user_bin_offsets(uint64_t seed, int law, double p0, double p1, uint64_t lo, uint64_t hi, uint64_t n,
                                uint64_t * offsets)
{
    offsets[0] = 0;
    for (uint64_t i = 0; i < n; ++i)
        offsets[i + 1] = offsets[i] + hg_user_bin_size(seed, law, p0, p1, lo, hi, i);
}

void orc_synth_queries(hg_query_spec const * q, uint64_t const * ub_offsets, uint64_t first, uint64_t n,
                       uint64_t * qoffsets, uint64_t * thresholds, uint64_t * values, int threads)
{
    if (!values)
    {
        qoffsets[0] = 0;
        for (uint64_t i = 0; i < n; ++i)
        {
            uint64_t const len = hg_query_length(q, first + i);
            qoffsets[i + 1] = qoffsets[i] + len;
            thresholds[i] = hg_query_threshold(q, len);
        }
        return;
    }
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads > 0 ? threads : omp_get_max_threads())
    for (uint64_t i = 0; i < n; ++i)
        hg_query_values(q, ub_offsets, first + i, values + qoffsets[i]);
}
