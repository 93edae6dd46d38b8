/* hibf_gb300_synthetic.h -- seeded synthetic workloads shared by the library, the benchmark and the test oracle.
 *
 * Header-only C (C99/C++/CUDA). Every generator is a pure function of (seed, index), so the host, the GPU and the
 * oracle produce the same inputs without exchanging them.
 *
 * Generator: splitmix64 (Steele, Lea, Flood, "Fast splittable pseudorandom number generators", OOPSLA 2014;
 * constants as in Vigna's public-domain reference).  The k-th output (k >= 0) of the stream seeded with s is
 * mix(s + (k + 1) * golden_gamma), so any position is reachable in O(1).
 *
 * User bin contents: user bin i holds n_i values taken from ONE splitmix64 stream seeded with the workload seed:
 * bin i owns stream positions [offset_i, offset_i + n_i), offset_i = n_0 + ... + n_{i-1}.  mix() is a bijection of
 * uint64 and the stream states are pairwise distinct, so all values of all bins are pairwise distinct: every bin is
 * a set, and the union of any bins has exactly the summed size.
 *
 * Sizes: drawn from a second stream; log-uniform (small HIBF) or log-normal (large HIBFs, Box-Muller) and clipped.
 * Queries: each query has its own splitmix64 state derived from (query seed, query index), so queries can be
 * generated in parallel, one thread per query, in any order.
 */
#ifndef HIBF_GB300_SYNTHETIC_H
#define HIBF_GB300_SYNTHETIC_H

#include <math.h>
#include <stddef.h>
#include <stdint.h>

#if defined(__CUDACC__)
#    define HG_HD __host__ __device__ __forceinline__
#else
#    define HG_HD static inline
#endif

#define HG_GAMMA 0x9E3779B97F4A7C15ULL

HG_HD uint64_t hg_mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

/* k-th output of the splitmix64 stream whose initial state is `seed`. */
HG_HD uint64_t hg_stream_at(uint64_t seed, uint64_t k)
{
    return hg_mix64(seed + (k + 1u) * HG_GAMMA);
}

/* Sequential splitmix64 generator. */
HG_HD uint64_t hg_next(uint64_t * state)
{
    *state += HG_GAMMA;
    return hg_mix64(*state);
}

/* Independent sub-seeds of a workload seed. */
#define HG_TAG_SIZES 0x53495A4553ULL   /* "SIZES" */
#define HG_TAG_QUERIES 0x5155455259ULL /* "QUERY" */

HG_HD uint64_t hg_subseed(uint64_t seed, uint64_t tag)
{
    return hg_mix64(seed ^ hg_mix64(tag));
}

/* Uniform double in [0, 1) from the top 53 bits. */
HG_HD double hg_unit(uint64_t x)
{
    return (double)(x >> 11) * (1.0 / 9007199254740992.0);
}

/* Order-sensitive digest of a sequence of uint64 (used to compare large result sets by checksum). */
#define HG_DIGEST_INIT 0x6A09E667F3BCC908ULL
HG_HD uint64_t hg_digest_step(uint64_t h, uint64_t x)
{
    return hg_mix64(h ^ hg_mix64(x + HG_GAMMA));
}

/* Value j of user bin b, given the bin offsets (prefix sums of the sizes). */
HG_HD uint64_t hg_user_bin_value(uint64_t seed, uint64_t const * offsets, uint64_t b, uint64_t j)
{
    return hg_stream_at(seed, offsets[b] + j);
}

/* ------------------------------------------------------------------------------------------------------------ */
/* Workload kinds.                                                                                                */
/* ------------------------------------------------------------------------------------------------------------ */

enum hg_size_law
{
    HG_SIZES_LOG_UNIFORM = 0, /* n = floor(exp(U(ln lo, ln hi)))                           */
    HG_SIZES_LOG_NORMAL = 1   /* n = floor(exp(ln median + sigma * N(0,1))), clipped [lo,hi] */
};

enum hg_query_law
{
    /* Length `len_lo` (fixed); even queries sample all values from one random user bin, odd ones are uniform. */
    HG_QUERIES_HALF_ONE_BIN = 0,
    /* Length U[len_lo, len_hi]; `mix_pct`% of queries sample from 1-3 random user bins with `noise_pct`% of the
     * values replaced by uniform ones, the rest are uniform. */
    HG_QUERIES_MIXED = 1
};

/* Host only (libm).  Size of user bin i. */
static inline uint64_t hg_user_bin_size(uint64_t seed, int law, double p0, double p1, uint64_t lo, uint64_t hi,
                                        uint64_t i)
{
    uint64_t const s = hg_subseed(seed, HG_TAG_SIZES);
    double n;
    if (law == HG_SIZES_LOG_UNIFORM)
    {
        double const u = hg_unit(hg_stream_at(s, i));
        n = floor(exp(log((double)lo) + u * (log((double)hi) - log((double)lo))));
    }
    else
    {
        /* p0 = median, p1 = sigma.  Box-Muller with u1 in (0, 1]. */
        double const u1 = 1.0 - hg_unit(hg_stream_at(s, 2u * i));
        double const u2 = hg_unit(hg_stream_at(s, 2u * i + 1u));
        double const z = sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
        n = floor(exp(log(p0) + p1 * z));
    }
    if (n < (double)lo)
        n = (double)lo;
    if (n > (double)hi)
        n = (double)hi;
    return (uint64_t)n;
}

/* Query parameters. */
typedef struct hg_query_spec
{
    uint64_t seed;       /* workload seed (user bins use the same seed)           */
    int law;             /* enum hg_query_law                                      */
    uint64_t len_lo;     /* minimum (or fixed) query length                        */
    uint64_t len_hi;     /* maximum query length (MIXED)                           */
    uint32_t mix_pct;    /* percentage of queries drawn from 1-3 user bins (MIXED) */
    uint32_t noise_pct;  /* percentage of values replaced by uniform ones (MIXED)  */
    uint32_t thr_num;    /* threshold = ceil(thr_num * len / thr_den)              */
    uint32_t thr_den;
    uint64_t n_user_bins;
} hg_query_spec;

HG_HD uint64_t hg_query_state(hg_query_spec const * q, uint64_t qi)
{
    return hg_mix64(hg_subseed(q->seed, HG_TAG_QUERIES) ^ hg_mix64(qi + 1u));
}

/* Length of query qi (uses the first draw of the query's own state). */
HG_HD uint64_t hg_query_length(hg_query_spec const * q, uint64_t qi)
{
    uint64_t st = hg_query_state(q, qi);
    uint64_t const r = hg_next(&st);
    if (q->law == HG_QUERIES_HALF_ONE_BIN || q->len_hi <= q->len_lo)
        return q->len_lo;
    return q->len_lo + r % (q->len_hi - q->len_lo + 1u);
}

HG_HD uint64_t hg_query_threshold(hg_query_spec const * q, uint64_t len)
{
    return (q->thr_num * len + q->thr_den - 1u) / q->thr_den;
}

/* Writes the `len` values of query qi to out[0..len).  `offsets` are the user bin offsets (n_user_bins + 1 entries). */
HG_HD void hg_query_values(hg_query_spec const * q, uint64_t const * offsets, uint64_t qi, uint64_t * out)
{
    uint64_t st = hg_query_state(q, qi);
    uint64_t const r0 = hg_next(&st);
    uint64_t len = q->len_lo;
    if (q->law != HG_QUERIES_HALF_ONE_BIN && q->len_hi > q->len_lo)
        len = q->len_lo + r0 % (q->len_hi - q->len_lo + 1u);
    if (q->law == HG_QUERIES_HALF_ONE_BIN)
    {
        if ((qi & 1u) == 0u)
        {
            uint64_t const b = hg_next(&st) % q->n_user_bins;
            uint64_t const nb = offsets[b + 1] - offsets[b];
            for (uint64_t k = 0; k < len; ++k)
                out[k] = hg_user_bin_value(q->seed, offsets, b, hg_next(&st) % nb);
        }
        else
        {
            for (uint64_t k = 0; k < len; ++k)
                out[k] = hg_next(&st);
        }
        return;
    }
    /* MIXED */
    if (hg_next(&st) % 100u < q->mix_pct)
    {
        uint64_t const m = 1u + hg_next(&st) % 3u;
        uint64_t bins[3];
        for (uint64_t i = 0; i < m; ++i)
            bins[i] = hg_next(&st) % q->n_user_bins;
        for (uint64_t k = 0; k < len; ++k)
        {
            if (hg_next(&st) % 100u < q->noise_pct)
            {
                out[k] = hg_next(&st);
            }
            else
            {
                uint64_t const b = bins[hg_next(&st) % m];
                uint64_t const nb = offsets[b + 1] - offsets[b];
                out[k] = hg_user_bin_value(q->seed, offsets, b, hg_next(&st) % nb);
            }
        }
    }
    else
    {
        for (uint64_t k = 0; k < len; ++k)
            out[k] = hg_next(&st);
    }
}

/* ---------------------------------------------------------------------------------------------------------- */
/* Single-level IBF workload: bin b holds stream outputs [b * values_per_bin, (b + 1) * values_per_bin) of       */
/* `seed`.  Query value i: with probability 1/2 a uniformly chosen element of a uniformly chosen bin (present),  */
/* otherwise a uniform random uint64 (absent except for false positives).                                        */
/* ---------------------------------------------------------------------------------------------------------- */
#define HG_TAG_IBF_QUERIES 0x4942465155ULL /* "IBFQU" */

HG_HD uint64_t hg_ibf_bin_value(uint64_t seed, uint64_t values_per_bin, uint64_t bin, uint64_t j)
{
    return hg_stream_at(seed, bin * values_per_bin + j);
}

HG_HD uint64_t hg_ibf_query_value(uint64_t seed, uint64_t n_bins, uint64_t values_per_bin, uint64_t i)
{
    uint64_t const qs = hg_subseed(seed, HG_TAG_IBF_QUERIES);
    uint64_t const r = hg_stream_at(qs, 2u * i);
    uint64_t const r2 = hg_stream_at(qs, 2u * i + 1u);
    if (r & 1u)
        return hg_ibf_bin_value(seed, values_per_bin, (r >> 1) % n_bins, r2 % values_per_bin);
    return r2;
}

#endif /* HIBF_GB300_SYNTHETIC_H */
