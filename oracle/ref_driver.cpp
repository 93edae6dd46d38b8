// ref_driver.cpp -- a C-callable driver over the REFERENCE library (seqan::hibf compiled from its own sources).
//
// Test infrastructure only.  It is compiled by oracle/Makefile (target `ref`) together with the reference's
// src/*.cpp, read in place, against the cereal/simde stand-ins in oracle/shim, into oracle/_ref/libhibf_ref.so.
// It exists to produce golden vectors (tests/golden/make_golden.py) and to pin the C restatement in
// oracle/hibf_oracle.c; nothing in the product links or loads it.
//
// Every entry point calls the reference's public API:
//   interleaved_bloom_filter ctor/emplace/clear/agents  include/hibf/interleaved_bloom_filter.hpp:225-391
//   hierarchical_interleaved_bloom_filter ctors/agents  include/hibf/hierarchical_interleaved_bloom_filter.hpp:197-247
//   layout::compute_layout / layout::write_to           include/hibf/layout/compute_layout.hpp, layout.hpp

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <sstream>
#include <type_traits>
#include <stdexcept>
#include <string_view>
#include <memory>
#include <string>
#include <vector>

#include <hibf/config.hpp>
#include <hibf/hierarchical_interleaved_bloom_filter.hpp>
#include <hibf/interleaved_bloom_filter.hpp>
#include <hibf/layout/compute_layout.hpp>
#include <hibf/layout/layout.hpp>
#include <hibf/misc/iota_vector.hpp>
#include <hibf/misc/timer.hpp>
#include <hibf/sketch/compute_sketches.hpp>
#include <hibf/sketch/estimate_kmer_counts.hpp>
#include <hibf/sketch/hyperloglog.hpp>

#include "../include/hibf_gb300_synthetic.h"

namespace hibf = seqan::hibf;

extern "C"
{
    // Mirrors the fields of seqan::hibf::config that the drivers set (config.hpp:75-413).
    struct ref_cfg
    {
        uint64_t number_of_user_bins;
        uint64_t number_of_hash_functions;
        double maximum_fpr;
        double relaxed_fpr;
        uint64_t threads;
        uint64_t sketch_bits;
        uint64_t tmax;
        double alpha;
        double max_rearrangement_ratio;
        int disable_estimate_union;
        int disable_rearrangement;
        int track_occupancy;
        double empty_bin_fraction;
    };
}

namespace
{

// User bin contents either from CSR arrays or from the synthetic stream.
struct ub_source
{
    uint64_t const * values{nullptr};
    uint64_t const * offsets{nullptr};
    uint64_t seed{0};
    bool synthetic{false};

    void emit(size_t ub, hibf::insert_iterator & it) const
    {
        uint64_t const b = offsets[ub];
        uint64_t const e = offsets[ub + 1];
        if (synthetic)
            for (uint64_t j = b; j < e; ++j)
                it = hg_stream_at(seed, j);
        else
            for (uint64_t j = b; j < e; ++j)
                it = values[j];
    }
};

hibf::config make_config(ref_cfg const & c, ub_source src)
{
    hibf::config cfg{};
    cfg.input_fn = [src](size_t const ub, hibf::insert_iterator && it)
    {
        src.emit(ub, it);
    };
    cfg.number_of_user_bins = c.number_of_user_bins;
    cfg.number_of_hash_functions = c.number_of_hash_functions;
    cfg.maximum_fpr = c.maximum_fpr;
    cfg.relaxed_fpr = c.relaxed_fpr;
    cfg.threads = c.threads;
    cfg.sketch_bits = static_cast<uint8_t>(c.sketch_bits);
    cfg.tmax = c.tmax;
    cfg.alpha = c.alpha;
    cfg.max_rearrangement_ratio = c.max_rearrangement_ratio;
    cfg.disable_estimate_union = c.disable_estimate_union != 0;
    cfg.disable_rearrangement = c.disable_rearrangement != 0;
    cfg.track_occupancy = c.track_occupancy != 0;
    cfg.empty_bin_fraction = c.empty_bin_fraction;
    return cfg;
}

char * dup_string(std::string const & s)
{
    char * out = static_cast<char *>(std::malloc(s.size() + 1));
    std::memcpy(out, s.c_str(), s.size() + 1);
    return out;
}

template <typename value_t>
void count_into(hibf::interleaved_bloom_filter const & ibf, uint64_t const * values, uint64_t n, void * out)
{
    auto agent = ibf.template counting_agent<value_t>();
    std::vector<uint64_t> v(values, values + n);
    auto & res = agent.bulk_count(v);
    std::memcpy(out, res.data(), ibf.bin_count() * sizeof(value_t));
}

template <typename value_t>
void hibf_count_into(hibf::hierarchical_interleaved_bloom_filter const & h,
                     uint64_t const * values,
                     uint64_t n,
                     uint64_t threshold,
                     void * out)
{
    auto agent = h.template counting_agent<value_t>();
    std::vector<uint64_t> v(values, values + n);
    auto & res = agent.bulk_count(v, threshold);
    std::memcpy(out, res.data(), h.number_of_user_bins * sizeof(value_t));
}

} // namespace

// ---------------------------------------------------------------------------------------------------------------
// A byte archive with cereal's binary-archive encoding, driving the reference's own serialize/save/load functions:
// arithmetic values as their raw little-endian bytes, binary_data as raw bytes, std::vector as a uint64 element count
// followed by raw elements (arithmetic) or each element in turn, base_class as the base object, name-value pairs as
// their value.  (cereal itself is not available here; this is that encoding, not cereal's code.)
// ---------------------------------------------------------------------------------------------------------------
template <class T>
struct is_std_vector : std::false_type
{};
template <class T, class A>
struct is_std_vector<std::vector<T, A>> : std::true_type
{};
template <class T>
struct is_base_class : std::false_type
{};
template <class T>
struct is_base_class<cereal::base_class<T>> : std::true_type
{};

struct byte_out_archive : cereal::detail::OutputArchiveBase
{
    std::string bytes;
    template <class... T>
    void operator()(T &&... xs)
    {
        (put(xs), ...);
    }
    void raw(void const * p, size_t n)
    {
        bytes.append(static_cast<char const *>(p), n);
    }
    template <class T>
    void put(T const & x)
    {
        using U = std::remove_cv_t<std::remove_reference_t<T>>;
        if constexpr (std::is_arithmetic_v<U>)
            raw(&x, sizeof(U));
        else if constexpr (std::is_same_v<U, cereal::binary_data_t>)
            raw(x.ptr, x.size);
        else if constexpr (is_std_vector<U>::value)
        {
            uint64_t const n = x.size();
            raw(&n, 8);
            using E = typename U::value_type;
            if constexpr (std::is_arithmetic_v<E> && !std::is_same_v<E, bool>)
                raw(x.data(), n * sizeof(E));
            else
                for (auto const & e : x)
                    put(e);
        }
        else if constexpr (is_base_class<U>::value)
            put(*x.base_ptr);
        else if constexpr (requires(U & u, byte_out_archive & a) { u.CEREAL_SAVE_FUNCTION_NAME(a); })
            x.CEREAL_SAVE_FUNCTION_NAME(*this);
        else
            const_cast<U &>(x).CEREAL_SERIALIZE_FUNCTION_NAME(*this);
    }
};

struct byte_in_archive : cereal::detail::InputArchiveBase
{
    std::string_view bytes;
    size_t pos{};
    template <class... T>
    void operator()(T &&... xs)
    {
        (get(xs), ...);
    }
    void raw(void * p, size_t n)
    {
        if (pos + n > bytes.size())
            throw std::runtime_error("archive truncated");
        std::memcpy(p, bytes.data() + pos, n);
        pos += n;
    }
    template <class T>
    void get(T && x)
    {
        using U = std::remove_cv_t<std::remove_reference_t<T>>;
        if constexpr (std::is_arithmetic_v<U>)
            raw(&x, sizeof(U));
        else if constexpr (std::is_same_v<U, cereal::binary_data_t>)
            raw(const_cast<void *>(x.ptr), x.size);
        else if constexpr (is_std_vector<U>::value)
        {
            uint64_t n = 0;
            raw(&n, 8);
            x.resize(n);
            using E = typename U::value_type;
            if constexpr (std::is_arithmetic_v<E> && !std::is_same_v<E, bool>)
                raw(x.data(), n * sizeof(E));
            else
                for (auto & e : x)
                    get(e);
        }
        else if constexpr (is_base_class<U>::value)
            get(*x.base_ptr);
        else if constexpr (requires(U & u, byte_in_archive & a) { u.CEREAL_LOAD_FUNCTION_NAME(a); })
            x.CEREAL_LOAD_FUNCTION_NAME(*this);
        else
            x.CEREAL_SERIALIZE_FUNCTION_NAME(*this);
    }
};

template <class T>
char * save_bytes(T const & obj, uint64_t * n)
{
    byte_out_archive ar;
    ar(obj);
    *n = ar.bytes.size();
    char * out = static_cast<char *>(std::malloc(std::max<size_t>(1, ar.bytes.size())));
    std::memcpy(out, ar.bytes.data(), ar.bytes.size());
    return out;
}

extern "C"
{
    void ref_free(void * p)
    {
        std::free(p);
    }

    // ---------------------------------------------------------------------------------------------------------
    // interleaved_bloom_filter
    // ---------------------------------------------------------------------------------------------------------
    void * ref_ibf_new(uint64_t bins, uint64_t bin_size, uint64_t h, int track_occupancy)
    {
        try
        {
            return new hibf::interleaved_bloom_filter{hibf::bin_count{bins},
                                                      hibf::bin_size{bin_size},
                                                      hibf::hash_function_count{h},
                                                      track_occupancy != 0};
        }
        catch (...)
        {
            return nullptr;
        }
    }

    // interleaved_bloom_filter(config&, max_bin_elements) over CSR user bins (IBF.cpp:104-117).
    void * ref_ibf_from_config(ref_cfg const * c,
                               uint64_t const * values,
                               uint64_t const * offsets,
                               uint64_t max_bin_elements)
    {
        try
        {
            auto cfg = make_config(*c, ub_source{values, offsets, 0, false});
            return new hibf::interleaved_bloom_filter{cfg, max_bin_elements};
        }
        catch (...)
        {
            return nullptr;
        }
    }

    void ref_ibf_free(void * p)
    {
        delete static_cast<hibf::interleaved_bloom_filter *>(p);
    }

    // out: bins, bin_size, hash_function_count, bit_size
    void ref_ibf_params(void * p, uint64_t * out)
    {
        auto & ibf = *static_cast<hibf::interleaved_bloom_filter *>(p);
        out[0] = ibf.bin_count();
        out[1] = ibf.bin_size();
        out[2] = ibf.hash_function_count();
        out[3] = ibf.bit_size();
    }

    void ref_ibf_emplace(void * p, uint64_t const * values, uint64_t const * bins, uint64_t n)
    {
        auto & ibf = *static_cast<hibf::interleaved_bloom_filter *>(p);
        for (uint64_t i = 0; i < n; ++i)
            ibf.emplace(values[i], hibf::bin_index{bins[i]});
    }

    void ref_ibf_clear(void * p, uint64_t bin)
    {
        static_cast<hibf::interleaved_bloom_filter *>(p)->clear(hibf::bin_index{bin});
    }

    void ref_ibf_clear_range(void * p, uint64_t const * bins, uint64_t n)
    {
        std::vector<hibf::bin_index> r;
        for (uint64_t i = 0; i < n; ++i)
            r.push_back(hibf::bin_index{bins[i]});
        static_cast<hibf::interleaved_bloom_filter *>(p)->clear(r);
    }

    int ref_ibf_try_increase_bin_number_to(void * p, uint64_t new_bins)
    {
        return static_cast<hibf::interleaved_bloom_filter *>(p)->try_increase_bin_number_to(hibf::bin_count{new_bins})
                 ? 1
                 : 0;
    }

    int ref_ibf_increase_bin_number_to(void * p, uint64_t new_bins)
    {
        try
        {
            static_cast<hibf::interleaved_bloom_filter *>(p)->increase_bin_number_to(hibf::bin_count{new_bins});
            return 0;
        }
        catch (...)
        {
            return -1;
        }
    }

    uint64_t ref_ibf_nwords(void * p)
    {
        auto & ibf = *static_cast<hibf::interleaved_bloom_filter *>(p);
        return (ibf.bit_size() + 63u) / 64u;
    }

    void ref_ibf_words(void * p, uint64_t * out)
    {
        auto & ibf = *static_cast<hibf::interleaved_bloom_filter *>(p);
        std::memcpy(out, ibf.data(), ref_ibf_nwords(p) * sizeof(uint64_t));
    }

    uint64_t ref_ibf_occupancy(void * p, uint64_t * out)
    {
        auto & ibf = *static_cast<hibf::interleaved_bloom_filter *>(p);
        if (out)
            std::copy(ibf.occupancy.begin(), ibf.occupancy.end(), out);
        return ibf.occupancy.size();
    }

    // out: n * ceil(bins/64) words, the bit_vector words of each bulk_contains result.
    void ref_ibf_bulk_contains(void * p, uint64_t const * values, uint64_t n, uint64_t * out)
    {
        auto & ibf = *static_cast<hibf::interleaved_bloom_filter *>(p);
        auto agent = ibf.containment_agent();
        size_t const words = (ibf.bin_count() + 63u) / 64u;
        for (uint64_t i = 0; i < n; ++i)
        {
            auto & res = agent.bulk_contains(values[i]);
            std::memcpy(out + i * words, res.data(), words * sizeof(uint64_t));
        }
    }

    // width in bytes: 1, 2, 4 or 8 (counting_agent<uint8_t/uint16_t/uint32_t/uint64_t>).
    void ref_ibf_bulk_count(void * p, uint64_t const * values, uint64_t n, int width, void * out)
    {
        auto & ibf = *static_cast<hibf::interleaved_bloom_filter *>(p);
        switch (width)
        {
        case 1:
            count_into<uint8_t>(ibf, values, n, out);
            break;
        case 2:
            count_into<uint16_t>(ibf, values, n, out);
            break;
        case 4:
            count_into<uint32_t>(ibf, values, n, out);
            break;
        default:
            count_into<uint64_t>(ibf, values, n, out);
        }
    }

    uint64_t ref_ibf_membership(void * p, uint64_t const * values, uint64_t n, uint16_t threshold, uint64_t * out)
    {
        auto & ibf = *static_cast<hibf::interleaved_bloom_filter *>(p);
        auto agent = ibf.membership_agent();
        std::vector<uint64_t> v(values, values + n);
        auto & res = agent.membership_for(v, threshold);
        std::copy(res.begin(), res.end(), out);
        return res.size();
    }

    // ---------------------------------------------------------------------------------------------------------
    // layout
    // ---------------------------------------------------------------------------------------------------------
    // The same steps as hierarchical_interleaved_bloom_filter(config&) (HIBF.cpp:211-245) up to the layout, which
    // is returned in the reference's layout-file format (layout.cpp write_to).  Free with ref_free.
    // hyperloglog(bits) + add(values[i]) (src/sketch/hyperloglog.cpp:55-70): the registers, read back through
    // hyperloglog::store (one byte of bits, then 2^bits register bytes), and estimate() (hyperloglog.cpp:72-128).
    int ref_hll(uint64_t const * values, uint64_t n, uint32_t bits, uint8_t * registers, double * estimate)
    {
        try
        {
            hibf::sketch::hyperloglog h(static_cast<uint8_t>(bits));
            for (uint64_t i = 0; i < n; ++i)
                h.add(values[i]);
            std::ostringstream os;
            h.store(os);
            std::string const raw = os.str();
            uint64_t const size = uint64_t{1} << bits;
            if (raw.size() != 1 + size)
                return 1;
            std::memcpy(registers, raw.data() + 1, size);
            *estimate = h.estimate();
            return 0;
        }
        catch (...)
        {
            return 1;
        }
    }

    char * ref_layout(ref_cfg const * c, uint64_t const * values, uint64_t const * offsets, uint64_t seed, int synthetic)
    {
        try
        {
            auto cfg = make_config(*c, ub_source{values, offsets, seed, synthetic != 0});
            cfg.validate_and_set_defaults();
            std::vector<hibf::sketch::hyperloglog> sketches{};
            std::vector<size_t> kmer_counts{};
            hibf::sketch::compute_sketches(cfg, sketches);
            hibf::sketch::estimate_kmer_counts(sketches, kmer_counts);
            hibf::concurrent_timer t1, t2;
            auto layout = hibf::layout::compute_layout(cfg,
                                                       kmer_counts,
                                                       sketches,
                                                       hibf::iota_vector(cfg.number_of_user_bins),
                                                       t1,
                                                       t2);
            std::ostringstream os;
            layout.write_to(os);
            return dup_string(os.str());
        }
        catch (...)
        {
            return nullptr;
        }
    }

    // ---------------------------------------------------------------------------------------------------------
    // hierarchical_interleaved_bloom_filter
    // ---------------------------------------------------------------------------------------------------------
    // layout_text == nullptr: HIBF(config&) (layout computed by the reference); else HIBF(config&, layout).
    void * ref_hibf_new(ref_cfg const * c,
                        uint64_t const * values,
                        uint64_t const * offsets,
                        uint64_t seed,
                        int synthetic,
                        char const * layout_text)
    {
        try
        {
            auto cfg = make_config(*c, ub_source{values, offsets, seed, synthetic != 0});
            if (layout_text == nullptr)
                return new hibf::hierarchical_interleaved_bloom_filter{cfg};
            hibf::layout::layout layout{};
            std::istringstream is{std::string{layout_text}};
            layout.read_from(is);
            return new hibf::hierarchical_interleaved_bloom_filter{cfg, layout};
        }
        catch (...)
        {
            return nullptr;
        }
    }

    void ref_hibf_free(void * p)
    {
        delete static_cast<hibf::hierarchical_interleaved_bloom_filter *>(p);
    }

    uint64_t ref_hibf_num_ibfs(void * p)
    {
        return static_cast<hibf::hierarchical_interleaved_bloom_filter *>(p)->ibf_vector.size();
    }

    // out: bins, bin_size, hash_function_count, words, prev ibf idx, prev bin idx
    void ref_hibf_ibf_params(void * p, uint64_t k, uint64_t * out)
    {
        auto & h = *static_cast<hibf::hierarchical_interleaved_bloom_filter *>(p);
        auto & ibf = h.ibf_vector[k];
        out[0] = ibf.bin_count();
        out[1] = ibf.bin_size();
        out[2] = ibf.hash_function_count();
        out[3] = (ibf.bit_size() + 63u) / 64u;
        out[4] = h.prev_ibf_id[k].ibf_idx;
        out[5] = h.prev_ibf_id[k].bin_idx;
    }

    void ref_hibf_ibf_words(void * p, uint64_t k, uint64_t * out)
    {
        auto & h = *static_cast<hibf::hierarchical_interleaved_bloom_filter *>(p);
        auto & ibf = h.ibf_vector[k];
        std::memcpy(out, ibf.data(), ((ibf.bit_size() + 63u) / 64u) * sizeof(uint64_t));
    }

    // Digest of the words of IBF k (checksum over the whole bit store, order-sensitive).
    uint64_t ref_hibf_ibf_digest(void * p, uint64_t k)
    {
        auto & h = *static_cast<hibf::hierarchical_interleaved_bloom_filter *>(p);
        auto & ibf = h.ibf_vector[k];
        uint64_t d = HG_DIGEST_INIT;
        uint64_t const * w = ibf.data();
        size_t const n = (ibf.bit_size() + 63u) / 64u;
        for (size_t i = 0; i < n; ++i)
            d = hg_digest_step(d, w[i]);
        return d;
    }

    // Table sizes equal the IBF's bin count (HIBF.cpp:49-55).
    void ref_hibf_tables(void * p, uint64_t k, uint64_t * next_ibf, uint64_t * user_bin)
    {
        auto & h = *static_cast<hibf::hierarchical_interleaved_bloom_filter *>(p);
        std::copy(h.next_ibf_id[k].begin(), h.next_ibf_id[k].end(), next_ibf);
        std::copy(h.ibf_bin_to_user_bin_id[k].begin(), h.ibf_bin_to_user_bin_id[k].end(), user_bin);
    }

    uint64_t ref_hibf_membership(void * p, uint64_t const * values, uint64_t n, uint16_t threshold, int sort,
                                 uint64_t * out)
    {
        auto & h = *static_cast<hibf::hierarchical_interleaved_bloom_filter *>(p);
        auto agent = h.membership_agent();
        std::vector<uint64_t> v(values, values + n);
        auto & res = agent.membership_for(v, threshold);
        if (sort)
            agent.sort_results();
        std::copy(res.begin(), res.end(), out);
        return res.size();
    }

    void ref_hibf_count(void * p, uint64_t const * values, uint64_t n, uint64_t threshold, int width, void * out)
    {
        auto & h = *static_cast<hibf::hierarchical_interleaved_bloom_filter *>(p);
        switch (width)
        {
        case 1:
            hibf_count_into<uint8_t>(h, values, n, threshold, out);
            break;
        case 2:
            hibf_count_into<uint16_t>(h, values, n, threshold, out);
            break;
        case 4:
            hibf_count_into<uint32_t>(h, values, n, threshold, out);
            break;
        default:
            hibf_count_into<uint64_t>(h, values, n, threshold, out);
        }
    }

    // Batched queries over CSR (values, qoffsets), one agent per thread as the reference's thread-safety contract
    // requires (HIBF.hpp:101-105).  Per query: the sorted membership list and the uint16 count vector, reduced to
    //   mem_len[q], mem_digest[q]  -- length and digest of the sorted user-bin list (membership_for + sort_results)
    //   cnt_nnz[q], cnt_digest[q]  -- number and digest of the (user bin, count) pairs with count != 0, ascending
    // If mem_ids != nullptr it receives the sorted lists, query q at mem_ids[q * n_user_bins].
    void ref_hibf_query_batch(void * p,
                              uint64_t const * values,
                              uint64_t const * qoffsets,
                              uint64_t nq,
                              uint16_t const * mem_thresholds,
                              uint64_t const * cnt_thresholds,
                              int threads,
                              uint64_t * mem_len,
                              uint64_t * mem_digest,
                              uint64_t * cnt_nnz,
                              uint64_t * cnt_digest,
                              uint64_t * mem_ids)
    {
        auto & h = *static_cast<hibf::hierarchical_interleaved_bloom_filter *>(p);
        size_t const nub = h.number_of_user_bins;
#pragma omp parallel num_threads(threads)
        {
            auto magent = h.membership_agent();
            auto cagent = h.counting_agent<uint16_t>();
            std::vector<uint64_t> v;
#pragma omp for schedule(dynamic, 16)
            for (uint64_t q = 0; q < nq; ++q)
            {
                v.assign(values + qoffsets[q], values + qoffsets[q + 1]);
                auto & m = magent.membership_for(v, mem_thresholds[q]);
                magent.sort_results();
                uint64_t d = HG_DIGEST_INIT;
                for (auto id : m)
                    d = hg_digest_step(d, id);
                mem_len[q] = m.size();
                mem_digest[q] = d;
                if (mem_ids)
                    std::copy(m.begin(), m.end(), mem_ids + q * nub);
                auto & c = cagent.bulk_count(v, cnt_thresholds[q]);
                uint64_t nnz = 0, cd = HG_DIGEST_INIT;
                for (size_t ub = 0; ub < nub; ++ub)
                    if (c[ub] != 0)
                    {
                        ++nnz;
                        cd = hg_digest_step(hg_digest_step(cd, ub), c[ub]);
                    }
                cnt_nnz[q] = nnz;
                cnt_digest[q] = cd;
            }
        }
    }

    // ---------------------------------------------------------------------------------------------------------
    // serialisation: the reference's serialize functions through the byte archive above (free with ref_free)
    // ---------------------------------------------------------------------------------------------------------
    char * ref_ibf_save(void * p, uint64_t * n)
    {
        try
        {
            return save_bytes(*static_cast<hibf::interleaved_bloom_filter *>(p), n);
        }
        catch (...)
        {
            return nullptr;
        }
    }

    void * ref_ibf_load(char const * bytes, uint64_t n)
    {
        try
        {
            auto ibf = std::make_unique<hibf::interleaved_bloom_filter>();
            byte_in_archive ar;
            ar.bytes = std::string_view{bytes, n};
            ar(*ibf);
            if (ar.pos != n)
                return nullptr;
            return ibf.release();
        }
        catch (...)
        {
            return nullptr;
        }
    }

    char * ref_hibf_save(void * p, uint64_t * n)
    {
        try
        {
            return save_bytes(*static_cast<hibf::hierarchical_interleaved_bloom_filter *>(p), n);
        }
        catch (...)
        {
            return nullptr;
        }
    }

} // extern "C"
