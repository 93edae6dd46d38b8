// hibf_gb300.hpp -- C++20 facade over the C ABI (hibf_gb300.h) with the shape of seqan::hibf's public classes, so a
// seqan::hibf user switches by namespace: strong types bin_count / bin_size / hash_function_count / bin_index
// (include/hibf/interleaved_bloom_filter.hpp:51-81), interleaved_bloom_filter with containment / counting /
// membership agents (interleaved_bloom_filter.hpp:225-391, 552-770), config with input_fn and insert_iterator
// (include/hibf/config.hpp:75-413, include/hibf/misc/insert_iterator.hpp:24-111), and
// hierarchical_interleaved_bloom_filter built from a layout with its membership and counting agents
// (include/hibf/hierarchical_interleaved_bloom_filter.hpp:197-247, 322-566).
//
// Errors follow the reference: construction logic errors throw std::logic_error, invalid arguments
// std::invalid_argument, other failures std::runtime_error.  Agents own their result buffers, valid until their next
// call, as in the reference.  Every computation runs on the device; nothing here falls back to the CPU.
#pragma once

#include <algorithm>
#include <compare>
#include <cstddef>
#include <cstdint>
#include <exception>
#include <functional>
#include <limits>
#include <ranges>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "hibf_gb300.h"

namespace hibf_gb300
{

inline void check(int status)
{
    if (status == HIBF_GPU_OK)
        return;
    std::string const msg = hibf_gpu_last_error();
    if (status == HIBF_GPU_ERR_LOGIC)
        throw std::logic_error{msg};
    if (status == HIBF_GPU_ERR_INVALID_ARG)
        throw std::invalid_argument{msg};
    throw std::runtime_error{msg};
}

// Sentinels of ibf_bin_to_user_bin_id (hierarchical_interleaved_bloom_filter.hpp:32-40).
namespace bin_kind
{
static constexpr uint64_t merged{HIBF_GPU_BIN_MERGED};
static constexpr uint64_t deleted{HIBF_GPU_BIN_DELETED};
} // namespace bin_kind

struct bin_count
{
    uint64_t value;
};
struct bin_size
{
    uint64_t value;
};
struct hash_function_count
{
    uint64_t value;
};
struct bin_index
{
    uint64_t value;
};

namespace detail
{
template <std::ranges::input_range values_t>
std::vector<uint64_t> to_vector(values_t && values)
{
    std::vector<uint64_t> v;
    if constexpr (std::ranges::sized_range<values_t>)
        v.reserve(std::ranges::size(values));
    for (auto && x : values)
        v.push_back(static_cast<uint64_t>(x));
    return v;
}

template <typename T>
constexpr int width_of()
{
    static_assert(std::is_integral_v<T> && std::is_unsigned_v<T> && sizeof(T) <= 8, "unsigned counter types");
    return static_cast<int>(sizeof(T));
}
} // namespace detail

// The result of bulk_contains: one bit per bin (the reference's bit_vector, read-only here).
class bit_vector
{
public:
    bit_vector() = default;
    bit_vector(std::vector<uint64_t> words, uint64_t bits) : words_{std::move(words)}, bits_{bits}
    {}
    bool operator[](uint64_t i) const
    {
        return (words_[i / 64] >> (i % 64)) & 1u;
    }
    uint64_t size() const
    {
        return bits_;
    }
    std::vector<uint64_t> const & data() const
    {
        return words_;
    }
    bool operator==(std::vector<bool> const & other) const
    {
        if (other.size() != bits_)
            return false;
        for (uint64_t i = 0; i < bits_; ++i)
            if ((*this)[i] != other[i])
                return false;
        return true;
    }

private:
    std::vector<uint64_t> words_;
    uint64_t bits_{};
};

// What config::input_fn receives: `it = value` inserts one value (insert_iterator.hpp:24-111).
class insert_iterator
{
public:
    explicit insert_iterator(hibf_gpu_sink * sink) : sink_{sink}
    {}
    insert_iterator & operator=(uint64_t value)
    {
        check(hibf_gpu_sink_push(sink_, &value, 1));
        return *this;
    }
    insert_iterator & operator*()
    {
        return *this;
    }
    insert_iterator & operator++()
    {
        return *this;
    }
    insert_iterator & operator++(int)
    {
        return *this;
    }
    // Many values in one call.
    void push(std::vector<uint64_t> const & values)
    {
        check(hibf_gpu_sink_push(sink_, values.data(), values.size()));
    }

private:
    hibf_gpu_sink * sink_;
};

// The fields of seqan::hibf::config the device build uses (config.hpp:75-413).
struct config
{
    std::function<void(size_t const, insert_iterator &&)> input_fn;
    size_t number_of_user_bins{};
    size_t number_of_hash_functions{2};
    double maximum_fpr{0.05};
    double relaxed_fpr{0.3};
    size_t threads{1};
    uint8_t sketch_bits{12};     // picks the largest user bin for interleaved_bloom_filter(config&)
    bool track_occupancy{false}; // interleaved_bloom_filter(config&) only
};

namespace detail
{
// config::input_fn behind the C ABI's callback: the sink is the insert_iterator's target.
inline void input_trampoline(void * user, uint64_t user_bin, hibf_gpu_sink * sink)
{
    auto & c = *static_cast<config *>(user);
    c.input_fn(static_cast<size_t>(user_bin), insert_iterator{sink});
}
} // namespace detail

class interleaved_bloom_filter
{
public:
    interleaved_bloom_filter(hibf_gb300::bin_count bins, hibf_gb300::bin_size size,
                             hibf_gb300::hash_function_count funs = {2},
                             bool track_occupancy_ = false)
    {
        check(hibf_gpu_ibf_create(bins.value, size.value, funs.value, track_occupancy_ ? 1 : 0, &f_));
        adopt();
    }
    // interleaved_bloom_filter(config&, size_t max_bin_elements) (interleaved_bloom_filter.hpp:241,
    // src/interleaved_bloom_filter.cpp:81-117): one technical bin per user bin, the bin size from the exact distinct
    // count of the largest user bin (picked by its HyperLogLog sketch unless max_bin_elements is given), then every
    // user bin's values inserted on the device.
    interleaved_bloom_filter(config & configuration, size_t max_bin_elements = 0)
    {
        if (!configuration.input_fn)
            throw std::invalid_argument{"[HIBF CONFIG ERROR] You did not set the required config::input_fn."};
        hibf_gpu_build_config c{configuration.number_of_user_bins, configuration.number_of_hash_functions,
                                configuration.maximum_fpr, configuration.relaxed_fpr, configuration.threads, 0};
        check(hibf_gpu_ibf_build(&c, max_bin_elements, configuration.sketch_bits,
                                 configuration.track_occupancy ? 1 : 0, &detail::input_trampoline, &configuration,
                                 &f_));
        adopt();
    }
    explicit interleaved_bloom_filter(hibf_gpu_ibf * adopted) : f_{adopted}
    {
        adopt();
    }
    interleaved_bloom_filter(interleaved_bloom_filter const &) = delete;
    interleaved_bloom_filter & operator=(interleaved_bloom_filter const &) = delete;
    interleaved_bloom_filter(interleaved_bloom_filter && o) noexcept :
        occupancy{std::move(o.occupancy)},
        track_occupancy{o.track_occupancy},
        f_{std::exchange(o.f_, nullptr)}
    {}
    ~interleaved_bloom_filter()
    {
        if (f_)
            hibf_gpu_ibf_destroy(f_);
    }

    // The reference's public members (interleaved_bloom_filter.hpp:451-458): one counter per technical bin, non-zero
    // only when the filter tracks occupancy.  This is a host copy of the device's counters, brought up to date by
    // every modifier called through this object.
    std::vector<size_t> occupancy{};
    bool track_occupancy{false};

    void emplace(uint64_t value, bin_index bin)
    {
        check(hibf_gpu_ibf_emplace(f_, &value, 1, bin.value));
        refresh_occupancy();
    }
    // Many values into one bin in one device call (the insert_iterator loop of the reference, batched).
    template <std::ranges::input_range values_t>
    void emplace(values_t && values, bin_index bin)
    {
        auto const v = detail::to_vector(values);
        check(hibf_gpu_ibf_emplace(f_, v.data(), v.size(), bin.value));
        refresh_occupancy();
    }
    void clear(bin_index bin)
    {
        check(hibf_gpu_ibf_clear(f_, bin.value));
        refresh_occupancy();
    }
    template <std::ranges::forward_range bins_t>
        requires std::same_as<std::ranges::range_value_t<bins_t>, bin_index>
    void clear(bins_t && bins)
    {
        std::vector<uint64_t> b;
        for (bin_index x : bins)
            b.push_back(x.value);
        check(hibf_gpu_ibf_clear_range(f_, b.data(), b.size()));
        refresh_occupancy();
    }
    bool try_increase_bin_number_to(hibf_gb300::bin_count new_bins)
    {
        int ok = 0;
        check(hibf_gpu_ibf_try_increase_bin_number_to(f_, new_bins.value, &ok));
        return ok != 0;
    }
    void increase_bin_number_to(hibf_gb300::bin_count new_bins)
    {
        check(hibf_gpu_ibf_increase_bin_number_to(f_, new_bins.value));
        load_occupancy(); // technical_bins may have grown
    }

    uint64_t bin_count() const
    {
        return info()[0];
    }
    uint64_t bin_size() const
    {
        return info()[1];
    }
    uint64_t hash_function_count() const
    {
        return info()[2];
    }
    uint64_t bit_size() const
    {
        return info()[3];
    }

    class containment_agent_type
    {
    public:
        explicit containment_agent_type(interleaved_bloom_filter const & ibf) : ibf_{&ibf}
        {}
        bit_vector const & bulk_contains(uint64_t value) & noexcept
        {
            uint64_t const words = (ibf_->bin_count() + 63) / 64;
            std::vector<uint64_t> w(words);
            if (hibf_gpu_ibf_bulk_contains(ibf_->f_, &value, 1, w.data()) != HIBF_GPU_OK)
                std::terminate(); // queries are noexcept in the reference
            result_ = bit_vector{std::move(w), ibf_->bin_count()};
            return result_;
        }

    private:
        interleaved_bloom_filter const * ibf_;
        bit_vector result_;
    };

    template <typename value_t = uint16_t>
    class counting_agent_type
    {
    public:
        explicit counting_agent_type(interleaved_bloom_filter const & ibf) : ibf_{&ibf}
        {}
        template <std::ranges::input_range values_t>
        std::vector<value_t> const & bulk_count(values_t && values) & noexcept
        {
            auto const v = detail::to_vector(values);
            result_.assign(ibf_->bin_count(), 0);
            if (hibf_gpu_ibf_bulk_count(ibf_->f_, v.data(), v.size(), detail::width_of<value_t>(), result_.data()) !=
                HIBF_GPU_OK)
                std::terminate();
            return result_;
        }

    private:
        interleaved_bloom_filter const * ibf_;
        std::vector<value_t> result_;
    };

    class membership_agent_type
    {
    public:
        explicit membership_agent_type(interleaved_bloom_filter const & ibf) : ibf_{&ibf}
        {}
        template <std::ranges::input_range values_t>
        std::vector<uint64_t> const & membership_for(values_t && values, uint16_t threshold) & noexcept
        {
            auto const v = detail::to_vector(values);
            result_.resize(ibf_->bin_count());
            uint64_t n = 0;
            if (hibf_gpu_ibf_membership_for(ibf_->f_, v.data(), v.size(), threshold, result_.data(), &n) !=
                HIBF_GPU_OK)
                std::terminate();
            result_.resize(n);
            return result_;
        }
        // Has no effect, as in the reference (interleaved_bloom_filter.hpp:712-720): the ids are already ascending.
        void sort_results()
        {}

    private:
        interleaved_bloom_filter const * ibf_;
        std::vector<uint64_t> result_;
    };

    containment_agent_type containment_agent() const
    {
        return containment_agent_type{*this};
    }
    template <typename value_t = uint16_t>
    counting_agent_type<value_t> counting_agent() const
    {
        return counting_agent_type<value_t>{*this};
    }
    membership_agent_type membership_agent() const
    {
        return membership_agent_type{*this};
    }

    void save(std::string const & path) const
    {
        check(hibf_gpu_ibf_save(f_, path.c_str()));
    }
    static interleaved_bloom_filter load(std::string const & path)
    {
        hibf_gpu_ibf * f = nullptr;
        check(hibf_gpu_ibf_load(path.c_str(), &f));
        return interleaved_bloom_filter{f};
    }
    hibf_gpu_ibf * handle() const
    {
        return f_;
    }

    // Equal shape, bits, occupancy and tracking flag (the reference's defaulted operator==,
    // interleaved_bloom_filter.hpp:433).  The bit stores are compared through host copies.
    bool operator==(interleaved_bloom_filter const & other) const
    {
        auto const a = info(), b = other.info();
        if (a[0] != b[0] || a[1] != b[1] || a[2] != b[2] || track_occupancy != other.track_occupancy ||
            occupancy != other.occupancy)
            return false;
        return words() == other.words();
    }

private:
    std::vector<uint64_t> words() const
    {
        auto const i = info();
        std::vector<uint64_t> w((i[0] + 63) / 64 * i[1]);
        check(hibf_gpu_ibf_download_words(f_, w.data(), w.size()));
        return w;
    }
    std::vector<uint64_t> info() const
    {
        std::vector<uint64_t> out(5);
        check(hibf_gpu_ibf_info(f_, out.data()));
        return out;
    }
    // Takes the new handle's occupancy; on failure releases the handle, since no destructor will run.
    void adopt()
    {
        try
        {
            load_occupancy();
        }
        catch (...)
        {
            hibf_gpu_ibf_destroy(std::exchange(f_, nullptr));
            throw;
        }
    }
    // Sizes occupancy to the technical bins and reads the tracking flag and the counters.
    void load_occupancy()
    {
        int tracks = 0;
        check(hibf_gpu_ibf_track_occupancy(f_, &tracks));
        track_occupancy = tracks != 0;
        auto const i = info();
        occupancy.assign(i[3] / i[1], 0u); // bit size / bin size = technical bins
        refresh_occupancy();
    }
    void refresh_occupancy()
    {
        if (!track_occupancy)
            return;
        static_assert(sizeof(size_t) == sizeof(uint64_t));
        check(hibf_gpu_ibf_download_occupancy(f_, reinterpret_cast<uint64_t *>(occupancy.data()), occupancy.size()));
    }
    hibf_gpu_ibf * f_{};
};

// The read side of the reference's concurrent_timer (include/hibf/misc/timer.hpp): a build phase's seconds, its
// longest interval and the interval count.
class build_timer
{
public:
    build_timer() = default;
    explicit build_timer(hibf_gpu_timer const & t) : t_{t} {}
    double in_seconds() const
    {
        return t_.seconds;
    }
    double max_in_seconds() const
    {
        return t_.max_seconds;
    }
    // as in the reference, only meaningful once an interval was added
    double avg_in_seconds() const
    {
        return t_.count ? t_.seconds / static_cast<double>(t_.count) : 0.0;
    }
    uint64_t count() const
    {
        return t_.count;
    }

private:
    hibf_gpu_timer t_{};
};

class hierarchical_interleaved_bloom_filter
{
public:
    // hierarchical_interleaved_bloom_filter(config&, layout const&) with the reference's layout file text.
    hierarchical_interleaved_bloom_filter(config & configuration, std::string const & layout_text)
    {
        if (!configuration.input_fn)
            throw std::invalid_argument{"[HIBF CONFIG ERROR] You did not set the required config::input_fn."};
        hibf_gpu_build_config c{configuration.number_of_user_bins, configuration.number_of_hash_functions,
                                configuration.maximum_fpr, configuration.relaxed_fpr, configuration.threads, 0};
        check(hibf_gpu_hibf_build(&c, layout_text.c_str(), &detail::input_trampoline, &configuration, &h_));
        adopt();
    }
    explicit hierarchical_interleaved_bloom_filter(hibf_gpu_hibf * adopted) : h_{adopted}
    {
        adopt();
    }
    hierarchical_interleaved_bloom_filter(hierarchical_interleaved_bloom_filter const &) = delete;
    hierarchical_interleaved_bloom_filter & operator=(hierarchical_interleaved_bloom_filter const &) = delete;
    hierarchical_interleaved_bloom_filter(hierarchical_interleaved_bloom_filter && o) noexcept :
        number_of_user_bins{o.number_of_user_bins},
        next_ibf_id{std::move(o.next_ibf_id)},
        prev_ibf_id{std::move(o.prev_ibf_id)},
        ibf_bin_to_user_bin_id{std::move(o.ibf_bin_to_user_bin_id)},
        index_allocation_timer{o.index_allocation_timer},
        user_bin_io_timer{o.user_bin_io_timer},
        merge_kmers_timer{o.merge_kmers_timer},
        fill_ibf_timer{o.fill_ibf_timer},
        h_{std::exchange(o.h_, nullptr)}
    {}
    ~hierarchical_interleaved_bloom_filter()
    {
        if (h_)
            hibf_gpu_hibf_destroy(h_);
    }

    size_t number_of_user_bins{};

    // The tables (hierarchical_interleaved_bloom_filter.hpp:208-238, 296-301), host copies read at construction:
    // per IBF and technical bin the child IBF (the IBF itself for a leaf bin) and the user bin (bin_kind::merged or
    // bin_kind::deleted), and per IBF its parent IBF and bin.  The IBFs themselves stay on the device (their shapes:
    // hibf_gpu_hibf_ibf_info).
    struct previous_ibf_id_pair
    {
        size_t ibf_idx{};
        size_t bin_idx{};
        friend constexpr auto operator<=>(previous_ibf_id_pair const &, previous_ibf_id_pair const &) = default;
    };
    std::vector<std::vector<uint64_t>> next_ibf_id;
    std::vector<previous_ibf_id_pair> prev_ibf_id;
    std::vector<std::vector<uint64_t>> ibf_bin_to_user_bin_id{};

    // The build's phase timers (hierarchical_interleaved_bloom_filter.hpp:283-290); zero unless this object was
    // built.  The layout_* timers of the reference time the layout computation, which seqan::hibf keeps.
    build_timer index_allocation_timer{};
    build_timer user_bin_io_timer{};
    build_timer merge_kmers_timer{};
    build_timer fill_ibf_timer{};

    class membership_agent_type
    {
    public:
        explicit membership_agent_type(hierarchical_interleaved_bloom_filter const & h) : h_{&h}
        {
            check(hibf_gpu_agent_create(h.h_, &a_));
        }
        membership_agent_type(membership_agent_type && o) noexcept :
            h_{o.h_},
            a_{std::exchange(o.a_, nullptr)},
            result_{std::move(o.result_)}
        {}
        ~membership_agent_type()
        {
            if (a_)
                hibf_gpu_agent_destroy(a_);
        }
        // User bins whose summed counts reach the threshold, in the reference's traversal order
        // (hierarchical_interleaved_bloom_filter.hpp:322-355, 424-439).
        template <std::ranges::input_range values_t>
        std::vector<uint64_t> const & membership_for(values_t && values, uint16_t threshold) & noexcept
        {
            auto const v = detail::to_vector(values);
            uint64_t const * ids = nullptr;
            uint64_t n = 0;
            if (hibf_gpu_agent_membership_for_unsorted(a_, v.data(), v.size(), threshold, &ids, &n) != HIBF_GPU_OK)
                std::terminate();
            result_.assign(ids, ids + n);
            return result_;
        }
        // hierarchical_interleaved_bloom_filter.hpp:380-383
        void sort_results()
        {
            std::ranges::sort(result_);
        }

        // Many queries in one persistent launch (no counterpart in the reference): query q is
        // values[offsets[q] .. offsets[q + 1]) with threshold thresholds[q]; its user bins are
        // ids[result_offsets[q] .. result_offsets[q + 1]), ascending (membership_for + sort_results).  Batches of at
        // least 64 MiB of values are streamed to the device.  Failures throw (std::invalid_argument, ...).
        struct batch_result
        {
            std::vector<uint64_t> offsets;
            std::vector<uint64_t> ids;
        };
        batch_result const & membership_for_batch(std::vector<uint64_t> const & values,
                                                  std::vector<uint64_t> const & offsets,
                                                  std::vector<uint16_t> const & thresholds) &
        {
            if (offsets.empty() || thresholds.size() + 1 != offsets.size() || offsets.back() > values.size())
                throw std::invalid_argument{"membership_for_batch: offsets must have one entry per query plus one"};
            std::vector<uint64_t> const t(thresholds.begin(), thresholds.end());
            uint64_t const nq = thresholds.size();
            uint64_t const *ro = nullptr, *ri = nullptr;
            check(hibf_gpu_agent_query_batch(a_, HIBF_GPU_QUERY_MEMBERSHIP, values.data(), offsets.data(), nq,
                                             t.data(), 2, &ro, &ri, nullptr));
            batch_.offsets.assign(ro, ro + nq + 1);
            batch_.ids.assign(ri, ri + batch_.offsets.back());
            return batch_;
        }

    private:
        hierarchical_interleaved_bloom_filter const * h_;
        hibf_gpu_agent * a_{};
        std::vector<uint64_t> result_;
        batch_result batch_;
    };

    template <typename value_t = uint16_t>
    class counting_agent_type
    {
    public:
        explicit counting_agent_type(hierarchical_interleaved_bloom_filter const & h) : h_{&h}
        {
            check(hibf_gpu_agent_create(h.h_, &a_));
        }
        counting_agent_type(counting_agent_type && o) noexcept :
            h_{o.h_},
            a_{std::exchange(o.a_, nullptr)},
            result_{std::move(o.result_)}
        {}
        ~counting_agent_type()
        {
            if (a_)
                hibf_gpu_agent_destroy(a_);
        }
        // hierarchical_interleaved_bloom_filter.hpp:463-566: per user bin the summed count if it reaches t, else 0.
        template <std::ranges::input_range values_t>
        std::vector<value_t> const & bulk_count(values_t && values, size_t threshold) & noexcept
        {
            auto const v = detail::to_vector(values);
            void const * counts = nullptr;
            if (hibf_gpu_agent_bulk_count(a_, v.data(), v.size(), threshold, detail::width_of<value_t>(), &counts) !=
                HIBF_GPU_OK)
                std::terminate();
            auto const * c = static_cast<value_t const *>(counts);
            result_.assign(c, c + h_->number_of_user_bins);
            return result_;
        }

        // Many queries in one persistent launch (no counterpart in the reference): query q's counting vector as
        // bulk_count(values[offsets[q] .. offsets[q + 1]), thresholds[q]) returns it, stored sparsely: its non-zero
        // entries are counts[result_offsets[q] ..] for the ascending user bins ids[result_offsets[q] ..].
        struct batch_result
        {
            std::vector<uint64_t> offsets;
            std::vector<uint64_t> ids;
            std::vector<value_t> counts;
        };
        batch_result const & bulk_count_batch(std::vector<uint64_t> const & values, std::vector<uint64_t> const & offsets,
                                              std::vector<uint64_t> const & thresholds) &
        {
            if (offsets.empty() || thresholds.size() + 1 != offsets.size() || offsets.back() > values.size())
                throw std::invalid_argument{"bulk_count_batch: offsets must have one entry per query plus one"};
            uint64_t const nq = thresholds.size();
            uint64_t const *ro = nullptr, *ri = nullptr;
            void const * rc = nullptr;
            check(hibf_gpu_agent_query_batch(a_, HIBF_GPU_QUERY_COUNT, values.data(), offsets.data(), nq,
                                             thresholds.data(), detail::width_of<value_t>(), &ro, &ri, &rc));
            batch_.offsets.assign(ro, ro + nq + 1);
            uint64_t const nr = batch_.offsets.back();
            batch_.ids.assign(ri, ri + nr);
            auto const * c = static_cast<value_t const *>(rc);
            batch_.counts.assign(c, c + nr);
            return batch_;
        }

    private:
        hierarchical_interleaved_bloom_filter const * h_;
        hibf_gpu_agent * a_{};
        std::vector<value_t> result_;
        batch_result batch_;
    };

    membership_agent_type membership_agent() const
    {
        return membership_agent_type{*this};
    }
    template <typename value_t = uint16_t>
    counting_agent_type<value_t> counting_agent() const
    {
        return counting_agent_type<value_t>{*this};
    }

    void save(std::string const & path) const
    {
        check(hibf_gpu_hibf_save(h_, path.c_str()));
    }
    static hierarchical_interleaved_bloom_filter load(std::string const & path)
    {
        hibf_gpu_hibf * h = nullptr;
        check(hibf_gpu_hibf_load(path.c_str(), &h));
        return hierarchical_interleaved_bloom_filter{h};
    }
    hibf_gpu_hibf * handle() const
    {
        return h_;
    }

    // Equal user bin count, tables, IBF shapes and bits (the reference's defaulted operator==,
    // hierarchical_interleaved_bloom_filter.hpp:252, 312; its timers always compare equal).  The bit stores are
    // compared IBF by IBF through host copies; the occupancy counters of the IBFs are not compared.
    bool operator==(hierarchical_interleaved_bloom_filter const & other) const
    {
        if (number_of_user_bins != other.number_of_user_bins || next_ibf_id != other.next_ibf_id ||
            prev_ibf_id != other.prev_ibf_id || ibf_bin_to_user_bin_id != other.ibf_bin_to_user_bin_id)
            return false;
        std::vector<uint64_t> wa, wb;
        for (uint64_t k = 0; k < next_ibf_id.size(); ++k)
        {
            uint64_t a[5], b[5];
            check(hibf_gpu_hibf_ibf_info(h_, k, a));
            check(hibf_gpu_hibf_ibf_info(other.h_, k, b));
            if (!std::equal(a, a + 4, b)) // bins, technical bins, bin size, hash functions
                return false;
            wa.resize(a[1] / 64 * a[2]);
            wb.resize(wa.size());
            check(hibf_gpu_hibf_download_words(h_, k, wa.data(), wa.size()));
            check(hibf_gpu_hibf_download_words(other.h_, k, wb.data(), wb.size()));
            if (wa != wb)
                return false;
        }
        return true;
    }

private:
    // Reads the new handle's tables; on failure releases the handle, since no destructor will run.
    void adopt()
    {
        try
        {
            load_tables();
        }
        catch (...)
        {
            hibf_gpu_hibf_destroy(std::exchange(h_, nullptr));
            throw;
        }
    }

    void load_tables()
    {
        uint64_t info[4];
        check(hibf_gpu_hibf_info(h_, info));
        number_of_user_bins = info[0];
        uint64_t const n_ibfs = info[1];
        std::vector<uint64_t> bins(n_ibfs), prev_ibf(n_ibfs), prev_bin(n_ibfs);
        check(hibf_gpu_hibf_get_tables(h_, bins.data(), nullptr, nullptr, nullptr, nullptr));
        uint64_t total = 0;
        for (uint64_t const b : bins)
            total += b;
        std::vector<uint64_t> next(total), user_bin(total);
        check(hibf_gpu_hibf_get_tables(h_, nullptr, nullptr, nullptr, next.data(), user_bin.data()));
        check(hibf_gpu_hibf_get_prev(h_, prev_ibf.data(), prev_bin.data()));
        next_ibf_id.assign(n_ibfs, {});
        ibf_bin_to_user_bin_id.assign(n_ibfs, {});
        prev_ibf_id.assign(n_ibfs, {});
        for (uint64_t k = 0, at = 0; k < n_ibfs; at += bins[k], ++k)
        {
            auto const first = next.begin() + static_cast<std::ptrdiff_t>(at);
            auto const last = first + static_cast<std::ptrdiff_t>(bins[k]);
            next_ibf_id[k].assign(first, last);
            ibf_bin_to_user_bin_id[k].assign(user_bin.begin() + (first - next.begin()),
                                             user_bin.begin() + (last - next.begin()));
            prev_ibf_id[k] = previous_ibf_id_pair{prev_ibf[k], prev_bin[k]};
        }
        hibf_gpu_timer t[HIBF_GPU_TIMER_COUNT];
        check(hibf_gpu_hibf_build_timers(h_, t));
        index_allocation_timer = build_timer{t[HIBF_GPU_TIMER_INDEX_ALLOCATION]};
        user_bin_io_timer = build_timer{t[HIBF_GPU_TIMER_USER_BIN_IO]};
        merge_kmers_timer = build_timer{t[HIBF_GPU_TIMER_MERGE_KMERS]};
        fill_ibf_timer = build_timer{t[HIBF_GPU_TIMER_FILL_IBF]};
    }

    hibf_gpu_hibf * h_{};
};

} // namespace hibf_gb300
