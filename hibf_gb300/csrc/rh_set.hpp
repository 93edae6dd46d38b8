// rh_set.hpp -- the slot order of robin_hood::unordered_flat_set<uint64_t> (robin-hood hashing with linear probing,
// as vendored by the reference in include/hibf/contrib/robin_hood.hpp), restated for the host builder.
//
// The reference's build splits a user bin over several technical bins in chunks of its hash set's iteration order
// (src/build/insert_into_ibf.cpp:28-47), so reproducing its bit store for split user bins needs that order.  The
// order depends on the set's whole history: clear() keeps the table size and hash multiplier, and sets are reused
// across the records of one IBF (src/hierarchical_interleaved_bloom_filter.cpp:39-171).  This class follows the
// published algorithm step by step:
//   slot:   h = murmur3 fmix64 first half of the key; h *= multiplier; h ^= h >> 33; the low 5 bits of h give the
//           info hash, the rest (masked) the home slot; info = info_inc + (hash bits >> info_shift).
//   insert: skip slots with a larger info, compare equal infos, then shift the run up by one slot and store;
//           grow (8 slots first, then double at 80% load) or, when a probe run gets too long at low load, halve
//           info_inc first and finally re-seed the multiplier and rehash in place.
//   order:  iteration visits occupied slots in index order.
#pragma once

#include <algorithm>
#include <cstdint>
#include <stdexcept>
#include <vector>

#if defined(__CUDACC__)
#    define RH_HD __host__ __device__ __forceinline__
#else
#    define RH_HD inline
#endif

namespace hibf_gb300
{

// Home slot of `key` in a table with hash multiplier `mult` and slot mask `mask` (the idx half of rh_set::slot).
// Iteration visits keys in non-decreasing home slot order, so this slot and the table's iteration order within one
// home slot fix a key's rank.
RH_HD uint64_t rh_home(uint64_t key, uint64_t mult, uint64_t mask)
{
    uint64_t h = key;
    h ^= h >> 33;
    h *= 0xff51afd7ed558ccdULL;
    h ^= h >> 33;
    h *= mult;
    h ^= h >> 33;
    return (h >> 5) & mask;
}

class rh_set
{
public:
    void insert(uint64_t key)
    {
        if (keys_.empty())
            init(8); // the first insert of an empty set allocates 8 slots
        for (int attempt = 0; attempt < 256; ++attempt)
        {
            size_t idx{};
            uint32_t info{};
            slot(key, idx, info);
            while (info < info_[idx])
                next(info, idx);
            while (info == info_[idx])
            {
                if (keys_[idx] == key)
                    return;
                next(info, idx);
            }
            if (num_ >= max_allowed_)
            {
                grow();
                continue;
            }
            size_t const at = idx;
            uint32_t const at_info = info;
            if (at_info + info_inc_ > 0xFF)
                max_allowed_ = 0;
            while (info_[idx] != 0)
                next(info, idx);
            if (idx != at)
                shift_up(idx, at);
            keys_[at] = key;
            info_[at] = static_cast<uint8_t>(at_info);
            ++num_;
            return;
        }
        throw std::overflow_error("hash set overflow");
    }

    void clear()
    {
        if (num_ == 0)
            return;
        num_ = 0;
        size_t const n = with_buffer(mask_ + 1);
        std::fill(info_.begin(), info_.begin() + static_cast<std::ptrdiff_t>(n + 8), uint8_t{0});
        info_[n] = 1;
        info_inc_ = kInitialInfoInc;
        info_shift_ = 0;
    }

    size_t size() const
    {
        return num_;
    }

    // The keys in iteration order.
    template <typename F>
    void for_each(F && f) const
    {
        if (num_ == 0)
            return;
        size_t const n = with_buffer(mask_ + 1);
        for (size_t i = 0; i < n; ++i)
            if (info_[i] != 0)
                f(keys_[i]);
    }

    uint64_t multiplier() const
    {
        return mult_;
    }

    uint64_t slot_mask() const
    {
        return mask_;
    }

    std::vector<uint64_t> ordered() const
    {
        std::vector<uint64_t> out;
        out.reserve(num_);
        for_each([&](uint64_t k) { out.push_back(k); });
        return out;
    }

private:
    static constexpr uint32_t kInitialInfoInc = 32; // 1 << 5 info bits
    static constexpr uint64_t kInfoMask = 31;

    static size_t max_allowed(size_t n)
    {
        return n <= SIZE_MAX / 100 ? n * 80 / 100 : (n / 100) * 80;
    }
    static size_t with_buffer(size_t n)
    {
        return n + std::min<size_t>(max_allowed(n), 0xFF);
    }

    void slot(uint64_t key, size_t & idx, uint32_t & info) const
    {
        uint64_t h = key;
        h ^= h >> 33;
        h *= 0xff51afd7ed558ccdULL;
        h ^= h >> 33;
        h *= mult_;
        h ^= h >> 33;
        info = info_inc_ + static_cast<uint32_t>((h & kInfoMask) >> info_shift_);
        idx = (static_cast<size_t>(h) >> 5) & mask_;
    }

    void next(uint32_t & info, size_t & idx) const
    {
        ++idx;
        info += info_inc_;
    }

    void shift_up(size_t start, size_t at)
    {
        for (size_t i = start; i != at; --i)
            keys_[i] = keys_[i - 1];
        for (size_t i = start; i != at; --i)
        {
            info_[i] = static_cast<uint8_t>(info_[i - 1] + info_inc_);
            if (info_[i] + info_inc_ > 0xFF)
                max_allowed_ = 0;
        }
    }

    void init(size_t slots)
    {
        num_ = 0;
        mask_ = slots - 1;
        max_allowed_ = max_allowed(slots);
        size_t const n = with_buffer(slots);
        keys_.assign(n, 0);
        info_.assign(n + 8, 0);
        info_[n] = 1;
        info_inc_ = kInitialInfoInc;
        info_shift_ = 0;
    }

    bool narrow_info()
    {
        if (info_inc_ <= 2)
            return false;
        info_inc_ >>= 1;
        ++info_shift_;
        size_t const n = with_buffer(mask_ + 1);
        size_t const end = (n + 7) / 8 * 8; // whole 8-byte groups, as the reference shifts them
        for (size_t i = 0; i < end; ++i)
            info_[i] = static_cast<uint8_t>((info_[i] >> 1) & 0x7F);
        info_[n] = 1;
        max_allowed_ = max_allowed(mask_ + 1);
        return true;
    }

    void grow()
    {
        if (num_ < max_allowed(mask_ + 1) && narrow_info())
            return;
        if (num_ * 2 < max_allowed(mask_ + 1))
        {
            mult_ += 0xc4ceb9fe1a85ec54ULL;
            rehash(mask_ + 1);
        }
        else
        {
            rehash((mask_ + 1) * 2);
        }
    }

    void rehash(size_t slots)
    {
        std::vector<uint64_t> const old_keys = std::move(keys_);
        std::vector<uint8_t> const old_info = std::move(info_);
        size_t const old_n = with_buffer(mask_ + 1);
        init(slots);
        if (old_n > 1)
            for (size_t i = 0; i < old_n; ++i)
                if (old_info[i] != 0)
                    insert_new(old_keys[i]);
    }

    // Insertion of a key known to be absent (rehash).
    void insert_new(uint64_t key)
    {
        if (max_allowed_ == 0 && !narrow_info())
            throw std::overflow_error("hash set overflow");
        size_t idx{};
        uint32_t info{};
        slot(key, idx, info);
        while (info <= info_[idx])
            next(info, idx);
        size_t const at = idx;
        uint8_t const at_info = static_cast<uint8_t>(info);
        if (at_info + info_inc_ > 0xFF)
            max_allowed_ = 0;
        while (info_[idx] != 0)
            next(info, idx);
        if (idx != at)
            shift_up(idx, at);
        keys_[at] = key;
        info_[at] = at_info;
        ++num_;
    }

    uint64_t mult_{0xc4ceb9fe1a85ec53ULL};
    size_t mask_{0};
    size_t num_{0};
    size_t max_allowed_{0};
    uint32_t info_inc_{kInitialInfoInc};
    uint32_t info_shift_{0};
    std::vector<uint64_t> keys_;
    std::vector<uint8_t> info_;
};

} // namespace hibf_gb300
