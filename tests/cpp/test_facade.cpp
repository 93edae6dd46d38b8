// The C++ facade (include/hibf_gb300.hpp) exercised like the reference's own unit tests
// (test/unit/hibf/interleaved_bloom_filter_test.cpp, test/unit/hibf/hierarchical_interleaved_bloom_filter_test.cpp,
// test/snippet/readme.cpp), with the expectations those tests state.  Usage: test_facade <dir with layout files>.
// Exits 0 when every check holds.
#include <algorithm>
#include <cstdio>
#include <fstream>
#include <functional>
#include <numeric>
#include <sstream>
#include <string>
#include <vector>

#include "hibf_gb300.hpp"

namespace h = hibf_gb300;

static int failures = 0;

#define CHECK(cond)                                                                                                     \
    do                                                                                                                 \
    {                                                                                                                  \
        if (!(cond))                                                                                                   \
        {                                                                                                              \
            std::fprintf(stderr, "%s:%d: CHECK failed: %s\n", __FILE__, __LINE__, #cond);                              \
            ++failures;                                                                                                \
        }                                                                                                              \
    } while (0)

template <typename F, typename E>
bool throws(F && f)
{
    try
    {
        f();
    }
    catch (E const &)
    {
        return true;
    }
    catch (...)
    {
        return false;
    }
    return false;
}

static std::string read_file(std::string const & path)
{
    std::ifstream in{path};
    std::stringstream ss;
    ss << in.rdbuf();
    return ss.str();
}

static std::vector<uint64_t> iota(uint64_t n)
{
    std::vector<uint64_t> v(n);
    std::iota(v.begin(), v.end(), 0u);
    return v;
}

// interleaved_bloom_filter_test.cpp: construction
static void ibf_construction()
{
    CHECK((throws<void (*)(), std::logic_error>(+[] { h::interleaved_bloom_filter{h::bin_count{64}, h::bin_size{0}}; })));
    CHECK((throws<void (*)(), std::logic_error>(+[] { h::interleaved_bloom_filter{h::bin_count{0}, h::bin_size{32}}; })));
    h::interleaved_bloom_filter ibf{h::bin_count{64}, h::bin_size{1024}};
    CHECK(ibf.bin_count() == 64 && ibf.bin_size() == 1024 && ibf.hash_function_count() == 2);
}

// interleaved_bloom_filter_test.cpp: bulk_contains on an empty filter, then after emplace
static void ibf_contains()
{
    h::interleaved_bloom_filter ibf{h::bin_count{64}, h::bin_size{1024}};
    auto agent = ibf.containment_agent();
    for (uint64_t v = 0; v < 64; ++v)
        CHECK(agent.bulk_contains(v) == std::vector<bool>(64, false));
    for (uint64_t b = 0; b < 64; ++b)
        ibf.emplace(b, h::bin_index{b});
    for (uint64_t v = 0; v < 64; ++v)
        CHECK(agent.bulk_contains(v)[v]);
}

// interleaved_bloom_filter_test.cpp: counting (every bin holds 0..127, so every count is 128)
static void ibf_counting()
{
    h::interleaved_bloom_filter ibf{h::bin_count{128}, h::bin_size{1024}, h::hash_function_count{2}};
    for (uint64_t b = 0; b < 128; ++b)
        ibf.emplace(iota(128), h::bin_index{b});
    auto agent = ibf.counting_agent<uint64_t>();
    CHECK(agent.bulk_count(iota(128)) == std::vector<uint64_t>(128, 128));
    auto agent8 = ibf.counting_agent<uint8_t>(); // 128 * 3 wraps modulo 256
    std::vector<uint64_t> thrice = iota(128);
    thrice.insert(thrice.end(), thrice.begin(), thrice.end());
    thrice.insert(thrice.end(), thrice.begin(), thrice.begin() + 128);
    CHECK(agent8.bulk_count(thrice) == std::vector<uint8_t>(128, static_cast<uint8_t>(384 % 256)));
}

// interleaved_bloom_filter_test.cpp: clear and clear(range)
static void ibf_clear()
{
    h::interleaved_bloom_filter ibf{h::bin_count{64}, h::bin_size{1024}};
    for (uint64_t b = 0; b < 64; ++b)
        ibf.emplace(iota(50), h::bin_index{b});
    ibf.clear(h::bin_index{17});
    std::vector<h::bin_index> r{h::bin_index{3}, h::bin_index{40}};
    ibf.clear(r);
    auto agent = ibf.counting_agent<uint16_t>(); // agents are lvalues, as in the reference (rvalue calls deleted)
    auto const & counts = agent.bulk_count(iota(50));
    for (uint64_t b = 0; b < 64; ++b)
        CHECK(counts[b] == ((b == 17 || b == 3 || b == 40) ? 0 : 50));
}

// interleaved_bloom_filter_test.cpp: membership_for (user bins {1..10}, {1..5}; query 1..5, threshold 2)
static void ibf_membership()
{
    h::interleaved_bloom_filter ibf{h::bin_count{2}, h::bin_size{1024}};
    for (uint64_t v = 1; v <= 10; ++v)
        ibf.emplace(v, h::bin_index{0});
    for (uint64_t v = 1; v <= 5; ++v)
        ibf.emplace(v, h::bin_index{1});
    auto agent = ibf.membership_agent();
    std::vector<uint64_t> const query{1, 2, 3, 4, 5};
    CHECK(agent.membership_for(query, 2) == (std::vector<uint64_t>{0, 1}));
    CHECK(agent.membership_for(std::vector<uint64_t>{6, 7, 8}, 2) == (std::vector<uint64_t>{0}));
}

// interleaved_bloom_filter_test.cpp: increase_bin_number_to keeps the content
static void ibf_increase()
{
    h::interleaved_bloom_filter ibf{h::bin_count{73}, h::bin_size{1024}};
    ibf.emplace(iota(30), h::bin_index{72});
    CHECK(ibf.try_increase_bin_number_to(h::bin_count{128}));
    CHECK(ibf.bin_count() == 128);
    CHECK(!ibf.try_increase_bin_number_to(h::bin_count{129}) || ibf.bin_count() == 129);
    auto agent = ibf.counting_agent<uint16_t>();
    auto const & counts = agent.bulk_count(iota(30));
    CHECK(counts[72] == 30);
    CHECK((throws<void (*)(), std::invalid_argument>(+[] {
        h::interleaved_bloom_filter f{h::bin_count{64}, h::bin_size{8}};
        f.increase_bin_number_to(h::bin_count{32});
    })));
}

// interleaved_bloom_filter_test.cpp: construction_from_config, construction_from_config_with_max_bin_elements and
// membership_for through the config constructor (user bins {1..10} and {0, 2, 3, 4, 5}, or {1..5})
static void ibf_from_config()
{
    std::vector<std::vector<uint64_t>> hashes{{1, 2, 3, 4, 5, 6, 7, 8, 9, 10}, {0, 2, 3, 4, 5}};
    h::config cfg{};
    cfg.input_fn = [&](size_t const num, h::insert_iterator it)
    {
        for (uint64_t const v : hashes[num])
            it = v;
    };
    cfg.number_of_user_bins = hashes.size();
    h::interleaved_bloom_filter ibf{cfg};
    CHECK(ibf.bin_count() == 2);
    auto agent = ibf.containment_agent();
    CHECK(agent.bulk_contains(2) == (std::vector<bool>{true, true}));
    CHECK(agent.bulk_contains(8) == (std::vector<bool>{true, false}));
    CHECK(agent.bulk_contains(0) == (std::vector<bool>{false, true}));

    h::interleaved_bloom_filter default_num_elements{cfg, 0u};
    h::interleaved_bloom_filter appropriate_num_elements{cfg, 10u};
    h::interleaved_bloom_filter larger_num_elements{cfg, 20u};
    CHECK(ibf == default_num_elements);
    CHECK(ibf == appropriate_num_elements);
    CHECK(!(ibf == larger_num_elements));
    CHECK(!(appropriate_num_elements == larger_num_elements));

    hashes[1] = {1, 2, 3, 4, 5};
    h::interleaved_bloom_filter both{cfg};
    auto m = both.membership_agent();
    auto const & result = m.membership_for(std::vector<uint64_t>{1, 2, 3, 4, 5}, 2u);
    CHECK(result == (std::vector<uint64_t>{0, 1}));
    m.sort_results();
    CHECK(result == (std::vector<uint64_t>{0, 1}));

    h::config no_input{};
    no_input.number_of_user_bins = 2;
    CHECK((throws<std::function<void()>, std::invalid_argument>([&] { h::interleaved_bloom_filter f{no_input}; })));
}

// interleaved_bloom_filter_test.cpp: emplace (occupancy untracked: technical_bins zeros) and emplace_with_occupancy
// (128 bins, bins 0-63 filled: their counters non-zero, the rest zero), clear resets a bin's counter
static void ibf_occupancy()
{
    h::interleaved_bloom_filter plain{h::bin_count{64}, h::bin_size{1024}};
    for (uint64_t b = 0; b < 64; ++b)
        for (uint64_t v = 0; v < 64; ++v)
            plain.emplace(v, h::bin_index{b});
    CHECK(!plain.track_occupancy);
    CHECK(plain.occupancy.size() == 64u);
    CHECK(std::ranges::all_of(plain.occupancy, [](size_t const occ) { return occ == 0u; }));

    h::interleaved_bloom_filter ibf{h::bin_count{128}, h::bin_size{512}, h::hash_function_count{2}, true};
    CHECK(ibf.track_occupancy);
    for (uint64_t b = 0; b < 64; ++b)
        for (uint64_t v = 0; v < 64; ++v)
            ibf.emplace(v, h::bin_index{b});
    auto agent = ibf.containment_agent();
    std::vector<bool> expected(128);
    std::fill(expected.begin(), expected.begin() + 64, true);
    for (uint64_t v = 0; v < 64; ++v)
        CHECK(agent.bulk_contains(v) == expected);
    CHECK(ibf.occupancy.size() == 128u);
    for (uint64_t b = 0; b < 64; ++b)
        CHECK(ibf.occupancy[b] != 0u);
    for (uint64_t b = 64; b < 128; ++b)
        CHECK(ibf.occupancy[b] == 0u);
    ibf.clear(h::bin_index{5});
    CHECK(ibf.occupancy[5] == 0u && ibf.occupancy[6] != 0u);
    ibf.increase_bin_number_to(h::bin_count{200});
    CHECK(ibf.occupancy.size() == 256u && ibf.occupancy[6] != 0u && ibf.occupancy[199] == 0u);
    h::interleaved_bloom_filter moved{std::move(ibf)};
    CHECK(moved.track_occupancy && moved.occupancy.size() == 256u);
}

// hierarchical_interleaved_bloom_filter_test.cpp small example and test/snippet/readme.cpp, with the layouts the
// reference computes for them.
// The tables' conventions (hierarchical_interleaved_bloom_filter.hpp:208-238): a merged bin names its child IBF, whose
// parent entry is that bin (or (0, 0), as the reference's build leaves it for some children); any other bin names
// its own IBF and a user bin (or bin_kind::deleted); every user bin appears.
static void check_tables(h::hierarchical_interleaved_bloom_filter const & hibf)
{
    size_t const n = hibf.next_ibf_id.size();
    CHECK(n >= 1 && hibf.ibf_bin_to_user_bin_id.size() == n && hibf.prev_ibf_id.size() == n);
    std::vector<bool> seen(hibf.number_of_user_bins);
    for (size_t k = 0; k < n; ++k)
    {
        CHECK(hibf.next_ibf_id[k].size() == hibf.ibf_bin_to_user_bin_id[k].size());
        for (size_t b = 0; b < hibf.next_ibf_id[k].size(); ++b)
        {
            uint64_t const ub = hibf.ibf_bin_to_user_bin_id[k][b];
            uint64_t const next = hibf.next_ibf_id[k][b];
            if (ub == h::bin_kind::merged)
            {
                CHECK(next != k && next < n);
                if (next < n)
                {
                    auto const p = hibf.prev_ibf_id[next];
                    using pair = h::hierarchical_interleaved_bloom_filter::previous_ibf_id_pair;
                    CHECK((p == pair{k, b}) || (p == pair{0, 0}));
                }
            }
            else
            {
                CHECK(next == k);
                CHECK(ub == h::bin_kind::deleted || ub < hibf.number_of_user_bins);
                if (ub < hibf.number_of_user_bins)
                    seen[ub] = true;
            }
        }
    }
    CHECK(std::ranges::all_of(seen, [](bool x) { return x; }));
}

static void hibf_small(std::string const & dir)
{
    std::vector<std::vector<uint64_t>> hashes{{1, 2, 3, 4, 5, 6, 7, 8, 9, 10}, {1, 2, 3, 4, 5}};
    h::config config{.input_fn =
                         [&](size_t const num, h::insert_iterator && it)
                     {
                         for (auto const hash : hashes[num])
                             it = hash;
                     },
                     .number_of_user_bins = 2};
    h::hierarchical_interleaved_bloom_filter hibf{config, read_file(dir + "/layout_snippet.txt")};
    auto agent = hibf.membership_agent();
    std::vector<uint64_t> const query{1, 2, 3, 4, 5};
    auto & result = agent.membership_for(query, 2);
    agent.sort_results();
    CHECK(result == (std::vector<uint64_t>{0, 1}));
    CHECK(hibf.number_of_user_bins == 2);
    check_tables(hibf);
    // the build's timers: two user bins read, one allocation, one fill
    CHECK(hibf.user_bin_io_timer.count() == 3 && hibf.user_bin_io_timer.in_seconds() > 0.0);
    CHECK(hibf.index_allocation_timer.count() == 1 && hibf.fill_ibf_timer.count() == 1);
    CHECK(hibf.fill_ibf_timer.max_in_seconds() == hibf.fill_ibf_timer.in_seconds());
    CHECK(hibf.merge_kmers_timer.avg_in_seconds() <= hibf.merge_kmers_timer.max_in_seconds());
    // copy_agents: counting {5, 5} at threshold 1 and {0, 0} at threshold 6
    auto counter = hibf.counting_agent<uint16_t>();
    CHECK(counter.bulk_count(query, 1) == (std::vector<uint16_t>{5, 5}));
    CHECK(counter.bulk_count(query, 6) == (std::vector<uint16_t>{0, 0}));
}

static void hibf_readme(std::string const & dir)
{
    std::vector<std::vector<uint64_t>> hashes{{1, 2, 3, 4, 5, 6, 7, 8, 9, 10}, {1, 2, 3, 4, 5}, {3, 9, 11}};
    h::config config{.input_fn =
                         [&](size_t const num, h::insert_iterator && it)
                     {
                         for (auto const hash : hashes[num])
                             it = hash;
                     },
                     .number_of_user_bins = 3};
    h::hierarchical_interleaved_bloom_filter hibf{config, read_file(dir + "/layout_readme.txt")};
    auto agent = hibf.membership_agent();
    // test/snippet/readme.out: "2 0" unsorted, then "0 1" for 0..14 at threshold 5 after sort_results()
    CHECK(agent.membership_for(std::vector<uint64_t>{3, 9, 12, 14}, 2) == (std::vector<uint64_t>{2, 0}));
    auto & r = agent.membership_for(iota(15), 5);
    agent.sort_results();
    CHECK(r == (std::vector<uint64_t>{0, 1}));
    // save and load keep the answers
    hibf.save(dir + "/readme.hibf");
    auto loaded = h::hierarchical_interleaved_bloom_filter::load(dir + "/readme.hibf");
    auto agent2 = loaded.membership_agent();
    CHECK(agent2.membership_for(std::vector<uint64_t>{3, 9, 12, 14}, 2) == (std::vector<uint64_t>{2, 0}));
    check_tables(hibf);
    CHECK(loaded == hibf);
    CHECK(loaded.next_ibf_id == hibf.next_ibf_id && loaded.prev_ibf_id == hibf.prev_ibf_id);
    // same layout and tables, other bits: not equal
    hashes[2] = {3, 9, 12};
    h::hierarchical_interleaved_bloom_filter other{config, read_file(dir + "/layout_readme.txt")};
    CHECK(other.ibf_bin_to_user_bin_id == hibf.ibf_bin_to_user_bin_id);
    CHECK(!(other == hibf));
    h::hierarchical_interleaved_bloom_filter moved{std::move(other)};
    CHECK(moved.next_ibf_id == hibf.next_ibf_id && moved.number_of_user_bins == 3);
}

// The batched calls (no counterpart in the reference) give, per query, what the one-query agents give.
static void hibf_batch(std::string const & dir)
{
    std::vector<std::vector<uint64_t>> hashes{{1, 2, 3, 4, 5, 6, 7, 8, 9, 10}, {1, 2, 3, 4, 5}, {3, 9, 11}};
    h::config config{.input_fn =
                         [&](size_t const num, h::insert_iterator && it)
                     {
                         for (auto const hash : hashes[num])
                             it = hash;
                     },
                     .number_of_user_bins = 3};
    h::hierarchical_interleaved_bloom_filter hibf{config, read_file(dir + "/layout_readme.txt")};
    std::vector<std::vector<uint64_t>> queries{{3, 9, 12, 14}, iota(15), {}, {1, 2, 3}, {11, 11, 9}};
    std::vector<uint16_t> thr{2, 5, 1, 3, 2};
    std::vector<uint64_t> values, offsets{0};
    for (auto const & q : queries)
    {
        values.insert(values.end(), q.begin(), q.end());
        offsets.push_back(values.size());
    }
    auto agent = hibf.membership_agent();
    auto single = hibf.membership_agent();
    auto const & b = agent.membership_for_batch(values, offsets, thr);
    CHECK(b.offsets.size() == queries.size() + 1);
    for (size_t q = 0; q < queries.size(); ++q)
    {
        auto & r = single.membership_for(queries[q], thr[q]);
        single.sort_results();
        CHECK(std::vector<uint64_t>(b.ids.begin() + b.offsets[q], b.ids.begin() + b.offsets[q + 1]) == r);
    }
    auto counter = hibf.counting_agent<uint16_t>();
    auto one = hibf.counting_agent<uint16_t>();
    std::vector<uint64_t> const cthr{1, 5, 1, 2, 1};
    auto const & c = counter.bulk_count_batch(values, offsets, cthr);
    for (size_t q = 0; q < queries.size(); ++q)
    {
        std::vector<uint16_t> dense(hibf.number_of_user_bins, 0);
        for (uint64_t i = c.offsets[q]; i < c.offsets[q + 1]; ++i)
            dense[c.ids[i]] = c.counts[i];
        CHECK(dense == one.bulk_count(queries[q], cthr[q]));
    }
    bool const rejected = throws<std::function<void()>, std::invalid_argument>(
        [&] { agent.membership_for_batch(values, std::vector<uint64_t>{0}, thr); });
    CHECK(rejected);
}

int main(int argc, char ** argv)
{
    if (argc < 2)
    {
        std::fprintf(stderr, "usage: test_facade <dir with layout_snippet.txt and layout_readme.txt>\n");
        return 2;
    }
    std::string const dir = argv[1];
    ibf_construction();
    ibf_contains();
    ibf_counting();
    ibf_clear();
    ibf_membership();
    ibf_increase();
    ibf_from_config();
    ibf_occupancy();
    hibf_small(dir);
    hibf_readme(dir);
    hibf_batch(dir);
    if (failures)
    {
        std::fprintf(stderr, "%d check(s) failed\n", failures);
        return 1;
    }
    std::printf("all facade checks passed\n");
    return 0;
}
