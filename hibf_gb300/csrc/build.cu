// build.cu -- host orchestration of an HIBF build from a layout, with every insert done on the device.
//
// Restates the reference's build driver (src/hierarchical_interleaved_bloom_filter.cpp:40-209; src/build/*.cpp;
// include/hibf/build/*.hpp) on top of the device bit stores:
//   layout text  -> layout records            (src/layout/layout.cpp:60-145)
//   records      -> IBF graph                 (src/layout/graph.cpp:19-125)
//   graph        -> per-IBF sizes and tables  (construct_ibf.cpp:26-64, bin_size_in_bits.hpp:35-45,
//                                              compute_fpr_correction.cpp:16-38, update_user_bins.hpp:19-25)
//   contents     -> device inserts            (insert_into_ibf.cpp:28-84; merged bins receive the union of their
//                                              subtree, i.e. every user bin below them)
// IBFs are numbered in depth-first pre-order with children in layout order (the reference numbers them in a
// randomised order, HIBF.cpp:111-116; numbering does not change any bit or query result).
//
// Split user bins: the input_fn build chunks them in the reference's order (the iteration order of its hash set,
// robin_hood::unordered_flat_set, insert_into_ibf.cpp:34-47, replayed by reference_split_orders), so its bit store
// equals the reference's.  The synthetic build (values generated on the device, no host sets) chunks in stream
// order: which of the split bins a value lands in differs; sizes, tables and every unsplit user bin's bins do not.

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <exception>
#include <functional>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_set>
#include <vector>

#include "../../include/hibf_gb300_synthetic.h"
#include "common.hpp"
#include "device.cuh"
#include "hibf_internal.cuh"
#include "rh_set.hpp"

// A split table (hibf_gpu_split_table_*): flattened split_entry records, one per split user bin, ascending.
struct hibf_gpu_split_table
{
    std::vector<uint64_t> user_bin, n, mult, mask, bnd_off{0}, home, before_off{0}, before;
};

namespace hibf_gb300
{
namespace build
{

struct user_bin_rec
{
    std::vector<uint64_t> prev;
    uint64_t storage{};
    uint64_t ntb{};
    uint64_t idx{};
};

struct max_bin_rec
{
    std::vector<uint64_t> prev;
    uint64_t id{};
};

struct layout_t
{
    uint64_t top_max{};
    std::vector<max_bin_rec> max_bins;
    std::vector<user_bin_rec> user_bins;
};

static std::vector<uint64_t> parse_list(std::string const & s, char sep)
{
    std::vector<uint64_t> out;
    size_t i = 0;
    while (i < s.size())
    {
        size_t j = s.find(sep, i);
        if (j == std::string::npos)
            j = s.size();
        if (j > i)
            out.push_back(std::stoull(s.substr(i, j - i)));
        i = j + 1;
    }
    return out;
}

// The layout file format of src/layout/layout.cpp:60-145 (an optional @HIBF_CONFIG block is skipped).
layout_t parse_layout(char const * text)
{
    layout_t L;
    std::string const t(text ? text : "");
    size_t pos = 0;
    auto next_line = [&](std::string & line) -> bool
    {
        if (pos >= t.size())
            return false;
        size_t e = t.find('\n', pos);
        if (e == std::string::npos)
            e = t.size();
        line = t.substr(pos, e - pos);
        if (!line.empty() && line.back() == '\r')
            line.pop_back();
        pos = e + 1;
        return true;
    };
    std::string line;
    std::string const key = "fullest_technical_bin_idx:";
    bool have_top = false;
    while (next_line(line))
    {
        if (line.empty() || line[0] == '@')
            continue;
        if (line.rfind("#TOP_LEVEL_IBF", 0) == 0)
        {
            size_t const k = line.find(key);
            if (k == std::string::npos)
                fail(HIBF_GPU_ERR_INVALID_ARG, "layout: malformed top-level header");
            L.top_max = std::stoull(line.substr(k + key.size()));
            have_top = true;
            continue;
        }
        if (line.rfind("#LOWER_LEVEL_IBF_", 0) == 0)
        {
            size_t const sp = line.find(' ');
            size_t const k = line.find(key);
            if (sp == std::string::npos || k == std::string::npos)
                fail(HIBF_GPU_ERR_INVALID_ARG, "layout: malformed lower-level header");
            max_bin_rec m;
            m.prev = parse_list(line.substr(17, sp - 17), ';');
            m.id = std::stoull(line.substr(k + key.size()));
            if (m.prev.empty())
                fail(HIBF_GPU_ERR_INVALID_ARG, "layout: lower-level header without bin indices");
            L.max_bins.push_back(std::move(m));
            continue;
        }
        if (line[0] == '#')
            continue; // column names
        size_t const t1 = line.find('\t');
        size_t const t2 = line.find('\t', t1 + 1);
        if (t1 == std::string::npos || t2 == std::string::npos)
            fail(HIBF_GPU_ERR_INVALID_ARG, "layout: malformed user bin line");
        user_bin_rec r;
        r.idx = std::stoull(line.substr(0, t1));
        std::vector<uint64_t> bins = parse_list(line.substr(t1 + 1, t2 - t1 - 1), ';');
        std::vector<uint64_t> ntb = parse_list(line.substr(t2 + 1), ';');
        if (bins.empty() || ntb.empty())
            fail(HIBF_GPU_ERR_INVALID_ARG, "layout: malformed user bin line");
        r.storage = bins.back();
        bins.pop_back();
        r.prev = std::move(bins);
        r.ntb = ntb.back();
        L.user_bins.push_back(std::move(r));
    }
    if (!have_top)
        fail(HIBF_GPU_ERR_INVALID_ARG, "layout: missing #TOP_LEVEL_IBF header");
    return L;
}

struct node_t
{
    std::vector<size_t> children;
    size_t parent{SIZE_MAX};
    uint64_t parent_bin_index{};
    uint64_t max_bin_index{};
    uint64_t ntb{};
    int64_t favourite{-1};
    std::vector<user_bin_rec> records;
};

// graph::graph (src/layout/graph.cpp:19-125).
std::vector<node_t> make_graph(layout_t const & L)
{
    std::vector<node_t> g(1);
    g[0].max_bin_index = L.top_max;
    for (auto const & mb : L.max_bins)
    {
        size_t parent = 0;
        for (size_t i = 0; i + 1 < mb.prev.size(); ++i)
        {
            for (size_t c : g[parent].children)
                if (g[c].parent_bin_index == mb.prev[i])
                {
                    parent = c;
                    break;
                }
        }
        node_t n;
        n.parent = parent;
        n.parent_bin_index = mb.prev.back();
        n.max_bin_index = mb.id;
        g.push_back(std::move(n));
        size_t const id = g.size() - 1;
        g[parent].children.push_back(id);
        if (g[parent].max_bin_index == mb.prev.back())
            g[parent].favourite = static_cast<int64_t>(g[parent].children.size() - 1);
    }
    for (auto const & r : L.user_bins)
    {
        size_t cur = 0;
        for (uint64_t bin : r.prev)
        {
            g[cur].ntb = std::max(g[cur].ntb, bin + 1);
            size_t nxt = SIZE_MAX;
            for (size_t c : g[cur].children)
                if (g[c].parent_bin_index == bin)
                {
                    nxt = c;
                    break;
                }
            if (nxt == SIZE_MAX)
                fail(HIBF_GPU_ERR_INVALID_ARG, "layout: user bin refers to a lower-level IBF without a header");
            cur = nxt;
        }
        g[cur].ntb = std::max(g[cur].ntb, r.storage + r.ntb);
        if (r.storage == g[cur].max_bin_index)
            g[cur].records.insert(g[cur].records.begin(), r);
        else
            g[cur].records.push_back(r);
    }
    return g;
}

// bin_size_in_bits (include/hibf/build/bin_size_in_bits.hpp:35-45).
uint64_t bin_size_in_bits(double fpr, uint64_t hash_count, uint64_t elements)
{
    double const numerator = -static_cast<double>(elements * hash_count);
    double const denominator = std::log(1 - std::exp(std::log(fpr) / static_cast<double>(hash_count)));
    return static_cast<uint64_t>(std::ceil(numerator / denominator));
}

// compute_fpr_correction (src/layout/compute_fpr_correction.cpp:16-38).
std::vector<double> fpr_correction(double fpr, uint64_t hash_count, uint64_t t_max)
{
    uint64_t const max_tb = ((t_max + 63) >> 6) << 6;
    std::vector<double> c(max_tb + 1, 0.0);
    c[1] = 1.0;
    double const h = static_cast<double>(hash_count);
    double const numerator = std::log1p(-std::exp(std::log(fpr) / h));
    for (uint64_t split = 2; split <= max_tb; ++split)
    {
        double const log_target_fpr = std::log1p(-std::exp(std::log1p(-fpr) / static_cast<double>(split)));
        c[split] = numerator / std::log1p(-std::exp(log_target_fpr / h));
    }
    return c;
}

struct plan_t
{
    std::vector<node_t> g;
    std::vector<size_t> order;  // IBF index -> graph node
    std::vector<size_t> ibf_of; // graph node -> IBF index
    std::vector<uint64_t> bins, bin_size, hash_funs, next_ibf, user_bin, tb_off;
    std::vector<uint64_t> parent_ibf, parent_bin;
    // per user bin: leaf IBF, leaf record, and the (IBF, merged bin) pairs of its ancestors
    std::vector<size_t> ub_leaf;
    std::vector<user_bin_rec> ub_rec;
    std::vector<std::vector<std::pair<uint64_t, uint64_t>>> ub_merged;
};

// Sizes every IBF like construct_ibf (src/build/construct_ibf.cpp:26-64): the max bin's content is the favourite
// child's union (merged max bin, relaxed fpr, one bin) or the max record's distinct values split over its
// technical bins (maximum fpr, times the fpr correction for split bins).  `distinct[u]` = distinct values of user
// bin u; `subtree_union(node)` = distinct values under a node.
template <typename union_fn>
plan_t make_plan(hibf_gpu_build_config const & cfg, layout_t const & L, std::vector<uint64_t> const & distinct,
                 union_fn && subtree_union)
{
    plan_t P;
    P.g = make_graph(L);
    auto & g = P.g;
    // pre-order numbering
    std::vector<size_t> st{0};
    P.ibf_of.assign(g.size(), SIZE_MAX);
    while (!st.empty())
    {
        size_t const n = st.back();
        st.pop_back();
        P.ibf_of[n] = P.order.size();
        P.order.push_back(n);
        for (auto it = g[n].children.rbegin(); it != g[n].children.rend(); ++it)
            st.push_back(*it);
    }
    size_t const n_ibfs = P.order.size();
    uint64_t const h = cfg.number_of_hash_functions;
    std::vector<double> const corr = fpr_correction(cfg.maximum_fpr, h, g[0].ntb);
    P.tb_off.assign(n_ibfs + 1, 0);
    P.parent_ibf.assign(n_ibfs, 0);
    P.parent_bin.assign(n_ibfs, 0);
    for (size_t k = 0; k < n_ibfs; ++k)
    {
        node_t const & nd = g[P.order[k]];
        if (nd.ntb == 0)
            fail(HIBF_GPU_ERR_INVALID_ARG, "layout: an IBF has no technical bins");
        uint64_t kmers = 0, nb = 1;
        double fpr = cfg.maximum_fpr;
        if (nd.favourite >= 0)
        {
            kmers = subtree_union(nd.children[static_cast<size_t>(nd.favourite)]);
            nb = 1;
            fpr = cfg.relaxed_fpr;
        }
        else
        {
            if (nd.records.empty())
                fail(HIBF_GPU_ERR_INVALID_ARG, "layout: an IBF has neither a merged nor a user max bin");
            user_bin_rec const & r = nd.records[0];
            if (r.idx >= distinct.size())
                fail(HIBF_GPU_ERR_INVALID_ARG, "layout: user bin index out of range");
            kmers = distinct[r.idx];
            nb = r.ntb;
        }
        uint64_t const per_bin = (kmers + nb - 1) / nb;
        uint64_t const bits = bin_size_in_bits(fpr, h, per_bin);
        uint64_t const size = nb == 1 ? bits : static_cast<uint64_t>(std::ceil(static_cast<double>(bits) * corr.at(nb)));
        if (size == 0)
            fail(HIBF_GPU_ERR_LOGIC, "The size of a bin must be > 0.");
        P.bins.push_back(nd.ntb);
        P.bin_size.push_back(size);
        P.hash_funs.push_back(h);
        P.tb_off[k + 1] = P.tb_off[k] + nd.ntb;
        if (nd.parent != SIZE_MAX)
        {
            P.parent_ibf[k] = P.ibf_of[nd.parent];
            P.parent_bin[k] = nd.parent_bin_index;
        }
    }
    // tables (HIBF.cpp:47-55, update_user_bins.hpp:19-25)
    P.next_ibf.assign(P.tb_off[n_ibfs], 0);
    P.user_bin.assign(P.tb_off[n_ibfs], HIBF_GPU_BIN_MERGED);
    for (size_t k = 0; k < n_ibfs; ++k)
    {
        node_t const & nd = g[P.order[k]];
        for (uint64_t b = 0; b < nd.ntb; ++b)
            P.next_ibf[P.tb_off[k] + b] = k;
        for (size_t c : nd.children)
            P.next_ibf[P.tb_off[k] + g[c].parent_bin_index] = P.ibf_of[c];
        for (auto const & r : nd.records)
            for (uint64_t b = r.storage; b < r.storage + r.ntb; ++b)
                P.user_bin[P.tb_off[k] + b] = r.idx;
    }
    // per user bin placement
    size_t const nub = cfg.number_of_user_bins;
    P.ub_leaf.assign(nub, SIZE_MAX);
    P.ub_rec.assign(nub, user_bin_rec{});
    P.ub_merged.assign(nub, {});
    for (size_t k = 0; k < n_ibfs; ++k)
    {
        size_t const n = P.order[k];
        for (auto const & r : g[n].records)
        {
            if (r.idx >= nub)
                fail(HIBF_GPU_ERR_INVALID_ARG, "layout: user bin index out of range");
            if (P.ub_leaf[r.idx] != SIZE_MAX)
                fail(HIBF_GPU_ERR_INVALID_ARG, "layout: a user bin occurs twice");
            P.ub_leaf[r.idx] = k;
            P.ub_rec[r.idx] = r;
            size_t cur = n;
            while (g[cur].parent != SIZE_MAX)
            {
                P.ub_merged[r.idx].push_back({P.ibf_of[g[cur].parent], g[cur].parent_bin_index});
                cur = g[cur].parent;
            }
        }
    }
    for (size_t u = 0; u < nub; ++u)
        if (P.ub_leaf[u] == SIZE_MAX)
            fail(HIBF_GPU_ERR_INVALID_ARG, "layout: a user bin is missing");
    return P;
}

// Replays the history of the reference's build sets (hierarchical_build, src/hierarchical_interleaved_bloom_filter.cpp:
// 39-171) on rh_set and calls on_split(user bin, technical bins, set) right after the set took a user bin that the
// reference splits over several technical bins: the reference chunks it in that set's iteration order
// (src/build/insert_into_ibf.cpp:34-47).  The reference keeps one set per IBF for the max bin and the records
// (cleared, not shrunk, between records), fills it through the favourite child when the max bin is merged, and adds
// every non-root set to its parent's; the root's other children run in a shuffled order but with sets of their own.
// `source(u, f)` calls f(v) for user bin u's values in input order.
//
// Only what can be observed is replayed: a set's fills are skipped when no later fill of it takes a split user bin
// and its contents do not flow into a set that is observed, and every subtree whose contents go nowhere (a child of
// the root other than the favourite, or any child of such a node that does not feed its parent) runs as a job of its
// own on the host threads.
template <typename Source, typename OnSplit>
void replay_split_history(plan_t const & P, Source const & source, OnSplit const & on_split, unsigned threads)
{
    std::mutex lock;
    std::condition_variable wake;
    std::vector<std::pair<size_t, bool>> queue{{0, true}};
    size_t outstanding = 1;
    std::exception_ptr error;

    auto spawn = [&](size_t n)
    {
        std::lock_guard<std::mutex> g(lock);
        queue.emplace_back(n, false);
        ++outstanding;
        wake.notify_one();
    };
    auto take = [&](rh_set & k, user_bin_rec const & r)
    {
        source(r.idx, [&](uint64_t v) { k.insert(v); });
        if (r.ntb > 1)
            on_split(r.idx, r.ntb, k);
    };
    auto add = [](rh_set const & from, rh_set & to) { from.for_each([&](uint64_t v) { to.insert(v); }); };

    std::function<void(size_t, rh_set *, bool)> run = [&](size_t n, rh_set * parent, bool is_root)
    {
        node_t const & nd = P.g[n];
        bool const max_merged = nd.favourite >= 0;
        bool const up = parent != nullptr && !is_root; // every fill of this node's set flows into `parent`
        size_t const start = max_merged ? 0 : 1;
        // fill 0 is the max bin (favourite subtree or records[0]); fill f >= 1 the f-th record taken afterwards
        int64_t last_split = (!max_merged && !nd.records.empty() && nd.records[0].ntb > 1) ? 0 : -1;
        {
            int64_t f = 1;
            for (size_t i = start; i < nd.records.size(); ++i)
            {
                if (is_root && nd.records[i].ntb == 1)
                    continue; // inserted straight from input_fn, no set
                if (nd.records[i].ntb > 1)
                    last_split = f;
                ++f;
            }
        }
        auto need = [&](int64_t f) { return up || f <= last_split; };
        rh_set kmers;
        if (max_merged)
        {
            size_t const fav = nd.children[static_cast<size_t>(nd.favourite)];
            if (need(0))
                run(fav, &kmers, false);
            else
                spawn(fav);
        }
        else if (!nd.records.empty() && need(0))
        {
            take(kmers, nd.records[0]);
        }
        if (up)
            add(kmers, *parent); // construct_ibf
        kmers.clear();
        for (size_t i = 0; i < nd.children.size(); ++i)
        {
            if (max_merged && static_cast<int64_t>(i) == nd.favourite)
                continue;
            if (up)
            {
                rh_set local;
                run(nd.children[i], &local, false);
                add(local, *parent);
            }
            else
            {
                spawn(nd.children[i]);
            }
        }
        int64_t f = 1;
        for (size_t i = start; i < nd.records.size(); ++i)
        {
            user_bin_rec const & r = nd.records[i];
            if (is_root && r.ntb == 1)
                continue;
            if (need(f))
            {
                take(kmers, r);
                if (up)
                    add(kmers, *parent);
                kmers.clear();
            }
            ++f;
        }
    };

    auto worker = [&]
    {
        while (true)
        {
            std::pair<size_t, bool> job;
            {
                std::unique_lock<std::mutex> g(lock);
                wake.wait(g, [&] { return !queue.empty() || outstanding == 0; });
                if (queue.empty())
                    return;
                job = queue.back();
                queue.pop_back();
            }
            try
            {
                run(job.first, nullptr, job.second);
            }
            catch (...)
            {
                std::lock_guard<std::mutex> g(lock);
                if (!error)
                    error = std::current_exception();
            }
            std::lock_guard<std::mutex> g(lock);
            if (--outstanding == 0)
                wake.notify_all();
        }
    };
    unsigned const nt = std::max(1u, threads ? threads : std::thread::hardware_concurrency());
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < nt; ++t)
        pool.emplace_back(worker);
    worker();
    for (std::thread & t : pool)
        t.join();
    if (error)
        std::rethrow_exception(error);
}

// The order in which the reference chunks every split user bin (the set's iteration order at that moment).
// `sets[u]` = user bin u's distinct values in input order.
std::vector<std::vector<uint64_t>> reference_split_orders(plan_t const & P,
                                                          std::vector<std::vector<uint64_t>> const & sets)
{
    std::vector<std::vector<uint64_t>> out(sets.size());
    replay_split_history(
        P, [&](uint64_t u, auto && f) { for (uint64_t v : sets[u]) f(v); },
        [&](uint64_t u, uint64_t, rh_set const & k) { out[u] = k.ordered(); }, 0);
    return out;
}

// A split user bin's chunking without its order.  The set's iteration order visits keys in non-decreasing home slot
// (rh_home with the set's multiplier and mask), so a key's rank is the number of keys in lower home slots plus its
// place among the keys of its own slot.  Chunk boundary b (rank b * ceil(n / tbs)) is therefore fixed by the home
// slot of the key at that rank and the keys of that slot ranked before it; a key's chunk is the number of
// boundaries it lies at or after.
struct split_entry
{
    uint64_t n{};    // distinct values of the user bin
    uint64_t mult{}; // the set's hash multiplier when it was chunked
    uint64_t mask{}; // the set's slot mask then
    std::vector<uint64_t> home;                // per boundary: home slot of the key at the boundary's rank
    std::vector<std::vector<uint64_t>> before; // per boundary: keys of that home slot ranked before it
};

split_entry split_entry_of(rh_set const & k, uint64_t tbs)
{
    split_entry e;
    e.n = k.size();
    e.mult = k.multiplier();
    e.mask = k.slot_mask();
    uint64_t const chunk = (e.n + tbs - 1) / tbs;
    uint64_t next = 1, rank = 0, cur = UINT64_MAX, prev = 0;
    bool sorted = true;
    std::vector<uint64_t> group;
    k.for_each(
        [&](uint64_t v)
        {
            uint64_t const h = rh_home(v, e.mult, e.mask);
            if (rank > 0 && h < prev)
                sorted = false;
            if (h != cur)
            {
                group.clear();
                cur = h;
            }
            if (next < tbs && next * chunk == rank)
            {
                e.home.push_back(h);
                e.before.push_back(group);
                ++next;
            }
            group.push_back(v);
            prev = h;
            ++rank;
        });
    if (!sorted)
        fail(HIBF_GPU_ERR_LOGIC, "hash set iteration is not in home slot order");
    return e;
}

// The chunk of value v of a split user bin (host form of the device's lookup).
uint64_t split_chunk(uint64_t v, uint64_t mult, uint64_t mask, uint64_t const * home, uint64_t n_bnd,
                     uint64_t const * before_off, uint64_t const * before)
{
    uint64_t const h = rh_home(v, mult, mask);
    uint64_t c = 0;
    while (c < n_bnd && home[c] < h)
        ++c;
    for (; c < n_bnd && home[c] == h; ++c)
    {
        bool in = false;
        for (uint64_t j = before_off[c]; j < before_off[c + 1]; ++j)
            in = in || before[j] == v;
        if (in)
            break;
    }
    return c;
}

// The split table of plan P: the replay with `source` giving every user bin's values in input order.
template <typename Source>
void compute_split_table(plan_t const & P, Source const & source, unsigned threads, hibf_gpu_split_table & t)
{
    size_t const nub = P.ub_rec.size();
    std::vector<split_entry> ent(nub);
    replay_split_history(P, source, [&](uint64_t u, uint64_t tbs, rh_set const & k) { ent[u] = split_entry_of(k, tbs); },
                         threads);
    t = hibf_gpu_split_table{};
    for (size_t u = 0; u < nub; ++u)
    {
        if (P.ub_rec[u].ntb <= 1)
            continue;
        split_entry const & e = ent[u];
        t.user_bin.push_back(u);
        t.n.push_back(e.n);
        t.mult.push_back(e.mult);
        t.mask.push_back(e.mask);
        for (size_t b = 0; b < e.home.size(); ++b)
        {
            t.home.push_back(e.home[b]);
            t.before.insert(t.before.end(), e.before[b].begin(), e.before[b].end());
            t.before_off.push_back(t.before.size());
        }
        t.bnd_off.push_back(t.home.size());
    }
}

// Checks that table t belongs to plan P with user bins of `distinct` values; returns per user bin 1 + its entry
// (0: not split).
std::vector<uint64_t> check_split_table(plan_t const & P, hibf_gpu_split_table const & t,
                                        std::vector<uint64_t> const & distinct)
{
    size_t const nub = P.ub_rec.size();
    size_t const ns = t.user_bin.size();
    auto bad = [](char const * what) { fail(HIBF_GPU_ERR_INVALID_ARG, std::string("split table: ") + what); };
    if (t.n.size() != ns || t.mult.size() != ns || t.mask.size() != ns || t.bnd_off.size() != ns + 1 ||
        t.bnd_off.back() != t.home.size() || t.before_off.size() != t.home.size() + 1 ||
        t.before_off.back() != t.before.size())
        bad("inconsistent array sizes");
    std::vector<uint64_t> entry(nub, 0);
    for (size_t i = 0; i < ns; ++i)
    {
        uint64_t const u = t.user_bin[i];
        if (u >= nub || P.ub_rec[u].ntb <= 1 || entry[u] != 0)
            bad("it lists a user bin the layout does not split, or one twice");
        entry[u] = i + 1;
        uint64_t const tbs = P.ub_rec[u].ntb;
        if (t.n[i] != distinct[u])
            bad("a user bin's size differs from the input's");
        uint64_t const chunk = (t.n[i] + tbs - 1) / tbs;
        uint64_t want = 0;
        for (uint64_t b = 1; b < tbs && b * chunk < t.n[i]; ++b)
            ++want;
        if (t.bnd_off[i + 1] < t.bnd_off[i] || t.bnd_off[i + 1] - t.bnd_off[i] != want)
            bad("a user bin has the wrong number of chunk boundaries");
        for (uint64_t b = t.bnd_off[i]; b < t.bnd_off[i + 1]; ++b)
            if (t.home[b] > t.mask[i] || (b > t.bnd_off[i] && t.home[b] < t.home[b - 1]) ||
                t.before_off[b + 1] < t.before_off[b])
                bad("boundaries out of order");
    }
    for (size_t u = 0; u < nub; ++u)
        if (P.ub_rec[u].ntb > 1 && entry[u] == 0)
            bad("a split user bin of the layout is missing");
    return entry;
}

// Distinct values under each node when user bins are pairwise disjoint: sums of their sizes.
std::vector<uint64_t> disjoint_unions(plan_t const & P, std::vector<uint64_t> const & distinct, layout_t const & L)
{
    (void)L;
    std::vector<uint64_t> sum(P.g.size(), 0);
    // accumulate user bins into their leaf node and every ancestor
    for (size_t u = 0; u < P.ub_leaf.size(); ++u)
    {
        size_t n = P.order[P.ub_leaf[u]];
        while (true)
        {
            sum[n] += distinct[u];
            if (P.g[n].parent == SIZE_MAX)
                break;
            n = P.g[n].parent;
        }
    }
    return sum;
}

// ---- device inserts -------------------------------------------------------------------------------------------
struct alignas(16) insert_job
{
    uint64_t start; // first value (stream position for synthetic jobs, buffer offset otherwise)
    uint64_t n;     // number of values
    uint64_t split; // split user bins: 1 + their entry in the split table; 0: all values into first_bin
    uint32_t ibf;
    uint32_t first_bin;
};

// Device form of a split table: per split user bin its set's multiplier and mask and its boundaries; per boundary
// the home slot and the keys of that slot ranked before it (split_entry).
struct alignas(16) dev_split
{
    uint64_t mult;
    uint64_t mask;
    uint32_t bnd_first;
    uint32_t bnd_count;
    uint32_t pad[2];
};

struct alignas(16) dev_bnd
{
    uint64_t home;
    uint32_t before_first;
    uint32_t before_count;
};

// The technical bin offset of value v of a split user bin: the number of chunk boundaries it lies at or after.
__device__ __forceinline__ uint32_t split_chunk_d(uint64_t v, dev_split const & sp, dev_bnd const * __restrict__ bnds,
                                                  uint64_t const * __restrict__ before)
{
    uint64_t const h = rh_home(v, sp.mult, sp.mask);
    uint32_t lo = 0, hi = sp.bnd_count;
    while (lo < hi)
    {
        uint32_t const mid = (lo + hi) >> 1;
        if (bnds[sp.bnd_first + mid].home < h)
            lo = mid + 1;
        else
            hi = mid;
    }
    uint32_t c = lo;
    for (; c < sp.bnd_count; ++c)
    {
        dev_bnd const bd = bnds[sp.bnd_first + c];
        if (bd.home != h)
            break;
        bool in = false;
        for (uint32_t j = 0; j < bd.before_count; ++j)
            in = in || before[bd.before_first + j] == v;
        if (in)
            break;
    }
    return c;
}

// Inserts every job's values; job j covers flattened positions [end[j] - n_j, end[j]).  Values come from the
// splitmix64 stream (values == nullptr) or from a device buffer.
__global__ void k_insert_jobs(dev_node const * __restrict__ nodes, insert_job const * __restrict__ jobs,
                              uint64_t const * __restrict__ job_end, uint32_t n_jobs, uint64_t total,
                              uint64_t seed, uint64_t const * __restrict__ values,
                              dev_split const * __restrict__ splits, dev_bnd const * __restrict__ bnds,
                              uint64_t const * __restrict__ before)
{
    uint64_t const stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
    uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
    if (i >= total)
        return;
    // first job with end > i
    uint32_t lo = 0, hi = n_jobs;
    while (lo < hi)
    {
        uint32_t const mid = (lo + hi) >> 1;
        if (job_end[mid] > i)
            hi = mid;
        else
            lo = mid + 1;
    }
    uint32_t j = lo;
    for (; i < total; i += stride)
    {
        while (job_end[j] <= i)
            ++j;
        insert_job const jb = jobs[j];
        uint64_t const local = i - (job_end[j] - jb.n);
        uint64_t const v = values ? values[jb.start + local] : hg_stream_at(seed, jb.start + local);
        uint64_t const b = jb.first_bin + (jb.split ? split_chunk_d(v, splits[jb.split - 1], bnds, before) : 0u);
        dev_node const nd = nodes[jb.ibf];
        if (b >= nd.bins)
            continue;
        unsigned long long const bit = 1ull << (b & 63u);
        uint64_t * const base = const_cast<uint64_t *>(nd.words) + (b >> 6);
        for (uint32_t k = 0; k < nd.hash_funs; ++k)
        {
            uint64_t const r = hash_row(v, c_hash_seeds[k], nd.hash_shift, nd.bin_size);
            atomicOr(reinterpret_cast<unsigned long long *>(base + r * nd.row_words), bit);
        }
    }
}

// The split table on the device (uploaded once per build).
struct dev_split_table
{
    dbuf splits, bnds, before;
};

void upload_split_table(hibf_gpu_split_table const & t, dev_split_table & dt, cudaStream_t s)
{
    size_t const ns = t.user_bin.size();
    if (t.home.size() > UINT32_MAX || t.before.size() > UINT32_MAX)
        fail(HIBF_GPU_ERR_INVALID_ARG, "split table too large");
    std::vector<dev_split> sp(ns);
    for (size_t i = 0; i < ns; ++i)
        sp[i] = dev_split{t.mult[i], t.mask[i], static_cast<uint32_t>(t.bnd_off[i]),
                          static_cast<uint32_t>(t.bnd_off[i + 1] - t.bnd_off[i]), {0, 0}};
    std::vector<dev_bnd> bd(t.home.size());
    for (size_t b = 0; b < bd.size(); ++b)
        bd[b] = dev_bnd{t.home[b], static_cast<uint32_t>(t.before_off[b]),
                        static_cast<uint32_t>(t.before_off[b + 1] - t.before_off[b])};
    dt.splits.ensure(sp.size() * sizeof(dev_split));
    dt.bnds.ensure(bd.size() * sizeof(dev_bnd));
    dt.before.ensure(t.before.size() * 8);
    if (!sp.empty())
        HG_CUDA(cudaMemcpyAsync(dt.splits.p, sp.data(), sp.size() * sizeof(dev_split), cudaMemcpyHostToDevice, s));
    if (!bd.empty())
        HG_CUDA(cudaMemcpyAsync(dt.bnds.p, bd.data(), bd.size() * sizeof(dev_bnd), cudaMemcpyHostToDevice, s));
    if (!t.before.empty())
        HG_CUDA(cudaMemcpyAsync(dt.before.p, t.before.data(), t.before.size() * 8, cudaMemcpyHostToDevice, s));
    HG_CUDA(cudaStreamSynchronize(s)); // the host vectors may go away
}

void run_jobs(hibf_gpu_hibf * h, std::vector<insert_job> const & jobs, uint64_t seed, uint64_t const * d_values,
              dev_split_table const * dt, cudaStream_t s)
{
    if (jobs.empty())
        return;
    std::vector<uint64_t> end(jobs.size());
    uint64_t acc = 0;
    for (size_t j = 0; j < jobs.size(); ++j)
    {
        acc += jobs[j].n;
        end[j] = acc;
    }
    if (acc == 0)
        return;
    dbuf dj, de;
    dj.ensure(jobs.size() * sizeof(insert_job));
    de.ensure(end.size() * 8);
    HG_CUDA(cudaMemcpyAsync(dj.p, jobs.data(), jobs.size() * sizeof(insert_job), cudaMemcpyHostToDevice, s));
    HG_CUDA(cudaMemcpyAsync(de.p, end.data(), end.size() * 8, cudaMemcpyHostToDevice, s));
    unsigned const block = 256;
    uint64_t const want = (acc + block - 1) / block;
    unsigned const grid = static_cast<unsigned>(std::min<uint64_t>(want, static_cast<uint64_t>(sm_count()) * 16));
    k_insert_jobs<<<grid, block, 0, s>>>(h->d_nodes.as<dev_node>(), dj.as<insert_job>(), de.as<uint64_t>(),
                                         static_cast<uint32_t>(jobs.size()), acc, seed, d_values,
                                         dt ? dt->splits.as<dev_split>() : nullptr,
                                         dt ? dt->bnds.as<dev_bnd>() : nullptr,
                                         dt ? dt->before.as<uint64_t>() : nullptr);
    HG_CUDA(cudaGetLastError());
    HG_CUDA(cudaStreamSynchronize(s));
}

hibf_gpu_hibf * create_from_plan(plan_t const & P, uint64_t n_user_bins)
{
    hibf_gpu_hibf * h = nullptr;
    int st = hibf_gpu_hibf_create(n_user_bins, P.bins.size(), P.bins.data(), P.bin_size.data(), P.hash_funs.data(),
                                  P.next_ibf.data(), P.user_bin.data(), &h);
    if (st != HIBF_GPU_OK)
        fail(st, "hibf_gpu_hibf_create failed");
    // prev_ibf_id as the reference's build leaves it (src/hierarchical_interleaved_bloom_filter.cpp:130): set for
    // the children it builds in its loop over merged bins, (0, 0) for the root and for favourite children
    std::vector<uint64_t> pi(P.bins.size(), 0), pb(P.bins.size(), 0);
    for (size_t k = 0; k < P.order.size(); ++k)
    {
        size_t const n = P.order[k];
        size_t const parent = P.g[n].parent;
        if (parent == SIZE_MAX)
            continue;
        node_t const & pn = P.g[parent];
        if (pn.favourite >= 0 && pn.children[static_cast<size_t>(pn.favourite)] == n)
            continue;
        pi[k] = P.ibf_of[parent];
        pb[k] = P.g[n].parent_bin_index;
    }
    st = hibf_gpu_hibf_set_prev(h, pi.data(), pb.data());
    if (st != HIBF_GPU_OK)
    {
        hibf_gpu_hibf_destroy(h);
        fail(st, "prev_ibf_id");
    }
    return h;
}

void validate(hibf_gpu_build_config const * cfg)
{
    if (!cfg)
        fail(HIBF_GPU_ERR_INVALID_ARG, "null config");
    // config::validate_and_set_defaults (src/config.cpp:64-130), the fields the builder reads
    if (cfg->number_of_user_bins == 0)
        fail(HIBF_GPU_ERR_INVALID_ARG, "[HIBF CONFIG ERROR] You did not set the required config::number_of_user_bins.");
    if (cfg->number_of_hash_functions == 0 || cfg->number_of_hash_functions > 5)
        fail(HIBF_GPU_ERR_INVALID_ARG, "[HIBF CONFIG ERROR] config::number_of_hash_functions must be in [1,5].");
    if (!(cfg->maximum_fpr > 0.0 && cfg->maximum_fpr < 1.0))
        fail(HIBF_GPU_ERR_INVALID_ARG, "[HIBF CONFIG ERROR] config::maximum_fpr must be in (0.0,1.0).");
    if (!(cfg->relaxed_fpr > 0.0 && cfg->relaxed_fpr < 1.0))
        fail(HIBF_GPU_ERR_INVALID_ARG, "[HIBF CONFIG ERROR] config::relaxed_fpr must be in (0.0,1.0).");
    if (cfg->relaxed_fpr < cfg->maximum_fpr)
        fail(HIBF_GPU_ERR_INVALID_ARG,
             "[HIBF CONFIG ERROR] config::relaxed_fpr must be greater than or equal to config::maximum_fpr.");
}

// ---- HyperLogLog, as the reference's IBF(config) constructor uses it to find the largest user bin ----------------
// src/sketch/hyperloglog.cpp:28-118: registers of 2^bits bytes; a value's 64-bit wyhash picks the register with
// its top `bits` bits and stores max(rank), rank = leading zeros of the remaining bits + 1; the estimate sums
// 2^-register in single precision over eight lanes (register 8k + 7 - l goes to lane l, lanes added in order),
// corrects with alpha * m^2, and falls back to linear counting when the raw estimate is at most 2.5 m.
struct hll
{
    uint32_t bits;
    uint64_t size;
    uint64_t rank_mask;
    double norm;
    std::vector<uint8_t> reg;

    explicit hll(uint32_t b) : bits{b}, size{1ull << b}, rank_mask{(1ull << b) - 1u}, reg(size, 0)
    {
        double alpha = 0;
        if (size == 32)
            alpha = 0.697;
        else if (size == 64)
            alpha = 0.709;
        else
            alpha = 0.7213 / (1.0 + 1.079 / static_cast<double>(size));
        norm = alpha * static_cast<double>(size) * static_cast<double>(size);
    }
    void add(uint64_t v)
    {
        unsigned __int128 const r = static_cast<unsigned __int128>(v) * 0x9E3779B97F4A7C15ULL;
        uint64_t const h = static_cast<uint64_t>(r) ^ static_cast<uint64_t>(r >> 64);
        uint64_t const idx = h >> (64 - bits);
        uint8_t const rank = static_cast<uint8_t>(__builtin_clzll((h << bits) | rank_mask) + 1);
        reg[idx] = std::max(reg[idx], rank);
    }
    double estimate() const
    {
        float lane[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (uint64_t i = 0; i < size / 32; ++i)
            for (uint64_t j = 0; j <= 24; j += 8)
                for (int l = 0; l < 8; ++l)
                {
                    uint8_t const x = reg[i * 32 + j + 7 - l];
                    lane[l] = lane[l] + 1.0f / static_cast<float>(1ull << x);
                }
        float sum = 0;
        for (int l = 0; l < 8; ++l)
            sum += lane[l];
        double e = norm / static_cast<double>(sum);
        if (e <= 2.5 * static_cast<double>(size))
        {
            uint32_t zeros = 0;
            for (uint8_t x : reg)
                zeros += x == 0;
            if (zeros)
                e = static_cast<double>(size) * std::log(static_cast<double>(size) / zeros);
        }
        return e;
    }
};

} // namespace build
} // namespace hibf_gb300

using namespace hibf_gb300;
using namespace hibf_gb300::build;

struct hibf_gpu_sink
{
    std::vector<uint64_t> values;
};

namespace hibf_gb300
{
// sets.cu: the set materialisation on the device
bool device_present();
void distinct_sets_device(uint64_t const * values, std::vector<uint64_t> const & offsets,
                          std::vector<std::vector<uint64_t>> & sets);
uint64_t union_size_device(std::vector<std::vector<uint64_t>> const & sets, std::vector<uint64_t> const & members);
} // namespace hibf_gb300

namespace
{

double seconds_since(std::chrono::steady_clock::time_point t0)
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// The plan of a synthetic build: pairwise distinct user bins of the given stream ranges, unions sized by sums.
plan_t synthetic_plan(hibf_gpu_build_config const & cfg, char const * layout_text, uint64_t const * user_bin_offsets)
{
    uint64_t const nub = cfg.number_of_user_bins;
    std::vector<uint64_t> distinct(nub);
    for (uint64_t u = 0; u < nub; ++u)
    {
        if (user_bin_offsets[u + 1] < user_bin_offsets[u])
            fail(HIBF_GPU_ERR_INVALID_ARG, "user bin offsets must not decrease");
        distinct[u] = user_bin_offsets[u + 1] - user_bin_offsets[u];
    }
    layout_t const L = parse_layout(layout_text);
    plan_t const P0 = make_plan(cfg, L, distinct, [](size_t) { return uint64_t{1}; });
    std::vector<uint64_t> const sums = disjoint_unions(P0, distinct, L);
    return make_plan(cfg, L, distinct, [&](size_t node) { return sums[node]; });
}

// The host part of hibf_gpu_hibf_build: reads every user bin once through input_fn (its distinct values in input
// order: the set the reference builds with compute_kmers, src/build/compute_kmers.cpp:23-32), sizes the IBFs
// (exact distinct counts of the unions that size merged max bins), and puts split user bins in the reference's
// chunk order.  `sets[u]` receives user bin u's values in device insertion order.  With a device present the distinct
// sets and the union sizes are sorts on the device (sets.cu); without one (planning only) host hash sets.
//
// With `table` the split user bins keep their input order and `table` receives their split table (the device
// chunks them); without it they are reordered into the reference's chunk order on the host.  `timers` (optional)
// receives the user_bin_io and merge_kmers intervals.
plan_t plan_inputs(hibf_gpu_build_config const & cfg_ref, char const * layout_text, hibf_gpu_input_fn input_fn,
                   void * user, std::vector<std::vector<uint64_t>> & sets_out, hibf_gpu_split_table * table,
                   phase_timer * timers = nullptr)
{
    using clock = std::chrono::steady_clock;
    phase_timer scratch[n_timers];
    phase_timer * const T = timers ? timers : scratch;
    auto read_user_bin = [&](uint64_t u, hibf_gpu_sink & sink)
    {
        auto const t0 = clock::now();
        input_fn(user, u, &sink);
        T[timer_user_bin_io].add(seconds_since(t0));
    };
    hibf_gpu_build_config const * cfg = &cfg_ref;
    uint64_t const nub = cfg->number_of_user_bins;
    bool const device = device_present();
    // Read every user bin once: its distinct values in first-appearance order (the set the reference
    // builds with compute_kmers, src/build/compute_kmers.cpp:23-32).
    std::vector<std::vector<uint64_t>> & sets = sets_out;
    sets.assign(nub, {});
    std::vector<uint64_t> distinct(nub);
    if (device)
    {
        std::vector<uint64_t> all, off(nub + 1, 0);
        for (uint64_t u = 0; u < nub; ++u)
        {
            hibf_gpu_sink sink;
            read_user_bin(u, sink);
            all.insert(all.end(), sink.values.begin(), sink.values.end());
            off[u + 1] = all.size();
        }
        auto const t0 = clock::now();
        distinct_sets_device(all.data(), off, sets);
        T[timer_merge_kmers].add(seconds_since(t0));
    }
    else
    {
        auto const t0 = clock::now();
        double const io0 = T[timer_user_bin_io].seconds;
        for (uint64_t u = 0; u < nub; ++u)
        {
            hibf_gpu_sink sink;
            read_user_bin(u, sink);
            std::unordered_set<uint64_t> seen;
            seen.reserve(sink.values.size() * 2);
            for (uint64_t v : sink.values)
                if (seen.insert(v).second)
                    sets[u].push_back(v);
        }
        T[timer_merge_kmers].add(seconds_since(t0) - (T[timer_user_bin_io].seconds - io0));
    }
    for (uint64_t u = 0; u < nub; ++u)
        distinct[u] = sets[u].size();
    layout_t const L = parse_layout(layout_text);
    plan_t const P0 = make_plan(*cfg, L, distinct, [](size_t) { return uint64_t{1}; });
    // exact distinct counts of subtree unions (merged max bins), or sums for disjoint user bins
    std::vector<uint64_t> sums;
    auto const t_union = clock::now();
    if (cfg->user_bins_disjoint)
        sums = disjoint_unions(P0, distinct, L);
    else
    {
        sums.assign(P0.g.size(), 0);
        std::vector<std::vector<uint64_t>> members(P0.g.size());
        for (uint64_t u = 0; u < nub; ++u)
        {
            size_t n = P0.order[P0.ub_leaf[u]];
            while (true)
            {
                members[n].push_back(u);
                if (P0.g[n].parent == SIZE_MAX)
                    break;
                n = P0.g[n].parent;
            }
        }
        for (size_t n = 0; n < P0.g.size(); ++n)
        {
            // only favourite children are sized by their union
            bool needed = false;
            if (P0.g[n].parent != SIZE_MAX)
            {
                node_t const & p = P0.g[P0.g[n].parent];
                needed = p.favourite >= 0 && p.children[static_cast<size_t>(p.favourite)] == n;
            }
            if (!needed)
                continue;
            if (device)
            {
                sums[n] = union_size_device(sets, members[n]);
                continue;
            }
            std::unordered_set<uint64_t> un;
            for (uint64_t u : members[n])
                un.insert(sets[u].begin(), sets[u].end());
            sums[n] = un.size();
        }
    }
    T[timer_merge_kmers].add(seconds_since(t_union));
    plan_t const P = make_plan(*cfg, L, distinct, [&](size_t node) { return sums[node]; });
    unsigned const threads = static_cast<unsigned>(cfg->threads);
    auto const t_split = clock::now();
    if (table)
    {
        compute_split_table(
            P, [&](uint64_t u, auto && f) { for (uint64_t v : sets[u]) f(v); }, threads, *table);
        T[timer_merge_kmers].add(seconds_since(t_split));
        return P;
    }
    // split user bins in the reference's chunk order
    std::vector<std::vector<uint64_t>> split = reference_split_orders(P, sets);
    for (uint64_t u = 0; u < nub; ++u)
        if (P.ub_rec[u].ntb > 1)
            sets[u] = std::move(split[u]);
    T[timer_merge_kmers].add(seconds_since(t_split));
    return P;
}

// create_from_plan with the index_allocation interval: the stores are allocated and zeroed when it returns.
hibf_gpu_hibf * allocate_timed(plan_t const & P, uint64_t n_user_bins, phase_timer & t)
{
    auto const t0 = std::chrono::steady_clock::now();
    hibf_gpu_hibf * h = create_from_plan(P, n_user_bins);
    cudaError_t const e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess)
    {
        hibf_gpu_hibf_destroy(h);
        fail(HIBF_GPU_ERR_CUDA, cudaGetErrorString(e));
    }
    t.add(seconds_since(t0));
    return h;
}

} // namespace

extern "C"
{

    int hibf_gpu_hll_sketch(uint64_t const * values, uint64_t n, uint32_t bits, uint8_t * registers)
    {
        return guarded(
            [&]
            {
                if ((n && !values) || !registers)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                if (bits < 5 || bits > 32)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "sketch bits must be in [5, 32]");
                hll h(bits);
                for (uint64_t i = 0; i < n; ++i)
                    h.add(values[i]);
                std::copy(h.reg.begin(), h.reg.end(), registers);
            });
    }

    int hibf_gpu_hll_estimate(uint8_t const * registers, uint32_t bits, double * estimate)
    {
        return guarded(
            [&]
            {
                if (!registers || !estimate)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                if (bits < 5 || bits > 32)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "sketch bits must be in [5, 32]");
                hll h(bits);
                std::copy(registers, registers + h.size, h.reg.begin());
                *estimate = h.estimate();
            });
    }

    int hibf_gpu_sink_push(hibf_gpu_sink * sink, uint64_t const * values, uint64_t n)
    {
        return guarded(
            [&]
            {
                if (!sink || (n && !values))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                sink->values.insert(sink->values.end(), values, values + n);
            });
    }

    int hibf_gpu_ibf_plan(hibf_gpu_build_config const * cfg, uint64_t max_bin_elements, uint32_t sketch_bits,
                          hibf_gpu_input_fn input_fn, void * user, uint64_t * bin_size, uint64_t * biggest_user_bin)
    {
        return guarded(
            [&]
            {
                validate(cfg);
                if (!input_fn || !bin_size)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument (config::input_fn is required)");
                if (sketch_bits < 5 || sketch_bits > 32)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "[HIBF CONFIG ERROR] config::sketch_bits must be in [5,32].");
                // max_bin_size (src/interleaved_bloom_filter.cpp:81-101): the largest user bin by sketch estimate
                // (the first one on ties), then its exact distinct count
                uint64_t max_size = max_bin_elements;
                uint64_t best = 0;
                if (max_size == 0)
                {
                    uint64_t best_est = 0;
                    for (uint64_t u = 0; u < cfg->number_of_user_bins; ++u)
                    {
                        hibf_gpu_sink sink;
                        input_fn(user, u, &sink);
                        hll sk(sketch_bits);
                        for (uint64_t v : sink.values)
                            sk.add(v);
                        uint64_t const est = static_cast<uint64_t>(sk.estimate());
                        if (est > best_est)
                        {
                            best_est = est;
                            best = u;
                        }
                    }
                    hibf_gpu_sink sink;
                    input_fn(user, best, &sink);
                    std::unordered_set<uint64_t> distinct(sink.values.begin(), sink.values.end());
                    max_size = distinct.size();
                }
                *bin_size = bin_size_in_bits(cfg->maximum_fpr, cfg->number_of_hash_functions, max_size);
                if (biggest_user_bin)
                    *biggest_user_bin = best;
            });
    }

    int hibf_gpu_ibf_build(hibf_gpu_build_config const * cfg, uint64_t max_bin_elements, uint32_t sketch_bits,
                           int track_occupancy, hibf_gpu_input_fn input_fn, void * user, hibf_gpu_ibf ** out)
    {
        return guarded(
            [&]
            {
                validate(cfg);
                if (!input_fn || !out)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument (config::input_fn is required)");
                if (sketch_bits < 5 || sketch_bits > 32)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "[HIBF CONFIG ERROR] config::sketch_bits must be in [5,32].");
                *out = nullptr;
                uint64_t const nub = cfg->number_of_user_bins;
                uint64_t bits = 0;
                int const pst = hibf_gpu_ibf_plan(cfg, max_bin_elements, sketch_bits, input_fn, user, &bits, nullptr);
                if (pst != HIBF_GPU_OK)
                    fail(pst, hibf_gpu_last_error());
                hibf_gpu_ibf * f = nullptr;
                int const st = hibf_gpu_ibf_create(nub, bits, cfg->number_of_hash_functions, track_occupancy, &f);
                if (st != HIBF_GPU_OK)
                    fail(st, std::string("IBF construction failed: ") + hibf_gpu_last_error());
                try
                {
                    // IBF.cpp:104-117: every user bin's values into its own bin
                    for (uint64_t u = 0; u < nub; ++u)
                    {
                        hibf_gpu_sink sink;
                        input_fn(user, u, &sink);
                        int const e = hibf_gpu_ibf_emplace(f, sink.values.data(), sink.values.size(), u);
                        if (e != HIBF_GPU_OK)
                            fail(e, hibf_gpu_last_error());
                    }
                }
                catch (...)
                {
                    hibf_gpu_ibf_destroy(f);
                    throw;
                }
                *out = f;
            });
    }

    int hibf_gpu_plan_disjoint(hibf_gpu_build_config const * cfg, char const * layout_text,
                               uint64_t const * user_bin_sizes, uint64_t * n_ibfs, uint64_t * total_bins,
                               uint64_t * bins, uint64_t * bin_sizes, uint64_t * next_ibf_id, uint64_t * user_bin_id,
                               uint64_t * parent_ibf, uint64_t * parent_bin)
    {
        return guarded(
            [&]
            {
                validate(cfg);
                if (!user_bin_sizes || !n_ibfs || !total_bins)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                layout_t const L = parse_layout(layout_text);
                std::vector<uint64_t> const distinct(user_bin_sizes, user_bin_sizes + cfg->number_of_user_bins);
                std::vector<uint64_t> sums;
                plan_t const P = make_plan(*cfg, L, distinct,
                                           [&](size_t node)
                                           {
                                               (void)node;
                                               return uint64_t{1}; // placeholder: only placements are used
                                           });
                // second pass with the subtree sums now that placements are known
                sums = disjoint_unions(P, distinct, L);
                plan_t const Q = make_plan(*cfg, L, distinct,
                                           [&](size_t node)
                                           {
                                               return sums[node];
                                           });
                *n_ibfs = Q.bins.size();
                *total_bins = Q.tb_off.back();
                if (bins)
                    std::copy(Q.bins.begin(), Q.bins.end(), bins);
                if (bin_sizes)
                    std::copy(Q.bin_size.begin(), Q.bin_size.end(), bin_sizes);
                if (next_ibf_id)
                    std::copy(Q.next_ibf.begin(), Q.next_ibf.end(), next_ibf_id);
                if (user_bin_id)
                    std::copy(Q.user_bin.begin(), Q.user_bin.end(), user_bin_id);
                if (parent_ibf)
                    std::copy(Q.parent_ibf.begin(), Q.parent_ibf.end(), parent_ibf);
                if (parent_bin)
                    std::copy(Q.parent_bin.begin(), Q.parent_bin.end(), parent_bin);
            });
    }

    int hibf_gpu_split_table_synthetic(hibf_gpu_build_config const * cfg, char const * layout_text, uint64_t seed,
                                       uint64_t const * user_bin_offsets, hibf_gpu_split_table ** out)
    {
        return guarded(
            [&]
            {
                validate(cfg);
                if (!user_bin_offsets || !out)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                *out = nullptr;
                plan_t const P = synthetic_plan(*cfg, layout_text, user_bin_offsets);
                auto * t = new hibf_gpu_split_table;
                try
                {
                    compute_split_table(
                        P,
                        [&](uint64_t u, auto && f)
                        {
                            for (uint64_t k = user_bin_offsets[u]; k < user_bin_offsets[u + 1]; ++k)
                                f(hg_stream_at(seed, k));
                        },
                        static_cast<unsigned>(cfg->threads), *t);
                }
                catch (...)
                {
                    delete t;
                    throw;
                }
                *out = t;
            });
    }

    int hibf_gpu_split_table_inputs(hibf_gpu_build_config const * cfg, char const * layout_text,
                                    hibf_gpu_input_fn input_fn, void * user, hibf_gpu_split_table ** out)
    {
        return guarded(
            [&]
            {
                validate(cfg);
                if (!input_fn || !out)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument (config::input_fn is required)");
                *out = nullptr;
                std::vector<std::vector<uint64_t>> sets;
                auto * t = new hibf_gpu_split_table;
                try
                {
                    plan_inputs(*cfg, layout_text, input_fn, user, sets, t);
                }
                catch (...)
                {
                    delete t;
                    throw;
                }
                *out = t;
            });
    }

    int hibf_gpu_split_table_sizes(hibf_gpu_split_table const * t, uint64_t * n_split, uint64_t * n_boundaries,
                                   uint64_t * n_before)
    {
        return guarded(
            [&]
            {
                if (!t || !n_split || !n_boundaries || !n_before)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                *n_split = t->user_bin.size();
                *n_boundaries = t->home.size();
                *n_before = t->before.size();
            });
    }

    int hibf_gpu_split_table_export(hibf_gpu_split_table const * t, uint64_t * user_bin, uint64_t * n_values,
                                    uint64_t * mult, uint64_t * mask, uint64_t * bnd_off, uint64_t * bnd_home,
                                    uint64_t * before_off, uint64_t * before)
    {
        return guarded(
            [&]
            {
                if (!t || !user_bin || !n_values || !mult || !mask || !bnd_off || !bnd_home || !before_off ||
                    (!before && !t->before.empty()))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                std::copy(t->user_bin.begin(), t->user_bin.end(), user_bin);
                std::copy(t->n.begin(), t->n.end(), n_values);
                std::copy(t->mult.begin(), t->mult.end(), mult);
                std::copy(t->mask.begin(), t->mask.end(), mask);
                std::copy(t->bnd_off.begin(), t->bnd_off.end(), bnd_off);
                std::copy(t->home.begin(), t->home.end(), bnd_home);
                std::copy(t->before_off.begin(), t->before_off.end(), before_off);
                std::copy(t->before.begin(), t->before.end(), before);
            });
    }

    int hibf_gpu_split_table_import(uint64_t n_split, uint64_t n_boundaries, uint64_t n_before,
                                    uint64_t const * user_bin, uint64_t const * n_values, uint64_t const * mult,
                                    uint64_t const * mask, uint64_t const * bnd_off, uint64_t const * bnd_home,
                                    uint64_t const * before_off, uint64_t const * before, hibf_gpu_split_table ** out)
    {
        return guarded(
            [&]
            {
                if (!out || (n_split && (!user_bin || !n_values || !mult || !mask)) || !bnd_off || !before_off ||
                    (n_boundaries && !bnd_home) || (n_before && !before))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                *out = nullptr;
                auto * t = new hibf_gpu_split_table;
                t->user_bin.assign(user_bin, user_bin + n_split);
                t->n.assign(n_values, n_values + n_split);
                t->mult.assign(mult, mult + n_split);
                t->mask.assign(mask, mask + n_split);
                t->bnd_off.assign(bnd_off, bnd_off + n_split + 1);
                t->home.assign(bnd_home, bnd_home + n_boundaries);
                t->before_off.assign(before_off, before_off + n_boundaries + 1);
                t->before.assign(before, before + n_before);
                *out = t;
            });
    }

    int hibf_gpu_split_table_chunks(hibf_gpu_split_table const * t, uint64_t user_bin, uint64_t const * values,
                                    uint64_t n, uint64_t * chunks)
    {
        return guarded(
            [&]
            {
                if (!t || (n && (!values || !chunks)))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                auto const it = std::lower_bound(t->user_bin.begin(), t->user_bin.end(), user_bin);
                if (it == t->user_bin.end() || *it != user_bin)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "the user bin is not split");
                size_t const i = static_cast<size_t>(it - t->user_bin.begin());
                uint64_t const b0 = t->bnd_off[i];
                for (uint64_t j = 0; j < n; ++j)
                    chunks[j] = split_chunk(values[j], t->mult[i], t->mask[i], t->home.data() + b0,
                                            t->bnd_off[i + 1] - b0, t->before_off.data() + b0, t->before.data());
            });
    }

    void hibf_gpu_split_table_destroy(hibf_gpu_split_table * t)
    {
        delete t;
    }

    int hibf_gpu_hibf_build_synthetic(hibf_gpu_build_config const * cfg, char const * layout_text, uint64_t seed,
                                      uint64_t const * user_bin_offsets, hibf_gpu_split_table const * table,
                                      hibf_gpu_hibf ** out)
    {
        return guarded(
            [&]
            {
                validate(cfg);
                if (!user_bin_offsets || !out)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                *out = nullptr;
                uint64_t const nub = cfg->number_of_user_bins;
                plan_t const P = synthetic_plan(*cfg, layout_text, user_bin_offsets);
                phase_timer timers[n_timers];
                hibf_gpu_split_table computed;
                if (!table)
                {
                    auto const t0 = std::chrono::steady_clock::now();
                    compute_split_table(
                        P,
                        [&](uint64_t u, auto && f)
                        {
                            for (uint64_t k = user_bin_offsets[u]; k < user_bin_offsets[u + 1]; ++k)
                                f(hg_stream_at(seed, k));
                        },
                        static_cast<unsigned>(cfg->threads), computed);
                    timers[timer_merge_kmers].add(seconds_since(t0));
                    table = &computed;
                }
                std::vector<uint64_t> distinct(nub);
                for (uint64_t u = 0; u < nub; ++u)
                    distinct[u] = user_bin_offsets[u + 1] - user_bin_offsets[u];
                std::vector<uint64_t> const entry = check_split_table(P, *table, distinct);
                hibf_gpu_hibf * h = allocate_timed(P, nub, timers[timer_index_allocation]);
                try
                {
                    dev_split_table dt;
                    upload_split_table(*table, dt, h->stream);
                    std::vector<insert_job> jobs;
                    for (uint64_t u = 0; u < nub; ++u)
                    {
                        uint64_t const n = distinct[u];
                        user_bin_rec const & r = P.ub_rec[u];
                        jobs.push_back(insert_job{user_bin_offsets[u], n, entry[u],
                                                  static_cast<uint32_t>(P.ub_leaf[u]),
                                                  static_cast<uint32_t>(r.storage)});
                        for (auto const & [ibf, bin] : P.ub_merged[u])
                            jobs.push_back(insert_job{user_bin_offsets[u], n, 0, static_cast<uint32_t>(ibf),
                                                      static_cast<uint32_t>(bin)});
                    }
                    auto const t0 = std::chrono::steady_clock::now();
                    run_jobs(h, jobs, seed, nullptr, &dt, h->stream);
                    timers[timer_fill_ibf].add(seconds_since(t0));
                    std::copy(timers, timers + n_timers, h->timers);
                }
                catch (...)
                {
                    hibf_gpu_hibf_destroy(h);
                    throw;
                }
                *out = h;
            });
    }

    int hibf_gpu_hibf_build(hibf_gpu_build_config const * cfg, char const * layout_text, hibf_gpu_input_fn input_fn,
                            void * user, hibf_gpu_hibf ** out)
    {
        return guarded(
            [&]
            {
                validate(cfg);
                if (!input_fn || !out)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument (config::input_fn is required)");
                *out = nullptr;
                uint64_t const nub = cfg->number_of_user_bins;
                std::vector<std::vector<uint64_t>> sets;
                hibf_gpu_split_table table;
                phase_timer timers[n_timers];
                plan_t const P = plan_inputs(*cfg, layout_text, input_fn, user, sets, &table, timers);
                std::vector<uint64_t> distinct(nub);
                for (uint64_t u = 0; u < nub; ++u)
                    distinct[u] = sets[u].size();
                std::vector<uint64_t> const entry = check_split_table(P, table, distinct);
                hibf_gpu_hibf * h = allocate_timed(P, nub, timers[timer_index_allocation]);
                try
                {
                    dev_split_table dt;
                    upload_split_table(table, dt, h->stream);
                    // all distinct values, concatenated, uploaded once
                    auto const t_io = std::chrono::steady_clock::now();
                    std::vector<uint64_t> off(nub + 1, 0);
                    for (uint64_t u = 0; u < nub; ++u)
                        off[u + 1] = off[u] + sets[u].size();
                    dbuf dv;
                    dv.ensure(off[nub] * 8);
                    for (uint64_t u = 0; u < nub; ++u)
                        if (!sets[u].empty())
                            HG_CUDA(cudaMemcpyAsync(dv.as<uint64_t>() + off[u], sets[u].data(), sets[u].size() * 8,
                                                    cudaMemcpyHostToDevice, h->stream));
                    HG_CUDA(cudaStreamSynchronize(h->stream));
                    timers[timer_user_bin_io].add(seconds_since(t_io));
                    std::vector<insert_job> jobs;
                    for (uint64_t u = 0; u < nub; ++u)
                    {
                        uint64_t const n = sets[u].size();
                        user_bin_rec const & r = P.ub_rec[u];
                        jobs.push_back(insert_job{off[u], n, entry[u], static_cast<uint32_t>(P.ub_leaf[u]),
                                                  static_cast<uint32_t>(r.storage)});
                        for (auto const & [ibf, bin] : P.ub_merged[u])
                            jobs.push_back(
                                insert_job{off[u], n, 0, static_cast<uint32_t>(ibf), static_cast<uint32_t>(bin)});
                    }
                    auto const t_fill = std::chrono::steady_clock::now();
                    run_jobs(h, jobs, 0, dv.as<uint64_t>(), &dt, h->stream);
                    timers[timer_fill_ibf].add(seconds_since(t_fill));
                    std::copy(timers, timers + n_timers, h->timers);
                }
                catch (...)
                {
                    hibf_gpu_hibf_destroy(h);
                    throw;
                }
                *out = h;
            });
    }

    int hibf_gpu_hibf_build_timers(hibf_gpu_hibf const * h, hibf_gpu_timer * timers)
    {
        return guarded(
            [&]
            {
                if (!h || !timers)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                for (int i = 0; i < n_timers; ++i)
                    timers[i] = hibf_gpu_timer{h->timers[i].seconds, h->timers[i].max_seconds, h->timers[i].count};
            });
    }

    int hibf_gpu_hibf_build_inputs(hibf_gpu_build_config const * cfg, char const * layout_text,
                                   hibf_gpu_input_fn input_fn, void * user, uint64_t * offsets, uint64_t * values)
    {
        return guarded(
            [&]
            {
                validate(cfg);
                if (!input_fn || !offsets)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                std::vector<std::vector<uint64_t>> sets;
                plan_inputs(*cfg, layout_text, input_fn, user, sets, nullptr);
                offsets[0] = 0;
                for (size_t u = 0; u < sets.size(); ++u)
                {
                    offsets[u + 1] = offsets[u] + sets[u].size();
                    if (values)
                        std::copy(sets[u].begin(), sets[u].end(), values + offsets[u]);
                }
            });
    }

} // extern "C"
