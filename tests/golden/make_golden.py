"""Generates the golden vectors in tests/golden from the REFERENCE itself.

Run where the seqan/hibf source tree is available (a checkout named `reference` beside this repository, or
HIBF_REFERENCE_DIR):

    python tests/golden/make_golden.py

It compiles the reference's own sources against the cereal/simde stand-ins (oracle/Makefile target `ref`) and drives
them through oracle/ref_driver.cpp:

  ibf_cases.npz      random IBF cases: emplace inputs, the digest of the reference's bit store, bulk_contains words,
                     bulk_count for counter widths 1/2/4/8 (wraparound included), membership_for at several
                     thresholds, occupancy, clear / clear(range) / increase_bin_number_to sequences.
  hibf_<name>.npz    small HIBFs built by the reference (HIBF(config)): the layout it computed, its tables and bit
                     words, queries, and the reference's outputs (membership in traversal order and sorted, dense
                     uint16/uint32/uint8 counting vectors, per-query digests).
  c3_layout.txt      the layout the reference computes (HyperLogLog sketches + DP) for the 8,192-user-bin workload
                     (sizes log-normal(2e5, 1.5) clipped to [1e3, 5e7], h=2, fpr 0.05, tmax 64, sketch_bits 12, seed 1).
  ibf_config.npz     interleaved_bloom_filter(config&, max_bin_elements): bin size (largest user bin by HyperLogLog
                     estimate, then its exact count), bit store digest, counts, for several configs.
  c1_reference.npz   the 64-user-bin workload (log-uniform [1e3, 1e5], h=2, fpr 0.05, tmax 64): layout, per-IBF
                     digests and tables, 10,000 queries' outputs digests.
  ref_c3_<s>.npz     the reference's build of the 8,192-user-bin workload from c3_layout.txt with every user bin at
  ref_c4_<s>.npz     scale s (1 = full size), and of the 65,536-user-bin one from c4_layout_sum.txt: tables and
                     per-IBF digests (targets refc3, refc3s, refc4s, refc4m; minutes each, not in the default set).

Nothing here is read by the product; tests compare the oracle and the GPU path against these files.
"""

from __future__ import annotations

import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from hibf_gb300 import synthetic as S  # noqa: E402
from oracle.bindings import Reference, build_reference, ref_cfg  # noqa: E402

OUT = Path(__file__).resolve().parent
MERGED = np.uint64(0xFFFFFFFFFFFFFFFF)


def digest_words(w: np.ndarray) -> int:
    # same fold as hg_digest_step, vectorised poorly but fine for fixture sizes
    return S.digest(w.tolist())


IBF_CASES = [
    # bins, bin_size, h, track_occupancy, n_insert, n_query
    (64, 1024, 2, 0, 3000, 400),
    (73, 1019, 3, 0, 3000, 400),
    (1, 100, 1, 0, 200, 100),
    (128, 512, 2, 1, 3000, 400),
    (1024, 4096, 3, 0, 20000, 300),
    (200, 777, 5, 0, 4000, 300),
    (65, 64, 4, 1, 2000, 300),
    (12, 8192, 2, 0, 500, 200),
    (192, 1500, 2, 0, 4000, 300),  # 3 words per row: padded on the device
    (2047, 333, 2, 0, 6000, 200),  # 32 words per row
    (2100, 100, 2, 0, 6000, 100),  # 33 words per row: wider than a warp
    (8, 64, 1, 0, 6000, 2000),     # tiny filter: counts above 255 wrap in uint8
]


def make_ibf_cases(R: Reference):
    out = {}
    for ci, (bins, bsz, h, track, n_ins, n_q) in enumerate(IBF_CASES):
        rng = np.random.default_rng(1000 + ci)
        vals = rng.integers(0, 2**64, n_ins, dtype=np.uint64)
        bns = rng.integers(0, bins, n_ins).astype(np.uint64)
        q = np.concatenate([vals[: n_q // 2], rng.integers(0, 2**64, n_q - n_q // 2, dtype=np.uint64)])
        ibf = R.ibf(bins, bsz, h, bool(track))
        ibf.emplace(vals, bns)
        p = f"c{ci}_"
        out[p + "params"] = np.array([bins, bsz, h, track], np.uint64)
        out[p + "values"] = vals
        out[p + "bins"] = bns
        out[p + "queries"] = q
        out[p + "digest"] = np.array([digest_words(ibf.words())], np.uint64)
        out[p + "contains"] = ibf.bulk_contains(q)
        for w in (1, 2, 4, 8):
            out[p + f"count{w}"] = ibf.bulk_count(q, w)
        for t in (0, 1, 2, 3, 50):
            out[p + f"member{t}"] = ibf.membership_for(q, t)
        if track:
            out[p + "occupancy"] = ibf.occupancy()
        # clear(bin), clear(range), then widen
        ibf.clear(bins // 2)
        out[p + "after_clear"] = ibf.bulk_count(q, 4)
        rb = np.unique(rng.integers(0, bins, 5)).astype(np.uint64)
        ibf.clear_range(rb)
        out[p + "clear_range_bins"] = rb
        out[p + "after_clear_range"] = ibf.bulk_count(q, 4)
        if track:
            out[p + "occupancy_after_clear"] = ibf.occupancy()
        new_bins = bins + 70
        ibf.increase_bin_number_to(new_bins)
        out[p + "widened_bins"] = np.array([new_bins], np.uint64)
        out[p + "widened_digest"] = np.array([digest_words(ibf.words())], np.uint64)
        out[p + "widened_count"] = ibf.bulk_count(q, 2)
    out["n_cases"] = np.array([len(IBF_CASES)], np.uint64)
    np.savez_compressed(OUT / "ibf_cases.npz", **out)


def hibf_case(R: Reference, name: str, cfg, values, offsets, queries, mem_t, cnt_t, widths=(2,), synthetic_seed=None):
    t0 = time.time()
    if synthetic_seed is None:
        layout = R.layout(cfg, values, offsets)
        H = R.hibf(cfg, values, offsets)
    else:
        layout = R.layout(cfg, None, offsets, seed=synthetic_seed, synthetic=True)
        H = R.hibf(cfg, None, offsets, seed=synthetic_seed, synthetic=True)
    T = H.tables(with_words=True)
    qv, qo = queries
    nq = qo.size - 1
    nub = int(cfg.number_of_user_bins)
    unsorted, sorted_, dense = [], [], {w: [] for w in widths}
    for i in range(nq):
        v = qv[qo[i]:qo[i + 1]]
        unsorted.append(H.membership_for(v, int(mem_t[i]), sort=False))
        sorted_.append(np.sort(unsorted[-1]))
        for w in widths:
            dense[w].append(H.bulk_count(v, int(cnt_t[i]), w))
    lens = np.array([u.size for u in unsorted], np.uint64)
    moff = np.zeros(nq + 1, np.uint64)
    np.cumsum(lens, out=moff[1:])
    out = dict(n_user_bins=np.array([nub], np.uint64), bins=T["bins"], bin_size=T["bin_size"],
               hash_funs=T["hash_funs"], next_ibf=T["next_ibf"], user_bin=T["user_bin"], digests=T["digests"],
               words=np.concatenate(T["words"]), layout=np.frombuffer(layout.encode(), np.uint8),
               config=np.array([cfg.number_of_hash_functions, cfg.tmax, cfg.sketch_bits], np.uint64),
               fpr=np.array([cfg.maximum_fpr, cfg.relaxed_fpr, cfg.alpha, cfg.max_rearrangement_ratio], np.float64),
               flags=np.array([cfg.disable_estimate_union, cfg.disable_rearrangement], np.uint64),
               q_values=qv, q_offsets=qo, mem_t=np.asarray(mem_t, np.uint64), cnt_t=np.asarray(cnt_t, np.uint64),
               mem_offsets=moff, mem_unsorted=np.concatenate(unsorted) if nq else np.zeros(0, np.uint64),
               mem_sorted=np.concatenate(sorted_) if nq else np.zeros(0, np.uint64))
    if values is not None:
        out["ub_values"] = np.asarray(values, np.uint64)
        out["ub_offsets"] = np.asarray(offsets, np.uint64)
    else:
        out["ub_offsets"] = np.asarray(offsets, np.uint64)
        out["synthetic_seed"] = np.array([synthetic_seed], np.uint64)
    for w in widths:
        out[f"count{w}"] = np.stack(dense[w]) if nq else np.zeros((0, nub))
    np.savez_compressed(OUT / f"hibf_{name}.npz", **out)
    print(f"hibf_{name}: {len(T['bins'])} IBFs, {sum(x.size for x in T['words'])} words, {nq} queries, "
          f"{time.time() - t0:.1f}s")


def csr(lists):
    v = np.concatenate([np.asarray(x, np.uint64) for x in lists]) if lists else np.zeros(0, np.uint64)
    o = np.zeros(len(lists) + 1, np.uint64)
    np.cumsum([len(x) for x in lists], out=o[1:])
    return v, o


def make_hibf_cases(R: Reference):
    # test/snippet/hibf/hierarchical_interleaved_bloom_filter.cpp and the unit test small example
    ubs = [[1, 2, 3, 4, 5, 6, 7, 8, 9, 10], [1, 2, 3, 4, 5]]
    v, o = csr(ubs)
    q = csr([[1, 2, 3, 4, 5], [1, 2, 3, 4, 5], [1, 2, 3, 4, 5]])
    hibf_case(R, "snippet", ref_cfg(2), v, o, q, [2, 6, 2], [1, 6, 1], widths=(2, 8))
    # test/snippet/readme.cpp
    ubs = [[1, 2, 3, 4, 5, 6, 7, 8, 9, 10], [1, 2, 3, 4, 5], [3, 9, 11]]
    v, o = csr(ubs)
    q = csr([[3, 9, 12, 14], list(range(15))])
    hibf_case(R, "readme", ref_cfg(3), v, o, q, [2, 5], [2, 5])
    # test/unit/hibf/hierarchical_interleaved_bloom_filter_test.cpp:112 three_level_hibf
    n = 4097
    ubs = [list(range(i * 16, i * 16 + 20)) for i in range(n)]
    v, o = csr(ubs)
    qs = []
    for ub in range(0, 4096, 100):
        s = ub * 16
        qs += [list(range(s + 16, s + 20)), list(range(s + 5, s + 9))]
    cfg = ref_cfg(n, fpr=0.001, threads=4, tmax=64, disable_estimate_union=True, disable_rearrangement=True)
    hibf_case(R, "three_level", cfg, v, o, csr(qs), [4] * len(qs), [1] * len(qs))
    # :164 unevenly_sized_and_unique_user_bins
    ubs = [list(range((i + 1) ** 2, (i + 2) ** 2 - 1)) for i in range(500)]
    v, o = csr(ubs)
    qs = [list(range((ub + 1) ** 2 + 5, (ub + 1) ** 2 + 9)) for ub in range(5, 499, 20)]
    qs.append(list(range(1, 251000)))
    cfg = ref_cfg(500, fpr=0.001, threads=4, tmax=64, disable_estimate_union=True, disable_rearrangement=True)
    hibf_case(R, "uneven", cfg, v, o, csr(qs), [4] * (len(qs) - 1) + [1], [1] * len(qs), widths=(2, 4))
    # :198 evenly_sized_and_highly_similar_user_bins
    ubs = [list(range(i * 5, i * 5 + 35)) for i in range(1000)]
    v, o = csr(ubs)
    qs = [list(range(ub * 5, ub * 5 + 5)) for ub in range(6, 994, 20)]
    cfg = ref_cfg(1000, fpr=0.001, threads=4, tmax=64, disable_estimate_union=True, disable_rearrangement=True)
    hibf_case(R, "similar", cfg, v, o, csr(qs), [5] * len(qs), [1] * len(qs))
    # :233 counting_agent_same_bins
    ubs = [list(range(500))] * 500
    v, o = csr(ubs)
    cfg = ref_cfg(500, fpr=0.001, threads=4, tmax=64, disable_estimate_union=True, disable_rearrangement=True)
    hibf_case(R, "same", cfg, v, o, csr([list(range(500))]), [1], [1], widths=(2, 4))
    # synthetic, 64 user bins (the small workload's shape at reduced sizes), with uint8 wraparound queries
    sizes = S.user_bin_sizes(7, 64, S.SIZES_LOG_UNIFORM, 0, 0, 50, 2000)
    offs = S.offsets_of(sizes)
    spec = S.query_spec(7, S.QUERIES_HALF_ONE_BIN, 100, 100, 0, 0, 1, 2, 64)
    qv, qo, thr = S.queries(spec, offs, 0, 400)
    spec2 = S.query_spec(8, S.QUERIES_HALF_ONE_BIN, 700, 700, 0, 0, 1, 2, 64)
    qv2, qo2, thr2 = S.queries(spec2, offs, 0, 40)
    qv = np.concatenate([qv, qv2])
    qo = np.concatenate([qo, qo2[1:] + qo[-1]])
    mem_t = np.concatenate([thr, np.full(40, 3, np.uint64)])
    cnt_t = np.concatenate([thr, np.ones(40, np.uint64)])
    cfg = ref_cfg(64, h=2, fpr=0.05, tmax=64)
    hibf_case(R, "synth64", cfg, None, offs, (qv, qo), mem_t, cnt_t, widths=(1, 2, 4), synthetic_seed=7)
    # synthetic, 600 user bins, three levels with tmax 64, h=3, fpr 0.02, mixed queries
    sizes = S.user_bin_sizes(11, 600, S.SIZES_LOG_NORMAL, 300.0, 1.2, 20, 20000)
    offs = S.offsets_of(sizes)
    spec = S.query_spec(11, S.QUERIES_MIXED, 20, 300, 70, 2, 7, 10, 600)
    qv, qo, thr = S.queries(spec, offs, 0, 300)
    cfg = ref_cfg(600, h=3, fpr=0.02, tmax=64)
    hibf_case(R, "synth600", cfg, None, offs, (qv, qo), thr, thr, widths=(2,), synthetic_seed=11)


def make_dups_case(R: Reference):
    """User bins read with repeated values (drawn with replacement from a per-bin pool plus a pool shared by all):
    the builder's distinct sets in first-appearance order and the split bins' hash-set order both see duplicates."""
    rng = np.random.default_rng(21)
    shared = rng.integers(0, 2**63, 64, dtype=np.uint64)
    sizes = np.clip(np.exp(rng.normal(np.log(300.0), 1.3, 200)).astype(np.int64), 5, 20000)
    ubs = []
    for n in sizes:
        pool = np.concatenate([rng.integers(0, 2**63, max(1, int(n) // 3), dtype=np.uint64), shared[:8]])
        ubs.append(rng.choice(pool, int(n), replace=True))
    v, o = csr(ubs)
    qs = [np.resize(ubs[u], 60) for u in range(0, 200, 7)] + [rng.integers(0, 2**63, 60, dtype=np.uint64)]
    thr = [20] * len(qs)
    cfg = ref_cfg(200, h=2, fpr=0.05, tmax=64)
    hibf_case(R, "dups", cfg, v, o, csr(qs), thr, thr, widths=(2,))


def make_sizing_cases(R: Reference):
    """A non-default relaxed_fpr (the merged max bins' sizing) and rows of 8 words (tmax 512: the default kernel
    variant)."""
    sizes = S.user_bin_sizes(37, 300, S.SIZES_LOG_NORMAL, 400.0, 1.4, 20, 20000)
    offs = S.offsets_of(sizes)
    spec = S.query_spec(37, S.QUERIES_MIXED, 20, 400, 70, 2, 7, 10, 300)
    qv, qo, thr = S.queries(spec, offs, 0, 300)
    cfg = ref_cfg(300, h=3, fpr=0.01, relaxed_fpr=0.1, tmax=64)
    hibf_case(R, "relaxed_fpr", cfg, None, offs, (qv, qo), thr, thr, widths=(2,), synthetic_seed=37)
    sizes = S.user_bin_sizes(41, 1500, S.SIZES_LOG_NORMAL, 80.0, 1.5, 5, 20000)
    offs = S.offsets_of(sizes)
    spec = S.query_spec(41, S.QUERIES_MIXED, 20, 300, 70, 2, 7, 10, 1500)
    qv, qo, thr = S.queries(spec, offs, 0, 300)
    cfg = ref_cfg(1500, h=2, fpr=0.05, tmax=512)
    hibf_case(R, "synth_t512", cfg, None, offs, (qv, qo), thr, thr, widths=(2,), synthetic_seed=41)


def make_empty_bins_case(R: Reference):
    """config::empty_bin_fraction: the layout keeps a quarter of every IBF's technical bins empty (and the reference
    then tracks occupancy)."""
    sizes = S.user_bin_sizes(31, 300, S.SIZES_LOG_NORMAL, 300.0, 1.3, 20, 20000)
    offs = S.offsets_of(sizes)
    spec = S.query_spec(31, S.QUERIES_MIXED, 20, 400, 70, 2, 7, 10, 300)
    qv, qo, thr = S.queries(spec, offs, 0, 300)
    cfg = ref_cfg(300, h=2, fpr=0.05, tmax=64, empty_bin_fraction=0.25)
    hibf_case(R, "empty_bins", cfg, None, offs, (qv, qo), thr, thr, widths=(2,), synthetic_seed=31)


def make_many_hash_cases(R: Reference):
    """HIBFs with 1, 4 and 5 hash functions (the query kernels for h = 4 and 5 run the default variant only)."""
    sizes = S.user_bin_sizes(29, 250, S.SIZES_LOG_NORMAL, 300.0, 1.3, 20, 20000)
    offs = S.offsets_of(sizes)
    spec = S.query_spec(29, S.QUERIES_MIXED, 20, 400, 70, 2, 7, 10, 250)
    qv, qo, thr = S.queries(spec, offs, 0, 300)
    cfg = ref_cfg(250, h=1, fpr=0.05, tmax=64)
    hibf_case(R, "synth_h1", cfg, None, offs, (qv, qo), thr, thr, widths=(2,), synthetic_seed=29)
    sizes = S.user_bin_sizes(19, 300, S.SIZES_LOG_NORMAL, 300.0, 1.3, 20, 20000)
    offs = S.offsets_of(sizes)
    spec = S.query_spec(19, S.QUERIES_MIXED, 20, 400, 70, 2, 7, 10, 300)
    qv, qo, thr = S.queries(spec, offs, 0, 300)
    cfg = ref_cfg(300, h=4, fpr=0.05, tmax=64)
    hibf_case(R, "synth_h4", cfg, None, offs, (qv, qo), thr, thr, widths=(2,), synthetic_seed=19)
    sizes = S.user_bin_sizes(23, 400, S.SIZES_LOG_NORMAL, 200.0, 1.5, 10, 20000)
    offs = S.offsets_of(sizes)
    spec = S.query_spec(23, S.QUERIES_MIXED, 20, 400, 70, 2, 6, 10, 400)
    qv, qo, thr = S.queries(spec, offs, 0, 300)
    cfg = ref_cfg(400, h=5, fpr=0.02, tmax=128)
    hibf_case(R, "synth_h5", cfg, None, offs, (qv, qo), thr, thr, widths=(1, 2), synthetic_seed=23)


def make_hibf_wide_cases(R: Reference):
    """Hierarchies whose IBFs have rows of 2 and 4 words (tmax 128 and 256), for the 16-byte-fetch kernels."""
    # the 65,536-user-bin workload's shape at reduced sizes: h=3, fpr 0.02, tmax 256, log-normal sizes (sigma 2)
    sizes = S.user_bin_sizes(13, 1000, S.SIZES_LOG_NORMAL, 60.0, 2.0, 5, 20000)
    offs = S.offsets_of(sizes)
    spec = S.query_spec(13, S.QUERIES_MIXED, 50, 500, 70, 2, 6, 10, 1000)
    qv, qo, thr = S.queries(spec, offs, 0, 300)
    cfg = ref_cfg(1000, h=3, fpr=0.02, tmax=256)
    hibf_case(R, "synth_t256", cfg, None, offs, (qv, qo), thr, thr, widths=(2,), synthetic_seed=13)
    sizes = S.user_bin_sizes(17, 300, S.SIZES_LOG_NORMAL, 200.0, 1.5, 10, 20000)
    offs = S.offsets_of(sizes)
    spec = S.query_spec(17, S.QUERIES_MIXED, 20, 400, 70, 2, 7, 10, 300)
    qv, qo, thr = S.queries(spec, offs, 0, 300)
    cfg = ref_cfg(300, h=2, fpr=0.05, tmax=128)
    hibf_case(R, "synth_t128", cfg, None, offs, (qv, qo), thr, thr, widths=(2, 4), synthetic_seed=17)


def make_ibf_config(R: Reference):
    """interleaved_bloom_filter(config&, max_bin_elements): bin size, bit store digest, counts."""
    out = {}
    cases = []
    # interleaved_bloom_filter_test.cpp:410-431
    cases.append(([[1, 2, 3, 4, 5, 6, 7, 8, 9, 10], [1, 2, 3, 4, 5]], dict(), 0))
    rng = np.random.default_rng(77)
    ubs = [rng.integers(0, 50000, rng.integers(10, 3000)).tolist() for _ in range(40)]  # duplicates and overlaps
    cases.append((ubs, dict(), 0))
    cases.append((ubs, dict(h=3, fpr=0.01), 0))
    cases.append((ubs, dict(sketch_bits=5), 0))
    cases.append((ubs, dict(), 777))
    cases.append((None, dict(h=2, fpr=0.05), 0))
    stream_sizes = rng.integers(100, 20000, 70)
    big = [S.stream_range(i, 0, int(n)).tolist() for i, n in enumerate(stream_sizes)]
    cases[-1] = (big, dict(h=2, fpr=0.05), 0)
    for ci, (ubs, kw, mbe) in enumerate(cases):
        v, o = csr(ubs)
        cfg = ref_cfg(len(ubs), **kw)
        ibf = R.ibf_from_config(cfg, v, o, mbe)
        q = np.concatenate([v[::3], np.arange(60000, 60500, dtype=np.uint64)])
        p_ = f"c{ci}_"
        if ubs is big:
            # user bin i = the first stream_sizes[i] outputs of the splitmix64 stream seeded with i (regenerated)
            out[p_ + "stream_sizes"] = stream_sizes.astype(np.uint64)
        else:
            out[p_ + "values"], out[p_ + "offsets"] = v, o
        out[p_ + "kw"] = np.array([kw.get("h", 2), int(kw.get("fpr", 0.05) * 1e6), kw.get("sketch_bits", 12), mbe],
                                  np.uint64)
        out[p_ + "params"] = np.array([ibf.bins, ibf.bin_size, ibf.hash_funs], np.uint64)
        out[p_ + "digest"] = np.array([digest_words(ibf.words())], np.uint64)
        if ubs is not big:
            out[p_ + "queries"] = q
        out[p_ + "count2"] = ibf.bulk_count(q, 2)
        out[p_ + "member"] = ibf.membership_for(q[:200], 2)
    out["n_cases"] = np.array([len(cases)], np.uint64)
    np.savez_compressed(OUT / "ibf_config.npz", **out)


def make_hll(R: Reference):
    """hyperloglog registers and estimates for a few value sets and widths (src/sketch/hyperloglog.cpp).  Value sets
    are the splitmix64 stream (seed, count: regenerated by the test), 0..n-1, or stored random values."""
    out = {}
    rng = np.random.default_rng(21)
    cases = [("stream", 3, 1000, 12), ("stream", 4, 200000, 12), ("stream", 5, 5, 5), ("random", 0, 30000, 8),
             ("stream", 0, 0, 12), ("arange", 0, 100000, 14), ("stream", 6, 50000, 16)]
    for i, (kind, seed, n, bits) in enumerate(cases):
        if kind == "stream":
            v = S.stream_range(seed, 0, n)
        elif kind == "arange":
            v = np.arange(n, dtype=np.uint64)
        else:
            v = rng.integers(0, 1 << 63, n, dtype=np.uint64)
            out[f"c{i}_values"] = v
        regs, est = R.hll(v, bits)
        out[f"c{i}_source"] = np.array([("stream", "arange", "random").index(kind), seed, n], np.uint64)
        out[f"c{i}_bits"] = np.array([bits], np.uint64)
        out[f"c{i}_registers"] = regs
        out[f"c{i}_estimate"] = np.array([est], np.float64)
    out["n_cases"] = np.array([len(cases)], np.uint64)
    np.savez_compressed(OUT / "hll_cases.npz", **out)


def make_serial(R: Reference):
    """Serialised filters: the reference's serialize functions through cereal's binary encoding (oracle/ref_driver.cpp
    byte archive), for an IBF with occupancy tracking and two HIBFs, with what is needed to rebuild them."""
    # IBF: 130 bins x 1000 rows, h = 3, occupancy tracked; value i of the stream seeded 3 goes to bin i % 130
    ibf = R.ibf(130, 1000, 3, True)
    v = S.stream_range(3, 0, 4000)
    ibf.emplace(v, np.arange(4000, dtype=np.uint64) % np.uint64(130))
    (OUT / "serial_ibf.bin").write_bytes(ibf.save())
    for name, seed in (("snippet", None), ("synth64", 7)):
        d = np.load(OUT / f"hibf_{name}.npz")
        cfg = ref_cfg(int(d["n_user_bins"][0]), h=int(d["config"][0]), fpr=float(d["fpr"][0]),
                      relaxed_fpr=float(d["fpr"][1]), tmax=int(d["config"][1]), sketch_bits=int(d["config"][2]))
        layout = bytes(d["layout"]).decode()
        if seed is None:
            H = R.hibf(cfg, d["ub_values"], d["ub_offsets"], layout=layout)
        else:
            H = R.hibf(cfg, None, d["ub_offsets"], seed=seed, synthetic=True, layout=layout)
        (OUT / f"serial_hibf_{name}.bin").write_bytes(H.save())


def make_c1(R: Reference):
    """The 64-user-bin workload at full size: everything except the bit words (which are 2.9 MB)."""
    sizes = S.user_bin_sizes(1, 64, S.SIZES_LOG_UNIFORM, 0, 0, 1000, 100000)
    offs = S.offsets_of(sizes)
    cfg = ref_cfg(64, h=2, fpr=0.05, tmax=64, threads=1)
    layout = R.layout(cfg, None, offs, seed=1, synthetic=True)
    H = R.hibf(cfg, None, offs, seed=1, synthetic=True)
    T = H.tables(with_words=False)
    spec = S.query_spec(1, S.QUERIES_HALF_ONE_BIN, 250, 250, 0, 0, 1, 2, 64)
    qv, qo, thr = S.queries(spec, offs, 0, 10000)
    res = H.query_batch(qv, qo, thr, thr, threads=8)
    np.savez_compressed(OUT / "c1_reference.npz", ub_offsets=offs, layout=np.frombuffer(layout.encode(), np.uint8),
                        bins=T["bins"], bin_size=T["bin_size"], hash_funs=T["hash_funs"], next_ibf=T["next_ibf"],
                        user_bin=T["user_bin"], digests=T["digests"], thresholds=thr, **res)
    print("c1_reference:", len(T["bins"]), "IBFs")


def make_c3_layout(R: Reference):
    sizes = S.user_bin_sizes(1, 8192, S.SIZES_LOG_NORMAL, 200000.0, 1.5, 1000, 50000000)
    offs = S.offsets_of(sizes)
    cfg = ref_cfg(8192, h=2, fpr=0.05, tmax=64, threads=8, sketch_bits=12)
    t0 = time.time()
    layout = R.layout(cfg, None, offs, seed=1, synthetic=True)
    (OUT / "c3_layout.txt").write_text(layout)
    print(f"c3_layout: {time.time() - t0:.0f}s")


def make_c4_layout(R: Reference, estimate_union=True):
    """The 65,536-user-bin layout (h=3, fpr 0.02, tmax 256): reference DP over HyperLogLog sketches of the
    synthetic user bins, streamed from the generator (about 4.8e10 values; no value is materialised).  With
    estimate_union=False the DP sums user bin sizes instead of estimating unions (config::disable_estimate_union,
    which also disables rearrangement): about an hour of one core.  The union-estimating DP merges sketches for
    every (column, earlier column) pair, ~2e9 union estimates at this size, and does not finish in hours."""
    sizes = S.user_bin_sizes(1, 65536, S.SIZES_LOG_NORMAL, 100000.0, 2.0, 500, 200000000)
    offs = S.offsets_of(sizes)
    cfg = ref_cfg(65536, h=3, fpr=0.02, tmax=256, threads=8, sketch_bits=12,
                  disable_estimate_union=not estimate_union, disable_rearrangement=not estimate_union)
    t0 = time.time()
    layout = R.layout(cfg, None, offs, seed=1, synthetic=True)
    name = "c4_layout.txt" if estimate_union else "c4_layout_sum.txt"
    (OUT / name).write_text(layout)
    print(f"{name}: {time.time() - t0:.0f}s")


def make_ref_build(R: Reference, name: str, scale: float):
    """The reference's own build of a benchmark workload from its committed layout, every user bin at `scale` of its
    size (the same sizes as bench.py --scale), streamed from the generator: its tables (in the reference's IBF
    numbering) and per-IBF digests of the bit words.  The device builds are compared with these by path of merged
    bins (tests/test_build_gpu.py, bench.py).  Full size for 8,192 user bins: 4.9e9 values, 13.4 GB of bit words,
    about 7 minutes on 8 threads."""
    from hibf_gb300.workloads import WORKLOADS

    wl = WORKLOADS[name]
    sizes = S.user_bin_sizes(1, wl.n_user_bins, wl.size_law, wl.size_p0, wl.size_p1, wl.size_lo, wl.size_hi)
    if scale != 1.0:
        sizes = np.maximum(1, np.floor(sizes.astype(np.float64) * scale)).astype(np.uint64)
    offs = S.offsets_of(sizes)
    cfg = ref_cfg(wl.n_user_bins, h=wl.h, fpr=wl.fpr, tmax=wl.tmax, threads=8, sketch_bits=12)
    t0 = time.time()
    H = R.hibf(cfg, None, offs, seed=wl.query.seed, synthetic=True, layout=wl.layout_text())
    T = H.tables(with_words=False)
    tag = {"hibf8192": "c3", "hibf65536": "c4"}[name]
    out = OUT / f"ref_{tag}_{scale:g}.npz"
    np.savez_compressed(out, ub_offsets=offs, scale=np.array([scale]),
                        **{k: T[k] for k in ("bins", "bin_size", "hash_funs", "next_ibf", "user_bin", "digests")})
    print(f"{out.name}: {len(T['bins'])} IBFs, {int(offs[-1])} values, {time.time() - t0:.0f}s")


def make_simple_case(R: Reference):
    # test/unit/hibf/hierarchical_interleaved_bloom_filter_test.cpp:47 simple_user_bins: 73 user bins holding only the
    # value 5 (the reference computes the layout); queries that hit every user bin, some, or none
    ubs = [[5]] * 73
    v, o = csr(ubs)
    q = csr([[5], [5, 6], [6], [5, 5, 5], [6, 7, 8, 5]])
    hibf_case(R, "simple", ref_cfg(73), v, o, q, [1, 2, 1, 3, 2], [1, 1, 1, 2, 1], widths=(1, 2, 8))


def main(argv):
    build_reference()
    R = Reference()
    which = set(argv) or {"ibf", "ibfcfg", "hll", "serial", "hibf", "hibfwide", "dups", "hashes", "empty", "sizing",
                          "simple", "c1", "c3"}
    if "ibf" in which:
        make_ibf_cases(R)
    if "serial" in which:
        make_serial(R)
    if "hll" in which:
        make_hll(R)
    if "hibfwide" in which:
        make_hibf_wide_cases(R)
    if "dups" in which:
        make_dups_case(R)
    if "hashes" in which:
        make_many_hash_cases(R)
    if "empty" in which:
        make_empty_bins_case(R)
    if "sizing" in which:
        make_sizing_cases(R)
    if "ibfcfg" in which:
        make_ibf_config(R)
    if "hibf" in which:
        make_hibf_cases(R)
    if "simple" in which:
        make_simple_case(R)
    if "c1" in which:
        make_c1(R)
    if "c3" in which:
        make_c3_layout(R)
    if "c4" in which:  # not in the default set: far more than hours of CPU
        make_c4_layout(R)
    if "c4sum" in which:  # not in the default set
        make_c4_layout(R, estimate_union=False)
    # the reference's builds of the benchmark workloads (not in the default set: minutes each)
    if "refc3" in which:
        make_ref_build(R, "hibf8192", 1.0)
    if "refc3s" in which:
        make_ref_build(R, "hibf8192", 0.05)
    if "refc4s" in which:
        make_ref_build(R, "hibf65536", 0.02)
    if "refc4m" in which:
        make_ref_build(R, "hibf65536", 0.1)


if __name__ == "__main__":
    main(sys.argv[1:])
