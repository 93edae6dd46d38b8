"""The host part of the build (layout parsing, IBF graph, sizing, tables) against the reference's own builds.

CPU only: hibf_gpu_plan_disjoint computes sizes and tables without a device.  For the synthetic workloads (pairwise
disjoint user bins) every IBF -- matched by its path of merged bins -- must have the reference's bin count, bin size
and bin-to-user-bin table, given the layout the reference computed."""

import numpy as np
import pytest

from hibf_gb300 import build as B
from hibf_gb300 import synthetic as S
from tests import golden_io as G
from tests.hibf_canon import canonical


def _cfg(d):
    h, tmax, sketch = (int(x) for x in d["config"])
    fpr, rfpr, alpha, ratio = (float(x) for x in d["fpr"])
    return B.config(number_of_user_bins=d["n_ub"], number_of_hash_functions=h, maximum_fpr=fpr, relaxed_fpr=rfpr)


@pytest.mark.parametrize("name", ["synth64", "synth600", "synth_t128", "synth_t256", "synth_h1", "synth_h4",
                                  "synth_h5", "empty_bins", "relaxed_fpr", "synth_t512"])
def test_plan_matches_reference_tables(name):
    d = G.hibf_case(name)
    sizes = np.diff(d["ub_offsets"].astype(np.int64)).astype(np.uint64)
    plan = B.plan_disjoint(_cfg(d), d["layout_text"], sizes)
    ref = canonical(G.tables(d))
    got = canonical(plan)
    assert set(ref) == set(got)
    for path in ref:
        assert ref[path][:3] == got[path][:3], path


def test_plan_c1_matches_reference():
    z = np.load(G.GOLDEN / "c1_reference.npz")
    sizes = np.diff(z["ub_offsets"].astype(np.int64)).astype(np.uint64)
    cfg = B.config(number_of_user_bins=64, number_of_hash_functions=2, maximum_fpr=0.05)
    plan = B.plan_disjoint(cfg, bytes(z["layout"]).decode(), sizes)
    ref = canonical(dict(bins=z["bins"], bin_size=z["bin_size"], next_ibf=z["next_ibf"], user_bin=z["user_bin"]))
    got = canonical(plan)
    assert {p: v[:3] for p, v in ref.items()} == {p: v[:3] for p, v in got.items()}


def test_plan_c3_layout():
    """The 8,192-user-bin layout: 606 IBFs over three levels, every user bin placed once."""
    text = (G.GOLDEN / "c3_layout.txt").read_text()
    sizes = S.user_bin_sizes(1, 8192, S.SIZES_LOG_NORMAL, 200000.0, 1.5, 1000, 50000000)
    plan = B.plan_disjoint(B.config(number_of_user_bins=8192), text, sizes)
    assert plan["bins"].size == 606
    ub = plan["user_bin"]
    ids = np.unique(ub[ub < np.uint64(8192)])
    assert ids.size == 8192
    assert int(plan["bins"][0]) == 64


def test_layout_errors():
    with pytest.raises(B.N.InvalidArgument):
        B.plan_disjoint(B.config(number_of_user_bins=2), "no header\n", [1, 1])
    with pytest.raises(B.N.InvalidArgument):
        B.plan_disjoint(B.config(number_of_user_bins=2, maximum_fpr=1.5), "#TOP_LEVEL_IBF fullest_technical_bin_idx:0\n", [1, 1])


def test_config_validation_mirrors_reference():
    c = B.config(input_fn=lambda u, it: None, number_of_user_bins=100)
    c.validate_and_set_defaults()
    assert c.tmax == 64
    c = B.config(input_fn=lambda u, it: None, number_of_user_bins=10, tmax=65)
    c.validate_and_set_defaults()
    assert c.tmax == 128 and c.warnings
    for bad in (dict(number_of_user_bins=0), dict(number_of_user_bins=2, number_of_hash_functions=6),
                dict(number_of_user_bins=2, maximum_fpr=0.0), dict(number_of_user_bins=2, relaxed_fpr=0.01),
                dict(number_of_user_bins=2, threads=0), dict(number_of_user_bins=2, sketch_bits=4),
                dict(number_of_user_bins=2, alpha=-1.0), dict(number_of_user_bins=2, empty_bin_fraction=1.0)):
        with pytest.raises(ValueError):
            B.config(input_fn=lambda u, it: None, **bad).validate_and_set_defaults()
    with pytest.raises(ValueError):
        B.config(number_of_user_bins=2).validate_and_set_defaults()


@pytest.mark.parametrize("case", G.ibf_config_cases(), ids=lambda c: f"ibfcfg{c['index']}")
def test_ibf_plan_matches_reference(case):
    """interleaved_bloom_filter(config&, max_bin_elements): the bin size the reference chose -- from the biggest user
    bin by HyperLogLog estimate (then counted exactly), or from max_bin_elements -- on the host, no device."""
    ubs = case["user_bins"]
    cfg = B.config(input_fn=lambda ub, it: it.push(ubs[ub]), **case["config"])
    size, _biggest = B.ibf_plan(cfg, case["max_bin_elements"])
    assert size == int(case["params"][1])


def _ub_values(d):
    if "ub_values" in d:
        v, o = d["ub_values"], d["ub_offsets"].astype(np.int64)
        return [v[o[u]:o[u + 1]] for u in range(o.size - 1)]
    seed = int(d["synthetic_seed"][0])
    return [S.user_bin_values(seed, d["ub_offsets"], u) for u in range(d["n_ub"])]


def test_bin_size_in_bits_known_answers():
    """include/hibf/build/bin_size_in_bits.hpp through the IBF sizing (test/unit/hibf/build/bin_size_in_bits_test.cpp
    :11-19): 1,000 elements at fpr 0.05 with two hash functions take 7,903 bits; user bins without elements, 0."""
    cfg = B.config(input_fn=lambda ub, it: None, number_of_user_bins=3, number_of_hash_functions=2, maximum_fpr=0.05)
    assert B.ibf_plan(cfg, max_bin_elements=1000)[0] == 7903
    cfg = B.config(input_fn=lambda ub, it: None, number_of_user_bins=3, number_of_hash_functions=1, maximum_fpr=0.05)
    assert B.ibf_plan(cfg)[0] == 0  # every user bin empty: the largest holds no element


@pytest.mark.parametrize("name", ["snippet", "readme", "three_level", "uneven", "similar", "same", "synth64",
                                  "synth600", "synth_t128", "synth_t256", "dups", "synth_h1", "synth_h4",
                                  "synth_h5", "empty_bins", "relaxed_fpr", "synth_t512"])
def test_insertion_order_reproduces_reference_bits(oracle, name):
    """Every IBF's bit store, split user bins included, rebuilt on the CPU oracle from the builder's insertion order
    (split user bins in the replayed hash-set order) and the reference's own tables, equals the reference's words."""
    d = G.hibf_case(name)
    ubs = _ub_values(d)
    h = int(d["hash_funs"][0])
    fpr, rfpr, _, _ = (float(x) for x in d["fpr"])
    cfg = B.config(input_fn=lambda u, it: it.push(ubs[u]), number_of_user_bins=d["n_ub"],
                   number_of_hash_functions=h, maximum_fpr=fpr, relaxed_fpr=rfpr)
    offs, vals = B.build_inputs(cfg, d["layout_text"])
    T = G.tables(d)
    bins = T["bins"].astype(np.int64)
    tb_off = np.concatenate([[0], np.cumsum(bins)])
    nxt, ub = T["next_ibf"], T["user_bin"]
    ibfs = [oracle.ibf(int(bins[k]), int(T["bin_size"][k]), h) for k in range(bins.size)]
    # parent (IBF, merged bin) of every non-root IBF
    parent = {}
    for k in range(bins.size):
        for tb in range(int(bins[k])):
            c = int(nxt[tb_off[k] + tb])
            if ub[tb_off[k] + tb] == np.uint64(2**64 - 1) and c != k:  # merged bin -> child IBF
                parent[c] = (k, tb)
    leaf = {}
    for k in range(bins.size):
        for tb in range(int(bins[k])):
            u = int(ub[tb_off[k] + tb])
            if u < d["n_ub"]:
                leaf.setdefault(u, (k, []))[1].append(tb)
    for u in range(d["n_ub"]):
        v = vals[offs[u]:offs[u + 1]]
        k, tbs = leaf[u]
        first, ntb = min(tbs), len(tbs)
        chunk = -(-v.size // ntb) if v.size else 1
        for c in range(ntb):
            part = v[c * chunk:(c + 1) * chunk]
            if part.size:
                ibfs[k].emplace(part, first + c)
        while k in parent:
            k, tb = parent[k]
            if v.size:
                ibfs[k].emplace(v, tb)
    for k in range(bins.size):
        assert S.digest(ibfs[k].words().tolist()) == int(d["digests"][k]), f"IBF {k}"


@pytest.mark.parametrize("name", ["snippet", "readme", "three_level", "uneven", "similar", "same", "synth64",
                                  "synth600", "synth_t128", "synth_t256", "dups", "synth_h1", "synth_h4",
                                  "synth_h5", "empty_bins", "relaxed_fpr", "synth_t512"])
def test_split_table_places_values_like_the_reference_order(name):
    """The split table (per split user bin: the set's multiplier and mask, and at each chunk boundary the home slot
    and the values of that slot ranked before it) places every value of every split user bin in the chunk the full
    replayed hash-set order gives it; for the synthetic user bins the table of the streamed replay is the same."""
    d = G.hibf_case(name)
    ubs = _ub_values(d)
    fpr, rfpr, _, _ = (float(x) for x in d["fpr"])
    kw = dict(number_of_user_bins=d["n_ub"], number_of_hash_functions=int(d["hash_funs"][0]), maximum_fpr=fpr,
              relaxed_fpr=rfpr)
    offs, vals = B.build_inputs(B.config(input_fn=lambda u, it: it.push(ubs[u]), **kw), d["layout_text"])
    table = B.split_table.inputs(B.config(input_fn=lambda u, it: it.push(ubs[u]), **kw), d["layout_text"])
    a = table.arrays()
    assert a["user_bin"].size > 0
    for i, u in enumerate(a["user_bin"]):
        v = vals[offs[u]:offs[u + 1]]
        assert int(a["n_values"][i]) == v.size
        got = table.chunks(int(u), v)
        # the reference order puts position p in chunk p // ceil(n / technical bins); compare chunk by chunk
        lay_ntb = _technical_bins(d, int(u))
        want = np.arange(v.size, dtype=np.uint64) // np.uint64(-(-v.size // lay_ntb) if v.size else 1)
        np.testing.assert_array_equal(got, want, err_msg=f"user bin {u}")
    if "synthetic_seed" in d:
        t2 = B.split_table.synthetic(B.config(**kw), d["layout_text"], int(d["synthetic_seed"][0]), d["ub_offsets"])
        b = t2.arrays()
        for k in a:
            np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    # an imported copy answers the same
    t3 = B.split_table.from_arrays(a)
    u = int(a["user_bin"][0])
    np.testing.assert_array_equal(t3.chunks(u, vals[offs[u]:offs[u + 1]]), table.chunks(u, vals[offs[u]:offs[u + 1]]))


def _technical_bins(d, u):
    T = G.tables(d)
    return int(np.count_nonzero(T["user_bin"] == np.uint64(u)))


@pytest.mark.gpu
def test_split_table_rejects_a_table_of_other_sizes(gpu_lib):
    d = G.hibf_case("synth64")
    kw = dict(number_of_user_bins=d["n_ub"], number_of_hash_functions=int(d["hash_funs"][0]),
              maximum_fpr=float(d["fpr"][0]), relaxed_fpr=float(d["fpr"][1]))
    a = B.split_table.synthetic(B.config(**kw), d["layout_text"], int(d["synthetic_seed"][0]),
                                d["ub_offsets"]).arrays()
    a["n_values"] = a["n_values"].copy()
    a["n_values"][0] += 1
    bad = B.split_table.from_arrays(a)
    with pytest.raises(B.N.InvalidArgument):
        B.build_synthetic(B.config(**kw), d["layout_text"], int(d["synthetic_seed"][0]), d["ub_offsets"], bad)
