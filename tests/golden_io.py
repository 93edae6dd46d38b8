"""Loading helpers for the golden vectors in tests/golden (written by tests/golden/make_golden.py)."""

from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"

HIBF_CASES = ["snippet", "readme", "three_level", "uneven", "similar", "same", "synth64", "synth600", "synth_t128",
              "synth_t256", "dups", "synth_h1", "synth_h4", "synth_h5", "empty_bins", "relaxed_fpr", "synth_t512",
              "simple"]


def ibf_cases():
    z = np.load(GOLDEN / "ibf_cases.npz")
    n = int(z["n_cases"][0])
    out = []
    for i in range(n):
        p = f"c{i}_"
        d = {k[len(p):]: z[k] for k in z.files if k.startswith(p)}
        d["index"] = i
        out.append(d)
    return out


def hibf_case(name):
    z = np.load(GOLDEN / f"hibf_{name}.npz")
    d = {k: z[k] for k in z.files}
    bins = d["bins"].astype(np.int64)
    sizes = d["bin_size"].astype(np.int64)
    nw = (bins + 63) // 64 * sizes
    off = np.concatenate([[0], np.cumsum(nw)])
    d["word_list"] = [d["words"][off[k]:off[k + 1]] for k in range(bins.size)]
    d["layout_text"] = bytes(d["layout"]).decode()
    d["n_ub"] = int(d["n_user_bins"][0])
    return d


def queries(d):
    qv, qo = d["q_values"], d["q_offsets"]
    return [qv[qo[i]:qo[i + 1]] for i in range(qo.size - 1)]


def mem_lists(d, key="mem_sorted"):
    mo = d["mem_offsets"]
    return [d[key][mo[i]:mo[i + 1]] for i in range(mo.size - 1)]


def tables(d):
    return dict(n_user_bins=d["n_ub"], bins=d["bins"], bin_size=d["bin_size"], hash_funs=d["hash_funs"],
                next_ibf=d["next_ibf"], user_bin=d["user_bin"], words=d["word_list"])


def ibf_config_cases():
    """interleaved_bloom_filter(config&, max_bin_elements) cases; user bins as lists, kw as config fields."""
    from hibf_gb300 import synthetic as S

    z = np.load(GOLDEN / "ibf_config.npz")
    out = []
    for i in range(int(z["n_cases"][0])):
        p = f"c{i}_"
        d = {k[len(p):]: z[k] for k in z.files if k.startswith(p)}
        if "stream_sizes" in d:  # user bin u = the first n_u outputs of the splitmix64 stream seeded with u
            ubs = [S.stream_range(u, 0, int(n)) for u, n in enumerate(d["stream_sizes"])]
            v = np.concatenate(ubs).astype(np.uint64)
            d["queries"] = np.concatenate([v[::3], np.arange(60000, 60500, dtype=np.uint64)])
        else:
            v, o = d["values"], d["offsets"].astype(np.int64)
            ubs = [v[o[u]:o[u + 1]] for u in range(o.size - 1)]
        h, fpr_ppm, sketch, mbe = (int(x) for x in d["kw"])
        d["user_bins"] = ubs
        d["config"] = dict(number_of_user_bins=len(ubs), number_of_hash_functions=h, maximum_fpr=fpr_ppm / 1e6,
                           sketch_bits=sketch)
        d["max_bin_elements"] = mbe
        d["index"] = i
        out.append(d)
    return out


def c1_reference():
    """The 64-user-bin workload as the reference built and queried it (make_golden.py make_c1): tables, per-IBF
    digests and, for 10,000 queries of 250 values at threshold 125, membership_for + sort_results and
    counting_agent<uint16_t>::bulk_count summarised per query (mem_len, mem_digest, cnt_nnz, cnt_digest)."""
    from hibf_gb300 import synthetic as S

    z = np.load(GOLDEN / "c1_reference.npz")
    d = {k: z[k] for k in z.files}
    d["layout_text"] = bytes(d["layout"]).decode()
    d["n_ub"] = 64
    spec = S.query_spec(1, S.QUERIES_HALF_ONE_BIN, 250, 250, 0, 0, 1, 2, 64)
    d["q_values"], d["q_offsets"], thr = S.queries(spec, d["ub_offsets"], 0, 10000)
    assert np.array_equal(thr, d["thresholds"])
    return d


def fold_digests(offsets, *columns):
    """Per segment [offsets[i], offsets[i+1]) the hg_digest_step fold over its rows, each row contributing its
    columns in order (the per-query summaries of the reference driver's ref_hibf_query_batch)."""
    from hibf_gb300 import synthetic as S

    offsets = np.asarray(offsets, dtype=np.int64)
    n = offsets.size - 1
    d = np.full(n, S.DIGEST_INIT, np.uint64)
    lens = np.diff(offsets)
    for j in range(int(lens.max()) if n else 0):
        sel = np.nonzero(lens > j)[0]
        pos = offsets[sel] + j
        for c in columns:
            d[sel] = S.digest_step_np(d[sel], np.asarray(c)[pos].astype(np.uint64))
    return d, lens.astype(np.uint64)


def oracle_hibf_from_inputs(oracle, t, offs, vals):
    """The C oracle's HIBF with tables `t` (the reference's numbering) filled from the builder's insertion order
    (user bin u = vals[offs[u]:offs[u+1]], split user bins in chunk order): each user bin into its own technical
    bins in chunks of ceil(n / bins), and whole into the merged bin of every ancestor IBF."""
    bins = np.asarray(t["bins"]).astype(np.int64)
    tb_off = np.concatenate([[0], np.cumsum(bins)])
    nxt, ub = t["next_ibf"], t["user_bin"]
    O = oracle.hibf({k: t[k] for k in ("n_user_bins", "bins", "bin_size", "hash_funs", "next_ibf", "user_bin")})
    parent, leaf = {}, {}
    for k in range(bins.size):
        for tb in range(int(bins[k])):
            c, u = int(nxt[tb_off[k] + tb]), int(ub[tb_off[k] + tb])
            if u == 2**64 - 1 and c != k:
                parent[c] = (k, tb)
            elif u < 2**64 - 2:
                leaf.setdefault(u, (k, []))[1].append(tb)
    for u in range(offs.size - 1):
        v = vals[int(offs[u]):int(offs[u + 1])]
        k, tbs = leaf[u]
        first, ntb = min(tbs), len(tbs)
        chunk = -(-v.size // ntb) if v.size else 1
        for c in range(ntb):
            part = v[c * chunk:(c + 1) * chunk]
            if part.size:
                O.emplace(k, part, first + c)
        while k in parent:
            k, tb = parent[k]
            if v.size:
                O.emplace(k, v, tb)
    return O
