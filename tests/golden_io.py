"""Loading helpers for the golden vectors in tests/golden (written by tests/golden/make_golden.py)."""

from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"

HIBF_CASES = ["snippet", "readme", "three_level", "uneven", "similar", "same", "synth64", "synth600", "synth_t128",
              "synth_t256", "dups", "synth_h1", "synth_h4", "synth_h5", "empty_bins", "relaxed_fpr", "synth_t512"]


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
