"""Loading helpers for the golden vectors in tests/golden (written by tests/golden/make_golden.py)."""

from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"

HIBF_CASES = ["snippet", "readme", "three_level", "uneven", "similar", "same", "synth64", "synth600"]


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
