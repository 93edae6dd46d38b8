"""Canonical form of an HIBF's tables: IBFs keyed by their path of merged bins from the root.

The reference numbers lower-level IBFs in a randomised order (HIBF.cpp:111-116); the bits and query results do not
depend on it.  Comparing two builds therefore maps IBFs by path, not by index."""

import numpy as np

MERGED = (1 << 64) - 1


def paths(bins, next_ibf, user_bin):
    bins = [int(b) for b in bins]
    off = np.concatenate([[0], np.cumsum(bins)]).astype(np.int64)
    out = {0: ()}
    stack = [0]
    while stack:
        k = stack.pop()
        for b in range(bins[k]):
            i = off[k] + b
            if int(user_bin[i]) == MERGED:
                c = int(next_ibf[i])
                if c != k and c not in out:
                    out[c] = out[k] + (b,)
                    stack.append(c)
    return out, off


def canonical(t):
    """{path: (bins, bin_size, user_bin row with merged bins as -1)}"""
    p, off = paths(t["bins"], t["next_ibf"], t["user_bin"])
    res = {}
    for k, path in p.items():
        row = np.asarray(t["user_bin"][off[k]:off[k + 1]], dtype=np.uint64).astype(object)
        row = tuple(-1 if int(x) == MERGED else int(x) for x in row)
        res[path] = (int(t["bins"][k]), int(t["bin_size"][k]), row, k)
    return res


def split_free(t, k):
    """True when IBF k stores no user bin across several technical bins."""
    p, off = paths(t["bins"], t["next_ibf"], t["user_bin"])
    row = [int(x) for x in t["user_bin"][off[k]:off[k + 1]]]
    ids = [x for x in row if x != MERGED]
    return len(ids) == len(set(ids))
