"""Seeded synthetic workloads -- the Python statement of include/hibf_gb300_synthetic.h.

User bin i holds positions [offset_i, offset_i + n_i) of one splitmix64 stream seeded with the workload seed, so all
values of all user bins are pairwise distinct.  Sizes come from a second stream (log-uniform or log-normal, clipped);
queries each have their own splitmix64 state.  The C header, the CUDA generator and this module must agree; the
tests check that.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

M64 = (1 << 64) - 1
GAMMA = 0x9E3779B97F4A7C15
TAG_SIZES = 0x53495A4553
TAG_QUERIES = 0x5155455259
DIGEST_INIT = 0x6A09E667F3BCC908

SIZES_LOG_UNIFORM = 0
SIZES_LOG_NORMAL = 1
QUERIES_HALF_ONE_BIN = 0
QUERIES_MIXED = 1


def mix64(z: int) -> int:
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


def mix64_np(z: np.ndarray) -> np.ndarray:
    z = np.asarray(z, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def stream_at(seed: int, k: int) -> int:
    return mix64((seed + (k + 1) * GAMMA) & M64)


def stream_range(seed: int, start: int, n: int) -> np.ndarray:
    """Outputs start .. start+n-1 of the stream seeded with `seed`."""
    k = np.arange(start + 1, start + n + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        s = np.uint64(seed) + k * np.uint64(GAMMA)
    return mix64_np(s)


def subseed(seed: int, tag: int) -> int:
    return mix64(seed ^ mix64(tag))


def unit(x: int) -> float:
    return (x >> 11) * (1.0 / 9007199254740992.0)


def digest_step_np(h: np.ndarray, x: np.ndarray) -> np.ndarray:
    """hg_digest_step elementwise."""
    with np.errstate(over="ignore"):
        return mix64_np(h ^ mix64_np(x + np.uint64(GAMMA)))


def digest(values) -> int:
    h = DIGEST_INIT
    for x in values:
        h = mix64(h ^ mix64((int(x) + GAMMA) & M64))
    return h


def user_bin_sizes(seed: int, n: int, law: int, p0: float, p1: float, lo: int, hi: int) -> np.ndarray:
    s = subseed(seed, TAG_SIZES)
    out = np.zeros(n, np.uint64)
    for i in range(n):
        if law == SIZES_LOG_UNIFORM:
            u = unit(stream_at(s, i))
            v = math.floor(math.exp(math.log(lo) + u * (math.log(hi) - math.log(lo))))
        else:
            u1 = 1.0 - unit(stream_at(s, 2 * i))
            u2 = unit(stream_at(s, 2 * i + 1))
            z = math.sqrt(-2.0 * math.log(u1)) * math.cos(6.283185307179586 * u2)
            v = math.floor(math.exp(math.log(p0) + p1 * z))
        out[i] = int(min(max(v, lo), hi))
    return out


def offsets_of(sizes: np.ndarray) -> np.ndarray:
    off = np.zeros(len(sizes) + 1, np.uint64)
    np.cumsum(sizes, out=off[1:])
    return off


def user_bin_values(seed: int, offsets: np.ndarray, b: int) -> np.ndarray:
    return stream_range(seed, int(offsets[b]), int(offsets[b + 1] - offsets[b]))


@dataclass
class query_spec:
    seed: int
    law: int
    len_lo: int
    len_hi: int
    mix_pct: int
    noise_pct: int
    thr_num: int
    thr_den: int
    n_user_bins: int


class _rng:
    __slots__ = ("s",)

    def __init__(self, s: int):
        self.s = s

    def next(self) -> int:
        self.s = (self.s + GAMMA) & M64
        return mix64(self.s)


def query_state(q: query_spec, qi: int) -> int:
    return mix64(subseed(q.seed, TAG_QUERIES) ^ mix64(qi + 1))


def query_length(q: query_spec, qi: int) -> int:
    r = _rng(query_state(q, qi)).next()
    if q.law == QUERIES_HALF_ONE_BIN or q.len_hi <= q.len_lo:
        return q.len_lo
    return q.len_lo + r % (q.len_hi - q.len_lo + 1)


def query_threshold(q: query_spec, length: int) -> int:
    return (q.thr_num * length + q.thr_den - 1) // q.thr_den


def query_values(q: query_spec, offsets: np.ndarray, qi: int) -> np.ndarray:
    g = _rng(query_state(q, qi))
    r0 = g.next()
    length = q.len_lo
    if q.law != QUERIES_HALF_ONE_BIN and q.len_hi > q.len_lo:
        length = q.len_lo + r0 % (q.len_hi - q.len_lo + 1)
    out = np.zeros(length, np.uint64)
    if q.law == QUERIES_HALF_ONE_BIN:
        if qi % 2 == 0:
            b = g.next() % q.n_user_bins
            nb = int(offsets[b + 1] - offsets[b])
            for k in range(length):
                out[k] = stream_at(q.seed, int(offsets[b]) + g.next() % nb)
        else:
            for k in range(length):
                out[k] = g.next()
        return out
    if g.next() % 100 < q.mix_pct:
        m = 1 + g.next() % 3
        bins = [g.next() % q.n_user_bins for _ in range(m)]
        for k in range(length):
            if g.next() % 100 < q.noise_pct:
                out[k] = g.next()
            else:
                b = bins[g.next() % m]
                nb = int(offsets[b + 1] - offsets[b])
                out[k] = stream_at(q.seed, int(offsets[b]) + g.next() % nb)
    else:
        for k in range(length):
            out[k] = g.next()
    return out


def queries(q: query_spec, offsets: np.ndarray, first: int, n: int):
    """(values, query_offsets, thresholds) for queries first .. first+n-1 (pure Python; small batches only)."""
    vals = [query_values(q, offsets, first + i) for i in range(n)]
    qoff = np.zeros(n + 1, np.uint64)
    np.cumsum([v.size for v in vals], out=qoff[1:])
    thr = np.array([query_threshold(q, v.size) for v in vals], np.uint64)
    return (np.concatenate(vals) if vals else np.zeros(0, np.uint64)), qoff, thr


# -- single-level IBF workload (hg_ibf_bin_value / hg_ibf_query_value) --------------------------------------------
TAG_IBF_QUERIES = 0x4942465155


def ibf_bin_values(seed: int, values_per_bin: int, b: int, first: int = 0, n: int | None = None) -> np.ndarray:
    """Values first .. first+n-1 of bin b."""
    n = values_per_bin - first if n is None else n
    return stream_range(seed, b * values_per_bin + first, n)


def ibf_query_values(seed: int, n_bins: int, values_per_bin: int, first: int, n: int) -> np.ndarray:
    qs = subseed(seed, TAG_IBF_QUERIES)
    k = 2 * np.arange(first, first + n, dtype=np.uint64)
    with np.errstate(over="ignore"):
        r = mix64_np(np.uint64(qs) + (k + np.uint64(1)) * np.uint64(GAMMA))
        r2 = mix64_np(np.uint64(qs) + (k + np.uint64(2)) * np.uint64(GAMMA))
        b = (r >> np.uint64(1)) % np.uint64(n_bins)
        j = r2 % np.uint64(values_per_bin)
        present = mix64_np(np.uint64(seed) + (b * np.uint64(values_per_bin) + j + np.uint64(1)) * np.uint64(GAMMA))
    return np.where((r & np.uint64(1)).astype(bool), present, r2)
