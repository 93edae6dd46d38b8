"""The benchmark workloads, by what they are (seeded synthetic data, see include/hibf_gb300_synthetic.h).

hibf64     64 user bins, sizes log-uniform in [1e3, 1e5], h=2, fpr 0.05, tmax 64; 10,000 queries of 250 values, half
           from one user bin, half uniform; threshold 125.
hibf65536  65,536 user bins, sizes log-normal (median 1e5, sigma 2.0) clipped to [500, 2e8] (4.8e10 values), h=3,
           fpr 0.02, tmax 256, layout from the reference's DP with summed user bin sizes (disable_estimate_union,
           which also disables rearrangement; the union-estimating DP needs ~2e9 HyperLogLog union estimates at
           this many user bins); 10,000,000 queries of length U[50, 5000], composition as above; threshold
           ceil(0.6 * length).
hibf8192   8,192 user bins, sizes log-normal (median 2e5, sigma 1.5) clipped to [1e3, 5e7], h=2, fpr 0.05, tmax 64,
           layout from the reference's DP over HyperLogLog sketches (sketch_bits 12); 1,000,000 queries of length
           U[20, 2000], 70% drawn from 1-3 user bins with 2% noise, 30% uniform; threshold ceil(0.7 * length).

Layouts were computed by the reference (tests/golden/make_golden.py) and are read from tests/golden.
"""

from __future__ import annotations

import ctypes
import time
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import _native as N
from . import synthetic as S

GOLDEN = Path(__file__).resolve().parents[1] / "tests" / "golden"


@dataclass
class workload:
    name: str
    n_user_bins: int
    size_law: int
    size_p0: float
    size_p1: float
    size_lo: int
    size_hi: int
    h: int
    fpr: float
    tmax: int
    n_queries: int
    query: S.query_spec
    layout_file: str | None
    split_table_file: str | None = None

    def user_bin_offsets(self) -> np.ndarray:
        off = np.zeros(self.n_user_bins + 1, np.uint64)
        N.call("hibf_gpu_synth_user_bin_offsets", self.query.seed, self.size_law, self.size_p0, self.size_p1,
               self.size_lo, self.size_hi, self.n_user_bins, off.ctypes.data)
        return off

    def layout_text(self) -> str:
        if self.layout_file is None:
            raise FileNotFoundError(f"{self.name}: no layout file")
        p = GOLDEN / self.layout_file
        if p.suffix == ".npz":
            return bytes(np.load(p)["layout"]).decode()
        return p.read_text()

    def split_table(self, offsets: np.ndarray):
        """How the reference chunks the split user bins of this layout for user bins of `offsets`: the committed
        table of the full-size workload when its sizes are these, else a replay of the reference's hash-set
        history (build.split_table.synthetic)."""
        from . import build as B

        if self.split_table_file is not None and (GOLDEN / self.split_table_file).exists():
            a = dict(np.load(GOLDEN / self.split_table_file))
            sizes = np.diff(offsets.astype(np.uint64))
            if a["n_values"].size and np.array_equal(sizes[a["user_bin"].astype(np.int64)], a["n_values"]):
                return B.split_table.from_arrays(a), "committed table (tests/golden/" + self.split_table_file + ")"
        import os

        t0 = time.perf_counter()
        c = B.config(number_of_user_bins=self.n_user_bins, number_of_hash_functions=self.h, maximum_fpr=self.fpr,
                     threads=os.cpu_count() or 1)
        t = B.split_table.synthetic(c, self.layout_text(), self.query.seed, offsets)
        return t, f"replayed on the host in {time.perf_counter() - t0:.1f} s"

    def query_offsets(self, first: int, n: int):
        q = self.query
        qo = np.zeros(n + 1, np.uint64)
        thr = np.zeros(n, np.uint64)
        N.call("hibf_gpu_synth_query_offsets", q.seed, q.law, q.len_lo, q.len_hi, q.mix_pct, q.noise_pct, q.thr_num,
               q.thr_den, q.n_user_bins, first, n, qo.ctypes.data, thr.ctypes.data)
        return qo, thr

    def queries_device(self, d_ub_offsets: int, first: int, n: int, d_qoff: int, d_values: int, stream=None):
        q = self.query
        N.call("hibf_gpu_synth_queries_d", q.seed, q.law, q.len_lo, q.len_hi, q.mix_pct, q.noise_pct, q.thr_num,
               q.thr_den, q.n_user_bins, d_ub_offsets, first, n, d_qoff, d_values, stream)

    def queries_host(self, ub_offsets: np.ndarray, first: int, n: int, qoff: np.ndarray) -> np.ndarray:
        q = self.query
        vals = np.zeros(int(qoff[-1]), np.uint64)
        N.call("hibf_gpu_synth_queries", q.seed, q.law, q.len_lo, q.len_hi, q.mix_pct, q.noise_pct, q.thr_num,
               q.thr_den, q.n_user_bins, ub_offsets.ctypes.data, first, n, qoff.ctypes.data, vals.ctypes.data)
        return vals


HIBF64 = workload("hibf64", 64, S.SIZES_LOG_UNIFORM, 0.0, 0.0, 1000, 100000, 2, 0.05, 64, 10000,
                  S.query_spec(1, S.QUERIES_HALF_ONE_BIN, 250, 250, 0, 0, 1, 2, 64), "c1_reference.npz")
HIBF8192 = workload("hibf8192", 8192, S.SIZES_LOG_NORMAL, 200000.0, 1.5, 1000, 50000000, 2, 0.05, 64, 1000000,
                    S.query_spec(1, S.QUERIES_MIXED, 20, 2000, 70, 2, 7, 10, 8192), "c3_layout.txt",
                    "c3_split_table.npz")

HIBF65536 = workload("hibf65536", 65536, S.SIZES_LOG_NORMAL, 100000.0, 2.0, 500, 200000000, 3, 0.02, 256, 10000000,
                     S.query_spec(1, S.QUERIES_MIXED, 50, 5000, 70, 2, 6, 10, 65536), "c4_layout_sum.txt",
                     "c4_split_table.npz")

WORKLOADS = {w.name: w for w in (HIBF64, HIBF8192, HIBF65536)}
