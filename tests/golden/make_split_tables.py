"""Split tables of the full-size benchmark workloads (8,192 and 65,536 user bins).

The reference chunks a user bin that it splits over several technical bins in its hash set's iteration order
(src/build/insert_into_ibf.cpp:28-47), which depends on the history of the sets in hierarchical_build
(src/hierarchical_interleaved_bloom_filter.cpp:39-171).  This library replays that history on a restatement of the
set (hibf_gb300/csrc/rh_set.hpp) and keeps only what places each value (include/hibf_gb300.h, hibf_gpu_split_table_*).
At full size the replay inserts 3.5e9 (8,192 user bins) and 2.8e10 (65,536 user bins) values into host hash sets,
minutes of all host cores, so the tables are computed once here and committed; bench.py imports them, and the
synthetic build checks that a table belongs to the layout and user bin sizes it is given.

These are outputs of this library's replay, not of the reference: the replay is pinned against the reference's own
builds by tests/test_build_plan.py (every golden HIBF) and, at the workloads' shapes, by the per-IBF digests of the
reference's own builds in tests/golden/ref_c3_*.npz and ref_c4_*.npz (make_golden.py refc3 / refc3s / refc4s; the
full-size 8,192-user-bin index is compared IBF by IBF in bench.py, the scaled ones in tests/test_build_gpu.py).

    python tests/golden/make_split_tables.py [hibf8192] [hibf65536]
"""

from __future__ import annotations

import os
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from hibf_gb300 import build as B  # noqa: E402
from hibf_gb300.workloads import WORKLOADS  # noqa: E402

OUT = Path(__file__).resolve().parent


def make(name: str) -> None:
    wl = WORKLOADS[name]
    offs = wl.user_bin_offsets()
    cfg = B.config(number_of_user_bins=wl.n_user_bins, number_of_hash_functions=wl.h, maximum_fpr=wl.fpr,
                   threads=os.cpu_count() or 1)
    t0 = time.time()
    a = B.split_table.synthetic(cfg, wl.layout_text(), wl.query.seed, offs).arrays()
    dt = time.time() - t0
    np.savez_compressed(OUT / wl.split_table_file, **a)
    print(f"{wl.split_table_file}: {a['user_bin'].size} split user bins, {a['bnd_home'].size} boundaries, "
          f"{a['before'].size} values before boundaries, {dt:.0f} s")


if __name__ == "__main__":
    for n in sys.argv[1:] or ["hibf8192", "hibf65536"]:
        make(n)
