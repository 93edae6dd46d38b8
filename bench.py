#!/usr/bin/env python
"""bench.py -- HIBF query throughput on GB300 (batched persistent launch vs plain per-query launches).

Default workload (hibf8192): 8,192 user bins (log-normal sizes, median 2e5, sigma 1.5, clipped [1e3, 5e7]; 4.9e9
values; layout from the reference's DP), h=2, fpr 0.05, tmax 64; one step = membership_for + sort_results for
1,000,000 queries of length U[20, 2000] (70% from 1-3 user bins with 2% noise, 30% uniform), threshold
ceil(0.7 * length).  Inputs (8 GB of query values) and the index (13.4 GB) are both larger than L2.  The index is
the reference's filter: split user bins are chunked in the reference's hash-set order (committed split table), and
every IBF is compared with the reference's own build of the same workload (tests/golden/ref_c3_1.npz).  A sub-record
measures the 65,536-user-bin workload the same way (--no-c4 skips it), another the single-level 1,024-bin IBF
(bulk_count + bulk_contains over 2^24 values, --workload ibf1024; --no-c2 skips it).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload hibf8192|...]

Prints one JSON line (rank 0).  Under torchrun each rank holds its own replica and answers the full batch
(replicas only, weak scaling); the step time is the maximum over ranks.  The compact `parity` object is the line's
last key.
"""

from __future__ import annotations

import argparse
import gc
import json
import os
import platform
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
GOLDEN = ROOT / "tests" / "golden"

METRIC = "HIBF query values/s on 1 GB300, batched vs plain (bit-exact); p99 serve latency"
WORKLOAD_DESC = {
    "hibf8192": "HIBF 8,192 user bins (log-normal median 2e5 sigma 1.5, [1e3,5e7]), h=2, fpr 0.05, tmax 64; "
                "1e6 queries len U[20,2000] (70% from 1-3 UBs, 2% noise), t=ceil(0.7 len); membership_for",
    "hibf65536": "HIBF 65,536 user bins (log-normal median 1e5 sigma 2.0, [500,2e8]), h=3, fpr 0.02, tmax 256, "
                 "layout from the reference's DP with summed sizes; 1e6 of 1e7 queries per step, len U[50,5000] "
                 "(70% from 1-3 UBs, 2% noise), t=ceil(0.6 len); membership_for",
    "hibf64": "HIBF 64 user bins (log-uniform [1e3,1e5]), h=2, fpr 0.05, tmax 64; 10,000 queries of 250 values "
              "(half from one UB), t=125; membership_for",
}
WORKLOAD_DESC["ibf1024"] = ("IBF 1,024 bins x 2^26 bits (8 GiB), h=3, emplace of 5e6 uniform values per bin; "
                             "bulk_contains + bulk_count<uint16> over 2^24 query values, 50% present in a random bin")
IBF1024 = dict(bins=1024, bin_size=1 << 26, h=3, values_per_bin=5_000_000, n_queries=1 << 24, seed=1)
REASON_KEYS = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
REF_TAG = {"hibf8192": "c3", "hibf65536": "c4"}


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["hibf8192", "hibf64", "hibf65536", "ibf1024"], default="hibf8192")
    ap.add_argument("--queries", type=int, default=0, help="override the number of queries per step")
    ap.add_argument("--plain-queries", type=int, default=2000, help="queries timed in the plain form")
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="CPU baseline sample budget")
    ap.add_argument("--e2e-steps", type=int, default=0, help="steps of the end-to-end measurement (0: --steps)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-c4", action="store_true", help="skip the 65,536-user-bin sub-record")
    ap.add_argument("--no-c2", action="store_true", help="skip the single-level 1,024-bin IBF sub-record")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default kernel schedule")
    ap.add_argument("--tuning", type=str, default="",
                    help="fixed kernel schedule 'values_per_lane,fetch_bytes,counter_bits[,adaptive_step,ee_min"
                         "[,schedule]]' (skips the autotuner; the optional fields select the adaptive early exit and "
                         "the task schedule: 0 work queue, 1 level by level)")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned scheduler measurement")
    ap.add_argument("--sched-queries", type=int, default=20000, help="batch size of the learned scheduler test")
    ap.add_argument("--tune-queries", type=int, default=200_000, help="sample batch of the autotuner")
    ap.add_argument("--l2-fetch", type=int, default=-1,
                    help="set the context's L2 fetch granularity hint (bytes) before the run; -1 leaves it")
    ap.add_argument("--scale", type=float, default=1.0,
                    help="scale every user bin's size (same layout); < 1 gives a smaller index for profiling")
    return ap.parse_args()


# ------------------------------------------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 20 ms while running."""

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.file = None

    def start(self):
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "20"], stdout=self.file,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        time.sleep(0.1)
        self.proc.terminate()
        self.proc.wait()
        self.file.seek(0)
        rows = [r.strip().split(",") for r in self.file.read().splitlines() if r.strip()]
        os.unlink(self.file.name)
        sm, mx, reasons = [], [], set()
        for r in rows:
            if len(r) < 8:
                continue
            try:
                sm.append(float(r[0]))
                mx.append(float(r[1]))
            except ValueError:
                continue
            for k, v in zip(REASON_KEYS, r[4:8]):
                if v.strip().lower() == "active":
                    reasons.add(k)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_per_value_visit(workload="hibf8192"):
    """DRAM bytes per executed (value, IBF) visit of the query kernel (per query value of a step for the single-level
    IBF) from the committed ncu summary, if present."""
    p = ROOT / "profiles" / "traffic.txt"
    if not p.exists():
        return None
    if workload == "ibf1024":
        key = "k_bulk_bytes_per_value_ibf1024="
    else:
        key = "k_query_bytes_per_value_visit" + ("" if workload == "hibf8192" else "_" + workload) + "="
    for line in p.read_text().splitlines():
        if line.startswith(key):
            return float(line.split("=", 1)[1])
    return None


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def host_ram_bytes():
    try:
        return os.sysconf("SC_PAGE_SIZE") * os.sysconf("SC_PHYS_PAGES")
    except (ValueError, OSError):
        return 1 << 40


def scaled(offs: np.ndarray, scale: float) -> np.ndarray:
    if scale == 1.0:
        return offs
    sizes = np.maximum(1, np.floor(np.diff(offs.astype(np.float64)) * scale)).astype(np.uint64)
    out = np.zeros(sizes.size + 1, np.uint64)
    np.cumsum(sizes, out=out[1:])
    return out


def config_of(wl, nq, nv, n_ibfs, scale, world) -> dict:
    """The workload as both arms name it (the reference arm's line carries the same dict)."""
    return {"workload": WORKLOAD_DESC[wl.name], "name": wl.name, "n_user_bins": wl.n_user_bins,
            "queries_per_step": nq, "values_per_step": nv, "n_ibfs": n_ibfs, "parallelism": f"replicas x{world}",
            "size_scale": scale, "l2": "inputs (values) and the index are larger than L2; no flush"}


def value_inserts(layout_text: str, offs: np.ndarray) -> int:
    """Inserted (value, IBF) pairs of a build: every value into its own IBF and every ancestor's merged bin."""
    n = 0
    for line in layout_text.splitlines():
        if not line or line[0] in "#@":
            continue
        idx, bins, _ = line.split("\t")
        u = int(idx)
        n += int(offs[u + 1] - offs[u]) * len(bins.split(";"))
    return n


def reference_build(wl, scale):
    """The reference's own build of this workload at this scale (tables and per-IBF digests), if committed."""
    if wl.name not in REF_TAG:
        return None
    p = GOLDEN / f"ref_{REF_TAG[wl.name]}_{scale:g}.npz"
    return dict(np.load(p)) if p.exists() else None


def index_vs_reference(hibf, wl, scale, offs):
    """Every IBF of the device index (matched by path of merged bins) against the reference's own build's digest."""
    from hibf_gb300.hibf import ibf_paths

    ref = reference_build(wl, scale)
    if ref is None or not np.array_equal(ref["ub_offsets"], offs):
        return {"index_reference": "no committed reference build of this workload at this scale"}
    got = hibf.digests()
    t = hibf.tables()
    mine = ibf_paths(t["bins"], t["next_ibf"], t["user_bin"])
    theirs = ibf_paths(ref["bins"], ref["next_ibf"], ref["user_bin"])
    equal = sum(1 for p, k in theirs.items() if p in mine and int(got[mine[p]]) == int(ref["digests"][k]))
    return {"index_ibfs": len(theirs), "index_ibfs_equal_reference": equal,
            "index_equals_reference": equal == len(theirs) == len(mine),
            "index_reference": f"tests/golden/ref_{REF_TAG[wl.name]}_{scale:g}.npz (reference build, per-IBF digests)"}


def build_index(wl, scale=1.0):
    """The reference's filter on the device: the workload's layout, user bins from the generator, split user bins
    chunked by the committed (or replayed) split table.  Returns (hibf, offsets, build record)."""
    from hibf_gb300 import build as B

    offs = scaled(wl.user_bin_offsets(), scale)
    t0 = time.perf_counter()
    table, table_note = wl.split_table(offs)
    t_table = time.perf_counter() - t0
    cfg = B.config(number_of_user_bins=wl.n_user_bins, number_of_hash_functions=wl.h, maximum_fpr=wl.fpr)
    t0 = time.perf_counter()
    hibf = B.build_synthetic(cfg, wl.layout_text(), wl.query.seed, offs, table)
    build_s = time.perf_counter() - t0
    ins = value_inserts(wl.layout_text(), offs)
    rec = {"seconds": build_s, "values": int(offs[-1]), "value_inserts": ins, "inserts_per_s": ins / build_s,
           "algorithmic_GBps": ins * wl.h * 64 / build_s / 1e9, "bytes_per_insert": wl.h * 64,
           "split_table": table_note, "split_table_s": t_table,
           "form": "hibf_gpu_hibf_build_synthetic: host plan, values generated on the device, atomicOr inserts; "
                   "the time includes planning and allocating the store"}
    return hibf, offs, rec


def oracle_from_device(hibf):
    """The C oracle holding the device-built bit store (downloaded in place)."""
    from hibf_gb300 import _native as N
    from oracle.bindings import Oracle, build_oracle

    build_oracle()
    OH = Oracle().hibf(hibf.tables())
    for k in range(hibf.n_ibfs):
        addr, n = OH.data_ptr(k)
        N.call("hibf_gpu_hibf_download_words", hibf._h, k, addr, n)
    return OH


def _mix64(z):
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def _digest_step(h, x):
    return _mix64(h ^ _mix64(x + np.uint64(0x9E3779B97F4A7C15)))


def count_digests(offs, ids, cnts):
    """Per query the digest of its non-zero (user bin, count) pairs in ascending user bin order, as the oracle's
    orc_hibf_query_batch forms it (hg_digest_step over ub then count, include/hibf_gb300_synthetic.h)."""
    nq = offs.size - 1
    d = np.full(nq, 0x6A09E667F3BCC908, np.uint64)
    lens = np.diff(offs).astype(np.int64)
    with np.errstate(over="ignore"):
        for j in range(int(lens.max()) if nq else 0):
            sel = np.nonzero(lens > j)[0]
            pos = offs[sel].astype(np.int64) + j
            d[sel] = _digest_step(_digest_step(d[sel], ids[pos]), cnts[pos].astype(np.uint64))
    return d, lens.astype(np.uint64)


def cpu_sample(OH, qgen, budget_s, threads, first=0, n_total=None):
    """Times the oracle's membership_for + sort_results on a bounded sample of the workload's queries; qgen(first, n)
    returns (values, query offsets, thresholds)."""
    probe = 400 if n_total is None else min(n_total, 400)
    v, qo, thr = qgen(first, probe)
    t0 = time.perf_counter()
    OH.run_queries(v, qo, thr, thr, mode=1, threads=threads)
    dt = max(time.perf_counter() - t0, 1e-6)
    n = int(max(probe, probe * budget_s / dt))
    if n_total is not None:
        n = min(n, n_total - first)
    v, qo, thr = qgen(first, n)
    t0 = time.perf_counter()
    pairs, chk = OH.run_queries(v, qo, thr, thr, mode=1, threads=threads)
    dt = time.perf_counter() - t0
    return dict(values=int(qo[-1]), queries=n, seconds=dt, value_visits=pairs, checksum=chk, qo=qo, thr=thr, v=v)


def product_qgen(wl, offs):
    def gen(first, n):
        qo, thr = wl.query_offsets(first, n)
        return wl.queries_host(offs, first, n, qo), qo, thr
    return gen


def oracle_parity(OH, hibf, s, res_offs, res_ids, threads, n_count=50_000):
    """The device's membership lists (from the batch) and counting_agent<uint16>::bulk_count (recomputed on the
    first n_count queries) against the oracle on the same bits."""
    o_off, o_ids = OH.membership_batch(s["v"], s["qo"], s["thr"], threads=threads)
    n = s["queries"]
    out = {"oracle_sample_queries": n,
           "oracle_sample_equal": bool(np.array_equal(o_off, res_offs[:n + 1]) and
                                       np.array_equal(o_ids, res_ids[:int(res_offs[n])]))}
    m = min(n, n_count)
    qo = s["qo"][:m + 1]
    v, thr = s["v"][:int(qo[-1])], s["thr"][:m]
    o = OH.query_batch(v, qo, thr, thr, threads=threads)
    g_off, g_ids, g_cnt = hibf.counting_agent(2).query_batch(v, qo, thr)
    dg, nnz = count_digests(g_off, g_ids, g_cnt)
    out["oracle_count_sample_queries"] = m
    out["oracle_count_sample_equal"] = bool(np.array_equal(dg, o["cnt_digest"]) and np.array_equal(nnz, o["cnt_nnz"]))
    return out


def _ranks(x):
    r = np.empty(x.size)
    r[np.argsort(x, kind="stable")] = np.arange(x.size)
    return r


def learned_scheduler(hibf, tuning, d_v, d_qo, d_thr, qo, nq, n, stream):
    """Trains the cost model on one sub-batch's measured per-query work and times another sub-batch's persistent
    kernel with its root tasks in query order, in order of length, and in order of the model's prediction."""
    import torch

    from hibf_gb300 import _native as N
    from hibf_gb300.scheduler import cost_model

    a = hibf.membership_agent()
    a.tuning = tuning
    a.reserve(n, int(qo[-1]), n * 8 + 65536, n * 8 + 65536)
    a.set_stream(stream.cuda_stream)

    def sub(first):
        return d_v.data_ptr(), d_qo.data_ptr() + 8 * first, d_thr.data_ptr() + 8 * first

    def feats_work(first):
        v, q, t = sub(first)
        f = torch.zeros(n * 6, dtype=torch.float32, device="cuda")
        w = torch.zeros(n, dtype=torch.int64, device="cuda")
        a.query_features(v, q, n, t, 32, f.data_ptr())
        a.set_work_out(w.data_ptr(), n)
        a.query_batch_device(v, q, n, t)
        stream.synchronize()
        a.status()
        a.set_work_out(None)
        return f, w

    t0 = time.perf_counter()
    f_tr, w_tr = feats_work(0)
    model = cost_model(seed=1)
    loss = model.train(f_tr.data_ptr(), w_tr.data_ptr(), n, steps=500, lr=1e-2)
    train_s = time.perf_counter() - t0
    first = nq // 2
    f_te, w_te = feats_work(first)
    pred = torch.empty(n, dtype=torch.float32, device="cuda")
    model.predict(f_te.data_ptr(), n, pred.data_ptr(), stream.cuda_stream)
    lengths = torch.from_numpy(np.diff(qo[first:first + n + 1]).astype(np.float32)).cuda()
    o_len = torch.empty(n, dtype=torch.int32, device="cuda")
    o_learned = torch.empty(n, dtype=torch.int32, device="cuda")
    model.sort_desc(lengths.data_ptr(), n, o_len.data_ptr(), stream.cuda_stream)
    t1 = time.perf_counter()
    model.order(f_te.data_ptr(), n, o_learned.data_ptr(), stream.cuda_stream)
    stream.synchronize()
    order_s = time.perf_counter() - t1
    work = w_te.cpu().numpy().astype(np.float64)
    rho = lambda x: float(np.corrcoef(_ranks(x), _ranks(work))[0, 1])
    v, q, t = sub(first)
    results = {}

    def timed_orders(schedule):
        a.tuning = dict(tuning, schedule=schedule)
        times = {}
        for name, order in (("query_order", None), ("length_order", o_len), ("learned_order", o_learned)):
            a.set_order(order.data_ptr() if order is not None else None, n)
            ks = []
            for _ in range(7):
                a.query_batch_device(v, q, n, t)
                stream.synchronize()
                ks.append(a.kernel_ms())
            a.status()
            times[name] = float(np.median(ks[2:]))
            o, i, _ = a.fetch_results(n)
            results[(schedule, name)] = (o, i)
        a.set_order(None)
        return times

    times = timed_orders(tuning["schedule"])
    # the work queue (the schedule of streamed host batches): its claim order decides which tasks run last
    times_queue = timed_orders(N.SCHEDULE_QUEUE) if tuning["schedule"] != N.SCHEDULE_QUEUE else times
    base = results[(tuning["schedule"], "query_order")]
    same = all(np.array_equal(r[0], base[0]) and np.array_equal(r[1], base[1]) for r in results.values())
    return {"batch_queries": n, "train_queries": n, "train_steps": 500, "train_s": train_s, "train_mse": loss,
            "order_s": order_s, "spearman_learned": rho(pred.cpu().numpy().astype(np.float64)),
            "spearman_length": rho(np.diff(qo[first:first + n + 1]).astype(np.float64)),
            "kernel_ms": times, "gain_vs_query_order": times["query_order"] / times["learned_order"],
            "gain_vs_length_order": times["length_order"] / times["learned_order"],
            "work_queue": {"kernel_ms": times_queue,
                           "gain_vs_query_order": times_queue["query_order"] / times_queue["learned_order"],
                           "gain_vs_length_order": times_queue["length_order"] / times_queue["learned_order"]},
            "results_identical": same,
            "model": "6 features -> 32 -> 32 -> 1 ReLU MLP, full-batch Adam on log(1 + executed visits), "
                     "hibf_gb300/csrc/cost_model.cu"}


def h2d_probe(nbytes):
    """The host-to-device rate of one pinned copy of `nbytes` in this process (CUDA events)."""
    import torch

    h = torch.empty(nbytes // 8, dtype=torch.int64, pin_memory=True)
    d = torch.empty_like(h, device="cuda")
    d.copy_(h, non_blocking=True)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    d.copy_(h, non_blocking=True)
    e1.record()
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    del h, d
    return nbytes / (ms / 1e3) / 1e9


def measure_hibf(args, wl, world, stream, full):
    """Builds the workload's index and measures it: the persistent batch (graph replay, K timed steps), the kernel's
    roofline, bulk_count, the plain per-query form, the end-to-end host call with its timeline, the CPU oracle and
    the parity checks.  `full` adds the autotuner, serving and the learned scheduler (headline workload only)."""
    import torch

    from hibf_gb300 import _native as N

    hibf, offs, build = build_index(wl, args.scale)
    parity = index_vs_reference(hibf, wl, args.scale, offs)
    nq = args.queries or min(wl.n_queries, 1_000_000)
    qo, thr = wl.query_offsets(0, nq)
    nv = int(qo[-1])
    d_ub = torch.from_numpy(offs.view(np.int64)).cuda()
    d_qo = torch.from_numpy(qo.view(np.int64)).cuda()
    d_thr = torch.from_numpy(thr.view(np.int64)).cuda()
    d_v = torch.empty(max(nv, 1), dtype=torch.int64, device="cuda")
    wl.queries_device(d_ub.data_ptr(), 0, nq, d_qo.data_ptr(), d_v.data_ptr())
    torch.cuda.synchronize()

    agent = hibf.membership_agent()
    agent.reserve(nq, nv, nq * 8 + 65536, nq * 8 + 65536)
    agent.set_stream(stream.cuda_stream)
    tune = None
    if args.tuning:
        f = [int(x) for x in args.tuning.split(",")]
        t = dict(agent.tuning, values_per_lane=f[0], fetch_bytes=f[1], counter_bits=f[2])
        if len(f) >= 5:
            t.update(early_exit_first=0, early_exit_step=f[3], early_exit_stages=N.EARLY_EXIT_ADAPTIVE,
                     early_exit_min=f[4])
        if len(f) >= 6:
            t.update(schedule=f[5])
        agent.tuning = t
        tune = {"fixed": agent.tuning}
    elif not args.no_autotune:
        tune = {}
        if full:
            ns = min(nq, args.tune_queries)
            t0 = time.perf_counter()
            trials = agent.autotune(d_v.data_ptr(), d_qo.data_ptr(), ns, d_thr.data_ptr(), reps=2)
            tune = {"sample_queries": ns, "seconds": time.perf_counter() - t0, "sample_best": agent.tuning,
                    "trials": len(trials), "default_kernel_ms": trials[0]["kernel_ms"],
                    "best_kernel_ms": min(t["kernel_ms"] for t in trials)}
        # the task schedule is decided on the whole batch: grouping a level's tasks by IBF pays more the more tasks
        # share an IBF, which a sample understates
        base = agent.tuning
        ab = {}
        for label, extra in (("queue", dict(schedule=N.SCHEDULE_QUEUE, level_values_per_lane=0)),
                             ("levels", dict(schedule=N.SCHEDULE_LEVELS, level_values_per_lane=0)),
                             ("levels_2_values_per_lane_below_root",
                              dict(schedule=N.SCHEDULE_LEVELS, level_values_per_lane=2))):
            try:
                agent.tuning = dict(base, **extra)
            except N.InvalidArgument:
                continue  # no such kernel for this hierarchy
            ks = []
            for _ in range(2):
                agent.query_batch_device(d_v.data_ptr(), d_qo.data_ptr(), nq, d_thr.data_ptr())
                stream.synchronize()
                ks.append(agent.kernel_ms())
            agent.status()
            ab[label] = (min(ks), dict(agent.tuning))
        best = min(ab, key=lambda k: ab[k][0])
        agent.tuning = ab[best][1]
        tune.update(schedule_trials_full_batch_ms={k: round(v[0], 3) for k, v in ab.items()}, schedule=best,
                    best=agent.tuning)
    agent.capture_batch_device(d_v.data_ptr(), d_qo.data_ptr(), nq, d_thr.data_ptr())
    for _ in range(max(args.warmup, 3)):
        agent.replay()
    stream.synchronize()
    agent.status()

    steps = args.steps if full else max(3, min(args.steps, 10))
    gpu_index = int(os.environ.get("CUDA_VISIBLE_DEVICES", str(torch.cuda.current_device())).split(",")[0] or 0)
    clocks = ClockSampler(gpu_index)
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        agent.replay()
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    agent.status()
    ms = e0.elapsed_time(e1) / steps
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    tasks, visits = agent.last_work()
    executed = agent.last_work_executed()
    kms = []
    for _ in range(3):
        agent.replay()
        stream.synchronize()
        kms.append(agent.kernel_ms())
    kernel_ms = sum(kms) / len(kms)
    level_ms = agent.level_ms()
    level_work = agent.level_work()
    res_offs, res_ids, _ = agent.fetch_results(nq)
    # the device's own random 8-byte read rate at the index's footprint (fully random, and 2 MiB-local)
    import ctypes as _ct

    probe = {}
    fp = min(int(hibf.info()["device_bytes"]), 16 << 30)
    for name, region in (("random", 0), ("window_2MiB", 2 << 20)):
        rps = _ct.c_double(0)
        N.call("hibf_gpu_probe_random_reads", fp, region, _ct.byref(rps))
        probe[name] = rps.value

    # plain form: one launch per query on the first P queries
    P = min(args.plain_queries if full else 1000, nq)
    pa = hibf.membership_agent()
    pa.tuning = agent.tuning
    pa.reserve(P, nv, 65536, P * 8 + 65536)
    pa.set_stream(stream.cuda_stream)
    pa.query_plain_device(d_v.data_ptr(), qo[:P + 1], thr[:P])  # warm-up
    stream.synchronize()
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    pa.query_plain_device(d_v.data_ptr(), qo[:P + 1], thr[:P])
    p1.record(stream)
    p1.synchronize()
    plain_s = p0.elapsed_time(p1) / 1e3
    plain_offs, plain_ids, _ = pa.fetch_results(P)
    parity["plain_equals_batch"] = bool(np.array_equal(plain_offs, res_offs[:P + 1]) and
                                        np.array_equal(plain_ids, res_ids[:int(res_offs[P])]))
    plain_vps = float(qo[P]) / plain_s
    del pa

    # counting_agent<uint16>::bulk_count over the same batch (every count exact); its user bins must be the lists
    ca = hibf.counting_agent(2)
    ca.tuning = agent.tuning
    ca.reserve(nq, nv, nq * 8 + 65536, nq * 8 + 65536)
    ca.set_stream(stream.cuda_stream)
    ca.capture_batch_device(d_v.data_ptr(), d_qo.data_ptr(), nq, d_thr.data_ptr(), mode=N.QUERY_COUNT, width=2)
    for _ in range(2):
        ca.replay()
    stream.synchronize()
    ca.status()
    c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    count_steps = max(1, min(steps, 5))
    c0.record(stream)
    for _ in range(count_steps):
        ca.replay()
    c1.record(stream)
    c1.synchronize()
    ca.status()
    count_ms = c0.elapsed_time(c1) / count_steps
    c_offs, c_ids, c_cnt = ca.fetch_results(nq, mode=N.QUERY_COUNT, width=2)
    parity["count_user_bins_equal_membership"] = bool(np.array_equal(c_offs, res_offs) and
                                                      np.array_equal(c_ids, res_ids))
    parity["counts_at_least_threshold"] = bool(np.all(c_cnt.astype(np.uint64) >= np.repeat(
        thr, np.diff(c_offs).astype(np.int64))))
    count = {"values_per_s": world * nv / (count_ms / 1e3), "ms_per_step": count_ms, "steps": count_steps,
             "form": "one persistent launch per batch, CUDA-graph replay, uint16 counts"}
    del ca, c_offs, c_ids, c_cnt

    # end to end through the C ABI host call: pinned host inputs -> H2D -> batch -> D2H results, with its timeline
    h_v = torch.empty(max(nv, 1), dtype=torch.int64, pin_memory=True)
    h_v.copy_(d_v)
    hv = h_v.numpy().view(np.uint64)[:nv]
    ea = hibf.membership_agent()
    ea.tuning = agent.tuning
    ea.reserve(nq, nv, nq * 8 + 65536, nq * 8 + 65536)
    for _ in range(2):
        ea.query_batch(hv, qo, thr)
    e2e_steps = args.e2e_steps or (max(3, min(steps, 10)) if full else 3)
    torch.cuda.synchronize()
    wall, timelines = [], []
    for _ in range(e2e_steps):
        t0 = time.perf_counter()
        eo, ei, _ = ea.query_batch(hv, qo, thr, copy=False)  # results: views of the agent's page-locked buffers
        wall.append(time.perf_counter() - t0)
        timelines.append(ea.last_timeline())
    e2e_s = sum(wall) / len(wall)
    parity["e2e_equals_batch"] = bool(np.array_equal(eo, res_offs) and np.array_equal(ei, res_ids))
    h2d = nv * 8 + (nq + 1) * 8 + nq * 8
    d2h = (nq + 1) * 8 + int(eo[-1]) * 8 + 8 * 8 + 16
    last = timelines[-1]
    n_chunks = len(last) - 3
    in_place = ea.last_in_place()
    e2e_level_ms = [round(x, 3) for x in ea.level_ms()]
    e2e_timeline = {
        "values": "read in place by the kernel over the host link" if in_place else f"copied in {n_chunks} chunks",
        "median_ms": {("inputs_ready" if in_place else "values_copied"):
                      float(np.median([t[n_chunks - 1] for t in timelines])),
                      "kernel_start": float(np.median([t[n_chunks] for t in timelines])),
                      "kernel_end": float(np.median([t[n_chunks + 1] for t in timelines])),
                      "results_back": float(np.median([t[n_chunks + 2] for t in timelines]))},
        "wall_ms_per_call": [round(w * 1e3, 2) for w in wall],
        "wall_ms_median": round(float(np.median(wall)) * 1e3, 2),
        "results_back_ms_per_call": [round(t[n_chunks + 2], 2) for t in timelines],
        "level_ms": e2e_level_ms,
        "note": "ms from the call's first device work; inputs_ready = offsets and thresholds on the device",
    }
    # the same calls with the values copied first (streamed in chunks while the work queue runs)
    ea.set_host_read(False)
    ea.query_batch(hv, qo, thr)
    wall_cp, timelines_cp = [], []
    for _ in range(e2e_steps):
        t0 = time.perf_counter()
        co, ci, _ = ea.query_batch(hv, qo, thr, copy=False)
        wall_cp.append(time.perf_counter() - t0)
        timelines_cp.append(ea.last_timeline())
    parity["e2e_copied_equals_batch"] = bool(not ea.last_in_place() and np.array_equal(co, res_offs) and
                                             np.array_equal(ci, res_ids))
    nc = len(timelines_cp[-1]) - 3
    e2e_copied = {"value": world * nv / (sum(wall_cp) / len(wall_cp)), "unit": "values/s",
                  "ms_per_step": sum(wall_cp) / len(wall_cp) * 1e3,
                  "wall_ms_median": round(float(np.median(wall_cp)) * 1e3, 2),
                  "wall_ms_per_call": [round(w * 1e3, 2) for w in wall_cp],
                  "chunks": nc,
                  "values_copied_ms_per_call": [round(t[nc - 1], 2) for t in timelines_cp],
                  # calls whose copy took over 1.5x the fastest call's: the host link, not the kernel, set their time
                  "slow_copy_calls": int(sum(t[nc - 1] > 1.5 * min(u[nc - 1] for u in timelines_cp)
                                             for t in timelines_cp)),
                  "h2d_GBps_probe": h2d_probe(min(nv * 8, 4 << 30)),
                  "call": "hibf_gpu_agent_query_batch after hibf_gpu_agent_set_host_read(0)"}
    del ea

    serving = []
    if full and not args.no_serve and wl.name == "hibf8192":
        from hibf_gb300.serve import server

        pool_q = min(nq, 100_000)
        # the requests' values live in their own page-locked pool written by the host, as a server's receive buffers
        # would be (not a view of the end-to-end buffer, which the device wrote)
        pool_t = torch.empty(int(qo[pool_q]), dtype=torch.int64, pin_memory=True)
        pool_v = pool_t.numpy().view(np.uint64)
        pool_v[:] = hv[:pool_v.size]

        def pool_copy_ms(src_t, mb=29):
            """Device time of plain copies of pool slices (CUDA events on a side stream): the link's own rate."""
            n = int(mb * (1 << 20) / 8)
            dst = torch.empty(n, dtype=torch.int64, device="cuda")
            side = torch.cuda.Stream()
            ms = []
            for rep in range(5):
                a = (rep * 1_000_003) % (pool_v.size - n)
                src = src_t[a:a + n]
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                with torch.cuda.stream(side):
                    e0.record(side)
                    dst.copy_(src, non_blocking=True)
                    e1.record(side)
                e1.synchronize()
                ms.append(e0.elapsed_time(e1))
                time.sleep(0.02)
            return round(float(np.median(ms)), 4)

        pool_copy_before = {"request_pool": pool_copy_ms(pool_t), "end_to_end_buffer": pool_copy_ms(h_v)}
        # 1e5 and 1e6 queries/s run for at least 10,000 requests (about 490 queries per request)
        for load, dur in ((1e4, 10.0), (1e5, 50.0), (1e6, 5.0)):
            srv = server(hibf, slots=4, max_batch_queries=65536, max_batch_values=1 << 27, admission_bytes=4 << 30)
            r = srv.open_loop(pool_v, qo[:pool_q + 1], offered_qps=load, duration_s=dur, max_request_queries=4096,
                              thr_lo=0.5, thr_hi=0.9, seed=int(load))
            r["mean_batch_phases_ms"] = srv.phase_times()
            r["tail_batch_phases"] = srv.tail_phases(0.99)
            if r["requests"] < 10_000:
                r["p999_ms"] = None  # fewer than 10,000 requests: no meaningful 99.9th percentile
            if r["requests"] < 1_000:
                r["p99_note"] = f"{r['requests']} requests: the 99th percentile is near the maximum"
            serving.append(r)
            srv.close()
        # plain copies of 29 MB slices before the load points (from the request pool and from the same range of the
        # end-to-end buffer) and after them
        serving[0]["pool_copy_29MB_ms"] = {"before": pool_copy_before,
                                           "after": {"request_pool": pool_copy_ms(pool_t),
                                                     "end_to_end_buffer": pool_copy_ms(h_v)}}
        del pool_t
    learned = None
    if full and not args.no_learned and nq >= 2 * args.sched_queries:
        learned = learned_scheduler(hibf, agent.tuning, d_v, d_qo, d_thr, qo, nq, args.sched_queries, stream)

    # CPU oracle (all host cores) on the same bits, and parity on its sample
    cpu = None
    if not args.no_cpu:
        dev_bytes = int(hibf.info()["device_bytes"])
        if dev_bytes < 0.6 * host_ram_bytes():
            OH = oracle_from_device(hibf)
            threads = os.cpu_count() or 1
            qgen = product_qgen(wl, offs)
            s = cpu_sample(OH, qgen, args.cpu_seconds, threads, n_total=nq)
            s1 = cpu_sample(OH, qgen, 3.0, 1, n_total=nq)
            cpu = {"value": s["values"] / s["seconds"], "unit": "values/s", "cores": threads, "kind": "port",
                   "machine": platform.machine(), "value_1_thread": s1["values"] / s1["seconds"],
                   "sample": f"first {s['queries']} queries ({s['values']} values) of the batch, membership_for + "
                             f"sort_results, oracle/hibf_oracle.c with {threads} OpenMP threads on the full index"}
            parity.update(oracle_parity(OH, hibf, s, res_offs, res_ids, threads))
            del OH
            gc.collect()
        else:
            parity["oracle"] = f"skipped: the {dev_bytes / 1e9:.0f} GB index exceeds 60% of host memory"

    hbm, peak_kind = peaks()
    bytes_per_visit = wl.h * 32  # h rows of ceil(tb/256) = 1 sector each (every IBF has tb <= tmax <= 256)
    achieved = visits * bytes_per_visit / (kernel_ms / 1e3) / 1e9
    achieved_executed = executed * bytes_per_visit / (kernel_ms / 1e3) / 1e9
    tpv = traffic_per_value_visit(wl.name)
    value = world * nv / (ms / 1e3)
    out = {
        "value": value, "unit": "values/s", "ms_per_step": ms, "steps": steps,
        "config": config_of(wl, nq, nv, hibf.n_ibfs, args.scale, world),
        "index_bytes": int(hibf.info()["device_bytes"]),
        "queries_per_s": world * nq / (ms / 1e3),
        "e2e": {"value": world * nv / e2e_s, "unit": "values/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3,
                "call": "hibf_gpu_agent_query_batch (host buffers, page-locked: values read in place; results "
                        "returned in the agent's page-locked buffers)",
                "timeline": e2e_timeline, "copied_first": e2e_copied},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "peak_kind": peak_kind, "achieved_executed": achieved_executed,
                     "frac_executed": achieved_executed / hbm,
                     "traffic": (tpv * executed) if tpv is not None else None,
                     "dram_bytes_per_executed_visit": tpv,
                     "kernel": "k_query", "kernel_ms": kernel_ms, "value_visits": visits,
                     "value_visits_executed": executed, "tasks": tasks,
                     "algorithmic_bytes_per_value_visit": bytes_per_visit,
                     "row_reads_per_s": executed * wl.h / (kernel_ms / 1e3),
                     "level_ms": [round(x, 3) for x in level_ms],
                     "level_value_visits": [w["value_visits"] for w in level_work],
                     "level_value_visits_executed": [w["value_visits_executed"] for w in level_work],
                     "random_read_ceiling": {"footprint_bytes": fp, "reads_per_s_random": probe["random"],
                                             "reads_per_s_2MiB_windows": probe["window_2MiB"],
                                             "probe": "hibf_gpu_probe_random_reads"}},
        "cpu_baseline": cpu, "clocks": clk,
        "plain": {"values_per_s": plain_vps, "queries": P, "form": "one launch per query"},
        "batched_vs_plain": value / world / plain_vps,
        "bulk_count": count, "build": build, "autotune": tune, "learned_scheduler": learned,
        "serving": serving, "parity": parity,
        # per step: control reset, the query kernel (one launch per level, and three grouping kernels between
        # levels, under the level schedule), six compaction kernels
        "gpu_launches": steps * (1 + (1 if not level_ms else 1 + 4 * (len(level_ms) - 1)) + 6),
    }
    del agent, hibf, d_v, d_qo, d_thr, d_ub, h_v
    gc.collect()
    torch.cuda.empty_cache()
    return out


def run_ours(args, wl, rank, world, local):
    import torch

    from hibf_gb300 import _native as N
    from hibf_gb300.workloads import WORKLOADS

    torch.cuda.set_device(local)
    if args.l2_fetch >= 0:
        N.call("hibf_gpu_set_l2_fetch_granularity", args.l2_fetch)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    stream = torch.cuda.Stream()
    m = measure_hibf(args, wl, world, stream, full=True)
    c4 = None
    if wl.name == "hibf8192" and not args.no_c4 and args.scale == 1.0 and not args.queries:
        w4 = WORKLOADS["hibf65536"]
        m4 = measure_hibf(args, w4, world, stream, full=False)
        c4 = {k: m4[k] for k in ("value", "unit", "ms_per_step", "steps", "config", "index_bytes", "queries_per_s",
                                 "e2e", "roofline", "cpu_baseline", "plain", "batched_vs_plain", "bulk_count",
                                 "build", "autotune", "clocks")}
        m["parity"].update({"c4_" + k: v for k, v in m4["parity"].items()})
        del m4
        gc.collect()
        torch.cuda.empty_cache()
    c2 = None
    if wl.name == "hibf8192" and not args.no_c2 and args.scale == 1.0 and not args.queries:
        r2 = run_ibf_ours(args, rank, world, local, own_pg=False)
        if r2 is not None:
            c2 = {k: r2[k] for k in ("metric", "value", "unit", "ms_per_step", "steps", "config", "kernels", "build",
                                     "e2e", "gpu_launches", "roofline", "cpu_baseline", "clocks")}
            m["parity"].update({"c2_" + k: v for k, v in r2["parity"].items()})
        gc.collect()
        torch.cuda.empty_cache()
    out = None
    if rank == 0:
        serving = m["serving"]
        parity = m.pop("parity")
        out = {
            "metric": METRIC, "value": m["value"], "unit": "values/s", "n_gpus": world, "steps": m["steps"],
            "warmup": args.warmup, "ms_per_step": m["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64",
            "data": "synthetic: seeded splitmix64 user bins and queries (include/hibf_gb300_synthetic.h)",
            "config": m["config"], "gpu_launches": m["gpu_launches"], "e2e": m["e2e"], "roofline": m["roofline"],
            "cpu_baseline": m["cpu_baseline"], "clocks": m["clocks"],
            "form": "one persistent launch per batch, CUDA-graph replay",
            "index_bytes": m["index_bytes"], "queries_per_s": m["queries_per_s"], "plain": m["plain"],
            "batched_vs_plain": m["batched_vs_plain"], "bulk_count": m["bulk_count"], "build": m["build"],
            "autotune": m["autotune"], "learned_scheduler": m["learned_scheduler"],
            "serving": serving,
            "p99_serve_latency_ms": ({f"{r['offered_qps']:.0e} queries/s offered": round(r["p99_ms"], 3)
                                      for r in serving} if serving else None),
            "serving_config": "open-loop Poisson, request sizes log-uniform 1-4096 queries from the batch's first "
                              "100k queries, thresholds U(0.5,0.9)*len, 4 slots, 4 GiB admission cap",
            "c4": c4,
            "c2": c2,
            "parity": parity,
        }
    if world > 1:
        torch.distributed.destroy_process_group()
    return out


def run_reference(args, wl, rank, world, local):
    """The reference CPU path on the host cores, with nothing of the product loaded: the C restatement of the
    reference's query (oracle/hibf_oracle.c) on all host threads, over an index the oracle fills itself from the
    reference's own tables (tests/golden/ref_*.npz), the committed split table and the generator; its IBFs are
    compared with the reference's digests before timing."""
    if rank != 0:
        return None
    from oracle.bindings import Oracle, build_oracle

    build_oracle()
    O = Oracle()
    ref = reference_build(wl, args.scale)
    table_file = GOLDEN / (wl.split_table_file or "")
    if ref is None or not wl.split_table_file or not table_file.exists():
        return {"impl": "reference", "unavailable": f"no committed reference build and split table of {wl.name} at "
                                                    f"scale {args.scale:g}"}
    q = wl.query
    offs = scaled(O.synth_user_bin_offsets(q.seed, wl.size_law, wl.size_p0, wl.size_p1, wl.size_lo, wl.size_hi,
                                           wl.n_user_bins), args.scale)
    split = dict(np.load(table_file))
    if not np.array_equal(ref["ub_offsets"], offs) or not np.array_equal(
            np.diff(offs)[split["user_bin"].astype(np.int64)], split["n_values"]):
        return {"impl": "reference", "unavailable": "the committed reference build does not match this host's sizes"}
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    OH = O.hibf(dict(n_user_bins=wl.n_user_bins, bins=ref["bins"], bin_size=ref["bin_size"],
                     hash_funs=ref["hash_funs"], next_ibf=ref["next_ibf"], user_bin=ref["user_bin"]))
    OH.fill_synthetic(q.seed, offs, split, threads)
    fill_s = time.perf_counter() - t0
    digests_equal = bool(np.array_equal(OH.digests(threads), ref["digests"]))
    nq = args.queries or min(wl.n_queries, 1_000_000)

    def qgen(first, n):
        return O.synth_queries(q, offs, first, n, threads)

    per_step = max(1.0, min(args.cpu_seconds, 60.0 / max(1, args.steps + args.warmup)))
    first = 0
    for _ in range(args.warmup):
        s = cpu_sample(OH, qgen, per_step, threads, first, n_total=nq)
        first = (first + s["queries"]) % max(1, nq - 1)
    vals, secs, nqs = 0, 0.0, 0
    for _ in range(args.steps):
        s = cpu_sample(OH, qgen, per_step, threads, first, n_total=nq)
        first = (first + s["queries"]) % max(1, nq - 1)
        vals += s["values"]
        secs += s["seconds"]
        nqs += s["queries"]
    value = vals / secs
    nv = int(O.synth_query_offsets(q, 0, nq)[0][-1])  # the step's values, as the GPU arm counts them
    sample = (f"{args.steps} steps of ~{per_step:.1f} s, {nqs} queries ({vals} values) in total, membership_for + "
              f"sort_results, oracle/hibf_oracle.c with {threads} OpenMP threads; index filled by the oracle in "
              f"{fill_s:.0f} s, every IBF equal to the reference's build: {digests_equal}")
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": "values/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": secs / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic: seeded splitmix64 user bins and queries (include/hibf_gb300_synthetic.h)",
            "config": config_of(wl, nq, nv, int(ref["bins"].size), args.scale, world),
            "cpu_baseline": {"value": value, "unit": "values/s", "cores": threads, "kind": "port",
                             "machine": platform.machine(), "sample": sample},
            "e2e": {"value": value, "unit": "values/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "parity": {"index_equals_reference": digests_equal}}


def ibf_oracle_from_device(ibf, w):
    """The C oracle's IBF holding the device-built bit store (downloaded in place)."""
    from hibf_gb300 import _native as N
    from oracle.bindings import Oracle, build_oracle

    build_oracle()
    O = Oracle().ibf(w["bins"], w["bin_size"], w["h"])
    addr, n = O.data_ptr()
    N.call("hibf_gpu_ibf_download_words", ibf._h, addr, n)
    return O


def ibf_cpu_sample(O, w, budget_s, threads):
    """Times the oracle's bulk_count<uint16> + bulk_contains over a bounded sample of the query values."""
    from hibf_gb300 import synthetic as S

    n = 1 << 14
    while True:
        q = S.ibf_query_values(w["seed"], w["bins"], w["values_per_bin"], 0, n)
        t0 = time.perf_counter()
        cnt = O.bulk_count(q, 2, threads=threads)
        con = O.bulk_contains(q, threads=threads)
        dt = time.perf_counter() - t0
        if dt * 4 > budget_s or n >= w["n_queries"]:
            return dict(values=n, seconds=dt, count=cnt, contains=con, q=q)
        n = min(w["n_queries"], n * 4)


def ibf_workload(scale=1.0):
    """The 1,024-bin IBF workload; scale < 1 shrinks the bin size, values per bin and query values together (for
    profiling captures that must stay small)."""
    w = dict(IBF1024)
    if scale != 1.0:
        w["bin_size"] = max(1 << 12, int(w["bin_size"] * scale))
        w["values_per_bin"] = max(1, int(w["values_per_bin"] * scale))
        w["n_queries"] = max(1 << 16, int(w["n_queries"] * scale))
    return w


def build_ibf1024(w, stream):
    import torch

    import hibf_gb300 as hg
    from hibf_gb300 import _native as N

    ibf = hg.interleaved_bloom_filter(hg.bin_count(w["bins"]), hg.bin_size(w["bin_size"]),
                                      hg.hash_function_count(w["h"]))
    torch.cuda.synchronize()
    b0, b1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    b0.record(stream)
    N.call("hibf_gpu_synth_ibf_emplace", ibf._h, w["seed"], w["values_per_bin"], 0, w["bins"], stream.cuda_stream)
    b1.record(stream)
    b1.synchronize()
    return ibf, b0.elapsed_time(b1)


def run_ibf_ours(args, rank, world, local, own_pg=True):
    """The single-level IBF workload; own_pg=False when it runs as a sub-record inside run_ours (whose process
    group it then uses)."""
    import torch

    from hibf_gb300 import _native as N

    torch.cuda.set_device(local)
    if world > 1 and own_pg:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    w = ibf_workload(args.scale)
    nq = args.queries or w["n_queries"]
    stream = torch.cuda.Stream()
    ibf, build_ms = build_ibf1024(w, stream)
    bw = ibf.bin_words
    d_q = torch.empty(nq, dtype=torch.int64, device="cuda")
    N.call("hibf_gpu_synth_ibf_queries_d", w["seed"], w["bins"], w["values_per_bin"], 0, nq, d_q.data_ptr(),
           stream.cuda_stream)
    d_cnt = torch.empty(w["bins"], dtype=torch.int16, device="cuda")
    d_con = torch.empty(nq * bw, dtype=torch.int64, device="cuda")
    sp = stream.cuda_stream

    def step(ev=None):
        if ev:
            ev[0].record(stream)
        N.call("hibf_gpu_ibf_bulk_count_d", ibf._h, d_q.data_ptr(), nq, 2, d_cnt.data_ptr(), sp)
        if ev:
            ev[1].record(stream)
        N.call("hibf_gpu_ibf_bulk_contains_d", ibf._h, d_q.data_ptr(), nq, d_con.data_ptr(), sp)
        if ev:
            ev[2].record(stream)

    for _ in range(max(args.warmup, 3)):
        step()
    stream.synchronize()
    gpu_index = int(os.environ.get("CUDA_VISIBLE_DEVICES", str(local)).split(",")[0] or 0)
    clocks = ClockSampler(gpu_index)
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    for k in range(args.steps):
        step(evs[k])
    stream.synchronize()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    count_ms = sum(e[0].elapsed_time(e[1]) for e in evs) / args.steps
    contains_ms = sum(e[1].elapsed_time(e[2]) for e in evs) / args.steps
    ms = sum(e[0].elapsed_time(e[2]) for e in evs) / args.steps
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())

    # size-independent check at full size: the counts are the column sums of the contains bit vectors (mod 2^16)
    c8 = d_con.view(torch.uint8).view(nq, bw * 8)
    col = torch.zeros(bw * 64, dtype=torch.int64, device="cuda")
    for k in range(8):
        col.view(bw * 8, 8)[:, k] = ((c8 >> k) & 1).sum(dim=0, dtype=torch.int64)
    col = (col[: w["bins"]] & 0xFFFF).to(torch.int32)
    counts_equal_contains = bool(torch.equal(col, d_cnt.to(torch.int32) & 0xFFFF))

    # end to end through the host entry points: pinned host values in, count vector and contains words out
    h_q = torch.empty(nq, dtype=torch.int64, pin_memory=True)
    h_q.copy_(d_q)
    h_cnt = torch.empty(w["bins"], dtype=torch.int16, pin_memory=True)
    h_con = torch.empty(nq * bw, dtype=torch.int64, pin_memory=True)

    def host_step():
        N.call("hibf_gpu_ibf_bulk_count", ibf._h, h_q.data_ptr(), nq, 2, h_cnt.data_ptr())
        N.call("hibf_gpu_ibf_bulk_contains", ibf._h, h_q.data_ptr(), nq, h_con.data_ptr())

    host_step()
    e2e_steps = args.e2e_steps or max(3, min(args.steps, 5))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        host_step()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e_equal = bool(torch.equal(h_cnt, d_cnt.cpu()))

    out = None
    if rank == 0:
        hbm, peak_kind = peaks()
        rows = w["h"] * bw * 8  # h rows of bin_words words: 384 B per value
        count_bytes = nq * (rows + 8)
        contains_bytes = nq * (rows + 8 + bw * 8)
        achieved = (count_bytes + contains_bytes) / (ms / 1e3) / 1e9
        tb = traffic_per_value_visit("ibf1024")
        parity = {"counts_equal_contains_column_sums": counts_equal_contains, "e2e_equals_device": e2e_equal}
        cpu = None
        if not args.no_cpu:
            O = ibf_oracle_from_device(ibf, w)
            threads = os.cpu_count() or 1
            smp = ibf_cpu_sample(O, w, args.cpu_seconds, threads)
            n = smp["values"]
            cpu = {"value": n / smp["seconds"], "unit": "values/s", "cores": threads, "kind": "port",
                   "machine": platform.machine(),
                   "sample": f"first {n} query values, bulk_count<uint16> + bulk_contains, oracle/hibf_oracle.c with "
                             f"{threads} OpenMP threads"}
            dq = torch.from_numpy(smp["q"].view(np.int64)).cuda()
            dc = torch.empty(w["bins"], dtype=torch.int16, device="cuda")
            N.call("hibf_gpu_ibf_bulk_count_d", ibf._h, dq.data_ptr(), n, 2, dc.data_ptr(), None)
            torch.cuda.synchronize()
            parity["oracle_sample_values"] = n
            parity["oracle_sample_count_equal"] = bool(np.array_equal(dc.cpu().numpy().view(np.uint16), smp["count"]))
            parity["oracle_sample_contains_equal"] = bool(np.array_equal(
                d_con[: n * bw].cpu().numpy().view(np.uint64).reshape(n, bw), smp["contains"]))
        value = world * nq / (ms / 1e3)
        out = {
            "metric": "IBF bulk_contains + bulk_count<uint16> query values/s on 1 GB300 (bit-exact)",
            "value": value, "unit": "values/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic: seeded splitmix64 bins and query values (include/hibf_gb300_synthetic.h)",
            "config": {"workload": WORKLOAD_DESC["ibf1024"], "name": "ibf1024", "size_scale": args.scale,
                       "bins": w["bins"],
                       "bin_size": w["bin_size"], "hash_functions": w["h"], "query_values_per_step": nq,
                       "index_bytes": w["bins"] // 64 * 8 * w["bin_size"], "parallelism": f"replicas x{world}",
                       "l2": "index (8 GiB) and outputs (2 GiB) larger than L2; no flush",
                       "form": "one launch per call (bulk_count_d, bulk_contains_d)"},
            "kernels": {"bulk_count_ms": count_ms, "bulk_contains_ms": contains_ms,
                        "bulk_count_values_per_s": nq / (count_ms / 1e3),
                        "bulk_contains_values_per_s": nq / (contains_ms / 1e3),
                        "bulk_count_GBps": count_bytes / (count_ms / 1e3) / 1e9,
                        "bulk_contains_GBps": contains_bytes / (contains_ms / 1e3) / 1e9},
            "build": {"inserts": w["bins"] * w["values_per_bin"], "ms": build_ms,
                      "inserts_per_s": w["bins"] * w["values_per_bin"] / (build_ms / 1e3),
                      "algorithmic_GBps": w["bins"] * w["values_per_bin"] * w["h"] * 64 / (build_ms / 1e3) / 1e9,
                      "bytes_per_insert": w["h"] * 64, "form": "hibf_gpu_synth_ibf_emplace (values generated on "
                                                               "the device, atomicOr)"},
            "e2e": {"value": world * nq / e2e_s, "unit": "values/s", "h2d_bytes_per_step": 2 * nq * 8,
                    "d2h_bytes_per_step": w["bins"] * 2 + nq * bw * 8, "ms_per_step": e2e_s * 1e3,
                    "call": "hibf_gpu_ibf_bulk_count + hibf_gpu_ibf_bulk_contains (pinned host buffers)"},
            "gpu_launches": 4 * args.steps,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                         "peak_kind": peak_kind,
                         # both kernels of a step, from the committed ncu capture scaled by the values
                         "traffic": None if tb is None else tb * nq,
                         "dram_bytes_per_value": tb,
                         "algorithmic_bytes_per_value": {"bulk_count": rows + 8, "bulk_contains": rows + 8 + bw * 8}},
            "cpu_baseline": cpu, "clocks": clk, "parity": parity,
        }
    if world > 1 and own_pg:
        torch.distributed.destroy_process_group()
    return out


def run_ibf_reference(args, rank, world, local):
    """The reference arm for the IBF workload: the oracle's bulk_count + bulk_contains on the host cores (bounded
    samples), over the bit store built on the device (set-up, not timed)."""
    if rank != 0:
        return None
    import torch

    torch.cuda.set_device(local)
    w = ibf_workload(args.scale)
    stream = torch.cuda.Stream()
    ibf, _ = build_ibf1024(w, stream)
    O = ibf_oracle_from_device(ibf, w)
    del ibf
    threads = os.cpu_count() or 1
    per_step = max(1.0, min(args.cpu_seconds, 60.0 / max(1, args.steps + args.warmup)))
    for _ in range(args.warmup):
        ibf_cpu_sample(O, w, per_step, threads)
    vals, secs = 0, 0.0
    for _ in range(args.steps):
        s = ibf_cpu_sample(O, w, per_step, threads)
        vals += s["values"]
        secs += s["seconds"]
    value = vals / secs
    return {"impl": "reference", "metric": "IBF bulk_contains + bulk_count<uint16> query values/s on 1 GB300 "
                                           "(bit-exact)",
            "value": value, "unit": "values/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": secs / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64", "data": "synthetic",
            "config": {"workload": WORKLOAD_DESC["ibf1024"], "name": "ibf1024"},
            "cpu_baseline": {"value": value, "unit": "values/s", "cores": threads, "kind": "port",
                             "machine": platform.machine(),
                             "sample": f"{args.steps} samples of ~{per_step:.1f} s ({vals} values), oracle/hibf_oracle.c"},
            "e2e": {"value": value, "unit": "values/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    args = parse_args()
    rank, world, local = dist_env()
    from hibf_gb300.workloads import WORKLOADS

    if args.workload == "ibf1024":
        out = run_ibf_reference(args, rank, world, local) if args.impl == "reference" else \
            run_ibf_ours(args, rank, world, local)
        if rank == 0 and out is not None:
            print(json.dumps(out), flush=True)
        return
    wl = WORKLOADS[args.workload]
    out = run_reference(args, wl, rank, world, local) if args.impl == "reference" else \
        run_ours(args, wl, rank, world, local)
    if rank == 0 and out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
