"""hierarchical_interleaved_bloom_filter -- device-resident HIBF (reference:
include/hibf/hierarchical_interleaved_bloom_filter.hpp, src/hierarchical_interleaved_bloom_filter.cpp).

    hibf = hierarchical_interleaved_bloom_filter.from_tables(...)     # tables of a built HIBF (+ its words)
    hibf = hierarchical_interleaved_bloom_filter(config, layout_text)  # built from a layout (hibf_gb300.build)
    agent = hibf.membership_agent()
    ids = agent.membership_for(values, threshold)   # user bins in the reference's traversal order
    agent.sort_results()                            # ascending, as HIBF.hpp:380-383
    counts = hibf.counting_agent(width=2).bulk_count(values, threshold)
    offs, ids, cnts = agent.query_batch(values, query_offsets, thresholds)   # one persistent launch

Tables use the reference's conventions: next_ibf_id[k][b] (self for non-merged bins) and
ibf_bin_to_user_bin_id[k][b] with BIN_MERGED / BIN_DELETED sentinels; IBF 0 is the root.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N

_DT = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}


def _u64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint64).reshape(-1))


def ibf_paths(bins, next_ibf, user_bin) -> dict:
    """{path of merged bins from the root: IBF index}.  The reference numbers the IBFs below the root in a shuffled
    order (src/hierarchical_interleaved_bloom_filter.cpp:111-116), so two builds of one layout are compared IBF by
    IBF through these paths."""
    bins = [int(b) for b in bins]
    off = np.zeros(len(bins) + 1, np.int64)
    off[1:] = np.cumsum(bins)
    nxt, ub = _u64(next_ibf), _u64(user_bin)
    out = {(): 0}
    seen = {0}
    stack = [(0, ())]
    while stack:
        k, path = stack.pop()
        for b in range(bins[k]):
            i = off[k] + b
            c = int(nxt[i])
            if int(ub[i]) == N.BIN_MERGED and c != k and c not in seen:
                seen.add(c)
                out[path + (b,)] = c
                stack.append((c, path + (b,)))
    return out


def traversal_rank(n_user_bins: int, bins, next_ibf, user_bin) -> np.ndarray:
    """Position of every user bin in the order membership_for reports it (HIBF.hpp:322-355): bins scanned in
    order, merged bins descended in place.  A user bin occurs in one place, so sorting a result by this rank gives
    the reference's unsorted output."""
    bins = [int(b) for b in bins]
    off = np.zeros(len(bins) + 1, np.int64)
    off[1:] = np.cumsum(bins)
    nxt, ub = _u64(next_ibf), _u64(user_bin)
    rank = np.full(n_user_bins, np.iinfo(np.int64).max, np.int64)
    r = 0
    stack = [(0, 0)]
    seen = 0
    while stack:
        k, b = stack.pop()
        seen += 1
        if seen > 4 * (off[-1] + 1):
            break
        if b >= bins[k]:
            continue
        stack.append((k, b + 1))
        i = off[k] + b
        u = int(ub[i])
        if u == N.BIN_MERGED:
            c = int(nxt[i])
            if c != k:
                stack.append((c, 0))
        elif u != N.BIN_DELETED and (b + 1 == bins[k] or int(ub[i + 1]) != u):
            if rank[u] == np.iinfo(np.int64).max:
                rank[u] = r
                r += 1
    return rank


class hierarchical_interleaved_bloom_filter:
    def __init__(self, *args, **kwargs):
        self._h = None
        if args or kwargs:
            from .build import build_from_layout

            built = build_from_layout(*args, **kwargs)
            self._adopt(built)

    def _adopt(self, other: "hierarchical_interleaved_bloom_filter") -> None:
        self.__dict__.update(other.__dict__)
        other._h = None

    @classmethod
    def from_tables(cls, n_user_bins, bins, bin_size, hash_funs, next_ibf, user_bin, words=None):
        self = cls.__new__(cls)
        self._h = None
        bins, bsz, hf = _u64(bins), _u64(bin_size), _u64(np.broadcast_to(np.asarray(hash_funs, np.uint64),
                                                                          np.shape(bins)))
        nxt, ub = _u64(next_ibf), _u64(user_bin)
        h = ctypes.c_void_p()
        N.call("hibf_gpu_hibf_create", int(n_user_bins), bins.size, bins.ctypes.data, bsz.ctypes.data,
               hf.ctypes.data, nxt.ctypes.data, ub.ctypes.data, ctypes.byref(h))
        self._h = h
        self.number_of_user_bins = int(n_user_bins)
        self.bins, self.bin_size, self.hash_funs = bins, bsz, hf
        self.next_ibf_id, self.ibf_bin_to_user_bin_id = nxt, ub
        self._rank = None
        if words is not None:
            for k, w in enumerate(words):
                self.set_words(k, w)
        return self

    def save(self, path) -> None:
        """Serialises the device stores and tables in the reference's byte layout (cereal binary encoding)."""
        N.call("hibf_gpu_hibf_save", self._h, str(path).encode())

    @classmethod
    def load(cls, path) -> "hierarchical_interleaved_bloom_filter":
        """Reads a serialised HIBF (as the reference writes it) into new device stores."""
        from .build import _adopt_handle

        h = ctypes.c_void_p()
        N.call("hibf_gpu_hibf_load", str(path).encode(), ctypes.byref(h))
        info = (ctypes.c_uint64 * 4)()
        N.call("hibf_gpu_hibf_info", h, info)
        return _adopt_handle(h, int(info[0]))

    def set_prev(self, prev_ibf, prev_bin) -> None:
        """prev_ibf_id: parent IBF and bin of every IBF (carried through serialisation)."""
        pi, pb = _u64(prev_ibf), _u64(prev_bin)
        N.call("hibf_gpu_hibf_set_prev", self._h, pi.ctypes.data, pb.ctypes.data)

    @property
    def prev_ibf_id(self) -> np.ndarray:
        """prev_ibf_id as an (n_ibfs, 2) array of (parent IBF, parent bin) rows."""
        n = int(self.bins.size)
        pi, pb = np.zeros(n, np.uint64), np.zeros(n, np.uint64)
        N.call("hibf_gpu_hibf_get_prev", self._h, pi.ctypes.data, pb.ctypes.data)
        return np.stack([pi, pb], axis=1)

    def __del__(self):
        if getattr(self, "_h", None):
            try:
                N.lib().hibf_gpu_hibf_destroy(self._h)
            except Exception:
                pass
            self._h = None

    def __eq__(self, other) -> bool:
        """Equal user bin count, tables, IBF shapes and bits (the reference's defaulted operator==,
        hierarchical_interleaved_bloom_filter.hpp:252, 312; its timers always compare equal).  The stores are compared
        IBF by IBF through host copies; the IBFs' occupancy counters are not compared."""
        if not isinstance(other, hierarchical_interleaved_bloom_filter):
            return NotImplemented
        if self.number_of_user_bins != other.number_of_user_bins or self.n_ibfs != other.n_ibfs:
            return False
        for x, y in ((self.bins, other.bins), (self.bin_size, other.bin_size), (self.hash_funs, other.hash_funs),
                     (self.next_ibf_id, other.next_ibf_id), (self.ibf_bin_to_user_bin_id, other.ibf_bin_to_user_bin_id),
                     (self.prev_ibf_id, other.prev_ibf_id)):
            if not np.array_equal(np.asarray(x, np.uint64), np.asarray(y, np.uint64)):
                return False
        return all(np.array_equal(self.words(k), other.words(k)) for k in range(self.n_ibfs))

    __hash__ = None  # mutable, compared by content

    # -- structure --------------------------------------------------------------------------------------------
    @property
    def n_ibfs(self) -> int:
        return int(self.bins.size)

    def info(self) -> dict:
        out = (ctypes.c_uint64 * 4)()
        N.call("hibf_gpu_hibf_info", self._h, out)
        return dict(n_user_bins=out[0], n_ibfs=out[1], max_depth=out[2], device_bytes=out[3])

    def ibf_words(self, k: int) -> int:
        return int((int(self.bins[k]) + 63) // 64 * int(self.bin_size[k]))

    def set_words(self, k: int, words) -> None:
        w = _u64(words)
        N.call("hibf_gpu_hibf_upload_words", self._h, k, w.ctypes.data, w.size)

    def words(self, k: int) -> np.ndarray:
        out = np.zeros(self.ibf_words(k), np.uint64)
        N.call("hibf_gpu_hibf_download_words", self._h, k, out.ctypes.data, out.size)
        return out

    def digests(self, threads: int = 0) -> np.ndarray:
        """Per IBF the hg_digest_step fold of its words in the reference's order (hibf_gpu_hibf_digests)."""
        out = np.zeros(max(self.n_ibfs, 1), np.uint64)
        N.call("hibf_gpu_hibf_digests", self._h, out.ctypes.data, int(threads))
        return out[:self.n_ibfs]

    def build_timers(self) -> dict:
        """The build's phase timers (hierarchical_interleaved_bloom_filter.hpp:283-290): per phase
        (index_allocation, user_bin_io, merge_kmers, fill_ibf) its seconds, longest interval and interval count;
        all zero for an HIBF that was loaded or created from tables."""
        t = (N.Timer * len(N.TIMER_NAMES))()
        N.call("hibf_gpu_hibf_build_timers", self._h, t)
        return {n: {"seconds": t[i].seconds, "max_seconds": t[i].max_seconds, "count": int(t[i].count)}
                for i, n in enumerate(N.TIMER_NAMES)}

    def emplace(self, k: int, values, bin: int) -> None:
        v = _u64(values)
        N.call("hibf_gpu_hibf_emplace", self._h, k, v.ctypes.data, v.size, int(bin))

    def traversal_rank(self) -> np.ndarray:
        if self._rank is None:
            self._rank = traversal_rank(self.number_of_user_bins, self.bins, self.next_ibf_id,
                                        self.ibf_bin_to_user_bin_id)
        return self._rank

    def tables(self) -> dict:
        return dict(n_user_bins=self.number_of_user_bins, bins=self.bins, bin_size=self.bin_size,
                    hash_funs=self.hash_funs, next_ibf=self.next_ibf_id, user_bin=self.ibf_bin_to_user_bin_id)

    # -- agents -----------------------------------------------------------------------------------------------
    def membership_agent(self) -> "membership_agent_type":
        return membership_agent_type(self)

    def counting_agent(self, width: int = 2) -> "counting_agent_type":
        return counting_agent_type(self, width)


class _agent_base:
    def __init__(self, hibf: hierarchical_interleaved_bloom_filter):
        self.hibf = hibf
        a = ctypes.c_void_p()
        N.call("hibf_gpu_agent_create", hibf._h, ctypes.byref(a))
        self._a = a

    def __del__(self):
        if getattr(self, "_a", None):
            try:
                N.lib().hibf_gpu_agent_destroy(self._a)
            except Exception:
                pass
            self._a = None

    def reserve(self, max_queries, max_values, max_tasks, max_results) -> None:
        N.call("hibf_gpu_agent_reserve", self._a, max_queries, max_values, max_tasks, max_results)

    def set_stream(self, stream_ptr: int | None) -> None:
        N.call("hibf_gpu_agent_set_stream", self._a, stream_ptr)

    def last_work(self) -> tuple[int, int]:
        t, v = ctypes.c_uint64(0), ctypes.c_uint64(0)
        N.call("hibf_gpu_agent_last_work", self._a, ctypes.byref(t), ctypes.byref(v))
        return t.value, v.value

    def last_work_executed(self) -> int:
        v = ctypes.c_uint64(0)
        N.call("hibf_gpu_agent_last_work_executed", self._a, ctypes.byref(v))
        return v.value

    def status(self) -> None:
        N.call("hibf_gpu_agent_status", self._a)

    def query_batch(self, values, query_offsets, thresholds, mode=N.QUERY_MEMBERSHIP, width=2, copy=True):
        """All queries in one persistent launch.  Returns (offsets, ids, counts); ids ascending per query; counts
        (mode COUNT) are the non-zero entries of each dense counting vector.  Values in page-locked memory are read
        in place by the kernel; batches of at least 64 MiB of pageable values are copied in chunks while the kernel
        answers the chunks already copied (input_chunks() reports how many).  The arrays are copies, or with
        copy=False views of the agent's page-locked result buffers, valid until the agent's next call (as the
        reference's agents hand out their own result buffers)."""
        v, qo = _u64(values), _u64(query_offsets)
        nq = qo.size - 1
        t = _u64(thresholds)
        ro, ri, rc = N.u64p(), N.u64p(), ctypes.c_void_p()
        N.call("hibf_gpu_agent_query_batch", self._a, mode, v.ctypes.data if v.size else None, qo.ctypes.data, nq,
               t.ctypes.data if nq else None, width, ctypes.byref(ro), ctypes.byref(ri), ctypes.byref(rc))
        offs = np.ctypeslib.as_array(ro, shape=(nq + 1,))
        nr = int(offs[-1])
        ids = np.ctypeslib.as_array(ri, shape=(nr,)) if nr else np.zeros(0, np.uint64)
        cnts = None
        if mode == N.QUERY_COUNT:
            if nr:
                ct = np.ctypeslib.as_ctypes_type(_DT[width])
                cnts = np.ctypeslib.as_array(ctypes.cast(rc, ctypes.POINTER(ct)), shape=(nr,))
            else:
                cnts = np.zeros(0, _DT[width])
        if copy:
            offs, ids = offs.copy(), ids.copy()
            cnts = None if cnts is None else cnts.copy()
        return offs, ids, cnts

    def query_batch_device(self, d_values: int, d_query_offsets: int, n_queries: int, d_thresholds: int,
                           mode=N.QUERY_MEMBERSHIP, width=2):
        """Inputs already on the device (raw pointers, e.g. torch tensor data_ptr()).  Asynchronous on the agent's
        stream; returns device pointers (offsets, ids, counts) into the agent's buffers."""
        ro, ri, rc = N.u64p(), N.u64p(), ctypes.c_void_p()
        N.call("hibf_gpu_agent_query_batch_d", self._a, mode, d_values, d_query_offsets, n_queries, d_thresholds,
               width, ctypes.byref(ro), ctypes.byref(ri), ctypes.byref(rc))
        return (ctypes.cast(ro, ctypes.c_void_p).value, ctypes.cast(ri, ctypes.c_void_p).value, rc.value)

    def capture_batch_device(self, d_values: int, d_query_offsets: int, n_queries: int, d_thresholds: int,
                             mode=N.QUERY_MEMBERSHIP, width=2) -> None:
        """Captures one batch on fixed device buffers into a CUDA graph; replay() launches it."""
        N.call("hibf_gpu_agent_capture_batch_d", self._a, mode, d_values, d_query_offsets, n_queries, d_thresholds,
               width)

    def replay(self) -> None:
        N.call("hibf_gpu_agent_replay", self._a)

    def kernel_ms(self) -> float:
        """Device time of the persistent query kernel of the last batch."""
        ms = ctypes.c_float(0)
        N.call("hibf_gpu_agent_kernel_ms", self._a, ctypes.byref(ms))
        return float(ms.value)

    def input_chunks(self) -> int:
        """Chunks in which the last host batch streamed its values (0: copied whole before the launch)."""
        n = ctypes.c_uint32(0)
        N.call("hibf_gpu_agent_input_chunks", self._a, ctypes.byref(n))
        return int(n.value)

    def level_ms(self) -> list[float]:
        """Per level of the last batch under the level schedule: device ms (root first); [] for the queue."""
        n = ctypes.c_uint32(0)
        out = (ctypes.c_float * 16)()
        N.call("hibf_gpu_agent_level_ms", self._a, out, 16, ctypes.byref(n))
        return [float(out[i]) for i in range(min(n.value, 16))]

    def set_host_read(self, in_place: bool) -> None:
        """Host batches in mapped page-locked memory are read in place by the kernel (the default) or copied first."""
        N.call("hibf_gpu_agent_set_host_read", self._a, int(in_place))

    def last_in_place(self) -> bool:
        """Whether the last host batch was read in place."""
        v = ctypes.c_int(0)
        N.call("hibf_gpu_agent_last_in_place", self._a, ctypes.byref(v))
        return bool(v.value)

    def level_work(self) -> list[dict]:
        """Per level of the last batch under the level schedule: its tasks, value visits and executed value visits
        (root first); [] for the queue."""
        n = ctypes.c_uint32(0)
        t, v, e = (np.zeros(64, np.uint64) for _ in range(3))
        N.call("hibf_gpu_agent_level_work", self._a, t.ctypes.data, v.ctypes.data, e.ctypes.data, 64,
               ctypes.byref(n))
        return [dict(tasks=int(t[i]), value_visits=int(v[i]), value_visits_executed=int(e[i]))
                for i in range(min(n.value, 64))]

    def last_timeline(self) -> list[float]:
        """ms from the last host batch's first device work: each value chunk's copy done, kernel start, kernel end,
        results back in host memory (hibf_gpu_agent_last_timeline)."""
        n = ctypes.c_uint32(0)
        N.call("hibf_gpu_agent_last_timeline", self._a, None, 0, ctypes.byref(n))
        out = (ctypes.c_double * n.value)()
        N.call("hibf_gpu_agent_last_timeline", self._a, out, n.value, ctypes.byref(n))
        return list(out)

    def set_order(self, d_order: int | None, n_queries: int = 0) -> None:
        """Claim order of root tasks for later batches of exactly n_queries queries (device uint32 permutation;
        None: query order)."""
        N.call("hibf_gpu_agent_set_order_d", self._a, d_order, n_queries if d_order else 0)

    def set_work_out(self, d_work: int | None, n_queries: int = 0) -> None:
        """Record each query's executed value visits into a device uint64 array of n_queries entries during later
        batches (None: off)."""
        N.call("hibf_gpu_agent_set_work_out_d", self._a, d_work, n_queries if d_work else 0)

    def query_features(self, d_values: int, d_query_offsets: int, n_queries: int, d_thresholds: int, probe: int,
                       d_features: int) -> None:
        """The learned scheduler's per-query features (float32, 6 per query), asynchronous on the agent's stream."""
        N.call("hibf_gpu_agent_query_features_d", self._a, d_values, d_query_offsets, n_queries, d_thresholds,
               probe, d_features)

    @property
    def tuning(self) -> dict:
        """The persistent kernel's schedule (hibf_gpu_tuning fields)."""
        t = N.Tuning()
        N.call("hibf_gpu_agent_get_tuning", self._a, ctypes.byref(t))
        return t.as_dict()

    @tuning.setter
    def tuning(self, value: dict) -> None:
        t = N.Tuning.from_dict(value)
        N.call("hibf_gpu_agent_set_tuning", self._a, ctypes.byref(t))

    def autotune(self, d_values: int, d_query_offsets: int, n_queries: int, d_thresholds: int,
                 mode=N.QUERY_MEMBERSHIP, width=2, reps=3) -> list[dict]:
        """Times every schedule the search visits on a device-resident sample batch, keeps the fastest on this agent
        and returns the trials [{**tuning, "kernel_ms": ms}] (results are checked identical across schedules)."""
        cap = 64
        trials = (N.TuneTrial * cap)()
        n = ctypes.c_uint64(0)
        N.call("hibf_gpu_agent_autotune", self._a, mode, d_values, d_query_offsets, n_queries, d_thresholds, width,
               reps, trials, cap, ctypes.byref(n))
        return [dict(trials[i].tuning.as_dict(), kernel_ms=trials[i].kernel_ms) for i in range(min(cap, n.value))]

    def fetch_results(self, n_queries: int, mode=N.QUERY_MEMBERSHIP, width=2):
        """Host copies (offsets, ids, counts) of the last device batch (query_batch_device / query_plain_device)."""
        ro, ri, rc = N.u64p(), N.u64p(), ctypes.c_void_p()
        N.call("hibf_gpu_agent_fetch_results", self._a, n_queries, mode, width, ctypes.byref(ro), ctypes.byref(ri),
               ctypes.byref(rc))
        offs = np.ctypeslib.as_array(ro, shape=(n_queries + 1,)).copy()
        nr = int(offs[-1])
        ids = np.ctypeslib.as_array(ri, shape=(nr,)).copy() if nr else np.zeros(0, np.uint64)
        cnts = None
        if mode == N.QUERY_COUNT:
            cnts = np.zeros(nr, _DT[width])
            if nr:
                ctypes.memmove(cnts.ctypes.data, rc.value, nr * width)
        return offs, ids, cnts

    def query_plain_device(self, d_values: int, query_offsets, thresholds, mode=N.QUERY_MEMBERSHIP, width=2):
        """The plain form: one launch per query (values on the device, offsets/thresholds on the host)."""
        qo, t = _u64(query_offsets), _u64(thresholds)
        N.call("hibf_gpu_agent_query_plain_d", self._a, mode, d_values, qo.ctypes.data, qo.size - 1,
               t.ctypes.data if t.size else None, width)


class membership_agent_type(_agent_base):
    def __init__(self, hibf):
        super().__init__(hibf)
        self.result_buffer = np.zeros(0, np.uint64)

    def membership_for(self, values, threshold: int) -> np.ndarray:
        """User bins whose summed counts reach `threshold`, in the reference's traversal order."""
        v = _u64(values)
        ids, n = N.u64p(), ctypes.c_uint64(0)
        N.call("hibf_gpu_agent_membership_for_unsorted", self._a, v.ctypes.data if v.size else None, v.size,
               int(threshold), ctypes.byref(ids), ctypes.byref(n))
        self.result_buffer = np.ctypeslib.as_array(ids, shape=(n.value,)).copy() if n.value else np.zeros(0, np.uint64)
        return self.result_buffer

    def sort_results(self) -> np.ndarray:
        self.result_buffer = np.sort(self.result_buffer)
        return self.result_buffer


class counting_agent_type(_agent_base):
    def __init__(self, hibf, width: int = 2):
        super().__init__(hibf)
        self.width = width

    def bulk_count(self, values, threshold: int) -> np.ndarray:
        """Dense counting vector of number_of_user_bins counters; entries below `threshold` are 0."""
        v = _u64(values)
        p = ctypes.c_void_p()
        N.call("hibf_gpu_agent_bulk_count", self._a, v.ctypes.data if v.size else None, v.size, int(threshold),
               self.width, ctypes.byref(p))
        out = np.zeros(self.hibf.number_of_user_bins, _DT[self.width])
        ctypes.memmove(out.ctypes.data, p.value, out.nbytes)
        return out

    def query_batch(self, values, query_offsets, thresholds, mode=N.QUERY_COUNT, width=None, copy=True):
        return super().query_batch(values, query_offsets, thresholds, mode, self.width if width is None else width,
                                   copy)


def stream_plan(query_offsets) -> np.ndarray:
    """The chunk boundaries (first query of every chunk, then the query count) in which a host batch with these query
    offsets streams its values to the device; fewer than three entries: copied whole (no device needed)."""
    qo = _u64(query_offsets)
    n = ctypes.c_uint64(0)
    N.call("hibf_gpu_stream_plan", qo.ctypes.data, qo.size - 1, None, 0, ctypes.byref(n))
    out = np.zeros(n.value, np.uint64)
    N.call("hibf_gpu_stream_plan", qo.ctypes.data, qo.size - 1, out.ctypes.data if n.value else None, n.value,
           ctypes.byref(n))
    return out


def tune_search(hash_count: int, max_row_words: int, measure) -> tuple[dict, list[dict]]:
    """The autotuner's search with a caller-supplied measure(tuning: dict) -> ms (no device involved): returns the
    fastest schedule and every trial in measurement order."""
    err = []

    def cb(tp, _user, out):
        try:
            out[0] = float(measure(tp.contents.as_dict()))
            return N.OK
        except Exception as e:  # reported through the status code
            err.append(e)
            return N.ERR_INVALID_ARG

    fn = N.TUNE_MEASURE_FN(cb)
    cap = 64
    trials = (N.TuneTrial * cap)()
    n = ctypes.c_uint64(0)
    best = N.Tuning()
    try:
        N.call("hibf_gpu_tune_search", hash_count, max_row_words, fn, None, trials, cap, ctypes.byref(n),
               ctypes.byref(best))
    except N.HibfGpuError:
        if err:
            raise err[0]
        raise
    return best.as_dict(), [dict(trials[i].tuning.as_dict(), kernel_ms=trials[i].kernel_ms)
                            for i in range(min(cap, n.value))]
