"""Continuous-batching query server over a resident HIBF (hibf_gpu_server_* in the C ABI).

    srv = server(hibf, slots=4, max_batch_queries=65536, max_batch_values=1 << 26, admission_bytes=4 << 30)
    rid = srv.submit(values, query_offsets, thresholds)
    status, offsets, ids, latency_s = srv.wait_result(rid, n_queries)
    stats = srv.open_loop(pool_values, pool_offsets, offered_qps=1e5, duration_s=1.0)

Requests arriving while batches run are admitted as slots and admission memory free up; their batches overlap on
the device.  Each request's results equal the same queries answered alone.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N


def _u64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint64).reshape(-1))


class server:
    def __init__(self, hibf, slots: int = 4, max_batch_queries: int = 65536, max_batch_values: int = 1 << 26,
                 admission_bytes: int = 4 << 30):
        self._s = None
        self.hibf = hibf  # keeps the HIBF alive
        s = ctypes.c_void_p()
        N.call("hibf_gpu_server_create", hibf._h, slots, max_batch_queries, max_batch_values, admission_bytes,
               ctypes.byref(s))
        self._s = s

    def close(self) -> None:
        if getattr(self, "_s", None):
            N.call("hibf_gpu_server_destroy", self._s)
            self._s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, values, query_offsets, thresholds, arrival_s: float = -1.0) -> int:
        v, qo, t = _u64(values), _u64(query_offsets), _u64(thresholds)
        rid = ctypes.c_uint64(0)
        N.call("hibf_gpu_server_submit", self._s, v.ctypes.data if v.size else None, qo.ctypes.data, qo.size - 1,
               t.ctypes.data if t.size else None, arrival_s, 1, ctypes.byref(rid))
        return rid.value

    def register_host(self, ptr: int, nbytes: int, already_pinned: bool = False) -> None:
        """Registers host memory for borrowed requests: their values are then copied to the device without staging."""
        N.call("hibf_gpu_server_register_host", self._s, ptr, nbytes, int(already_pinned))

    def set_zero_copy(self, on: bool) -> None:
        """Batches of back-to-back borrowed requests in one mapped registered range are read in place (default on)."""
        N.call("hibf_gpu_server_set_zero_copy", self._s, int(on))

    def unregister_host(self, ptr: int) -> None:
        N.call("hibf_gpu_server_unregister_host", self._s, ptr)

    def submit_borrowed(self, values_ptr: int, query_offsets, thresholds, arrival_s: float = -1.0) -> int:
        """Submits without copying: the server reads `values_ptr` (values inside a registered range go to the device
        directly) and the offsets/thresholds arrays until release().  Keep all three alive until then."""
        qo, t = _u64(query_offsets), _u64(thresholds)
        rid = ctypes.c_uint64(0)
        N.call("hibf_gpu_server_submit", self._s, values_ptr, qo.ctypes.data, qo.size - 1,
               t.ctypes.data if t.size else None, arrival_s, 0, ctypes.byref(rid))
        return rid.value

    def wait(self, rid: int, timeout_ms: float = -1.0):
        """(status, offsets pointer, ids pointer, latency_s); the pointers stay valid until release(rid)."""
        st = ctypes.c_int(0)
        ro, ri = N.u64p(), N.u64p()
        lat = ctypes.c_double(0)
        N.call("hibf_gpu_server_wait", self._s, rid, timeout_ms, ctypes.byref(st), ctypes.byref(ro),
               ctypes.byref(ri), ctypes.byref(lat))
        return st.value, ro, ri, lat.value

    def release(self, rid: int) -> None:
        N.call("hibf_gpu_server_release", self._s, rid)

    def wait_result(self, rid: int, n_queries: int, timeout_ms: float = -1.0):
        """(status, offsets (n_queries + 1), ids, latency_s) as numpy copies; releases the request."""
        st, ro, ri, lat = self.wait(rid, timeout_ms)
        offs = ids = None
        if st == N.OK:
            offs = np.ctypeslib.as_array(ro, shape=(n_queries + 1,)).copy()
            nr = int(offs[-1])
            ids = np.ctypeslib.as_array(ri, shape=(nr,)).copy() if nr else np.zeros(0, np.uint64)
        N.call("hibf_gpu_server_release", self._s, rid)
        return st, offs, ids, lat

    def stats(self) -> dict:
        out = (ctypes.c_uint64 * 4)()
        N.call("hibf_gpu_server_stats", self._s, out)
        return dict(batches=out[0], batched_queries=out[1], rejected=out[2], inflight_bytes=out[3])

    def phase_times(self) -> dict:
        """Mean milliseconds per batch: queueing, staging + launch, device work, result fetch, split."""
        out = (ctypes.c_double * 5)()
        N.call("hibf_gpu_server_phase_times", self._s, out)
        return dict(zip(("queue_ms", "stage_ms", "device_ms", "fetch_ms", "split_ms"), (x * 1e3 for x in out)))

    def batch_log(self) -> np.ndarray:
        """Per batch: oldest arrival, slot start, launched, device done, fetched, finished (s), queries, values,
        device time of the input copies and of the query kernel (s), values staged through the slot's pinned
        buffer, 1 if the kernel read the values in place (zero copy)."""
        n = ctypes.c_uint64(0)
        N.call("hibf_gpu_server_batch_log", self._s, None, 0, ctypes.byref(n))
        out = np.zeros(max(n.value, 1) * 12, np.float64)
        N.call("hibf_gpu_server_batch_log", self._s, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), n.value,
               ctypes.byref(n))
        return out[:n.value * 12].reshape(n.value, 12)

    def tail_phases(self, quantile: float = 0.99) -> dict:
        """Phase times (ms) of the batches whose oldest request waited longest (the top 1 - quantile share), beside
        the median batch: where the latency tail comes from."""
        log = self.batch_log()
        if log.shape[0] == 0:
            return {}
        ph = np.stack([log[:, 1] - log[:, 0], log[:, 2] - log[:, 1], log[:, 3] - log[:, 2], log[:, 4] - log[:, 3],
                       log[:, 5] - log[:, 4], log[:, 8], log[:, 9]], axis=1) * 1e3
        total = log[:, 5] - log[:, 0]
        cut = np.quantile(total, quantile)
        tail = ph[total >= cut]
        names = ("queue_ms", "stage_ms", "device_ms", "fetch_ms", "split_ms", "copy_in_ms", "kernel_ms")
        return {"batches": int(log.shape[0]), "tail_batches": int(tail.shape[0]),
                "median_batch": dict(zip(names, np.median(ph, axis=0).round(4).tolist())),
                "tail_mean": dict(zip(names, tail.mean(axis=0).round(4).tolist())),
                "tail_queries_mean": float(log[total >= cut, 6].mean()),
                "tail_staged_share": float(log[total >= cut, 10].sum() / max(log[total >= cut, 7].sum(), 1.0)),
                "zero_copy_batches_share": float(log[:, 11].mean()),
                "median_queries": float(np.median(log[:, 6]))}

    def open_loop(self, pool_values, pool_offsets, offered_qps: float, duration_s: float = 1.0,
                  max_request_queries: int = 4096, thr_lo: float = 0.5, thr_hi: float = 0.9, seed: int = 1) -> dict:
        v, qo = _u64(pool_values), _u64(pool_offsets)
        out = (ctypes.c_double * 8)()
        N.call("hibf_gpu_server_open_loop", self._s, v.ctypes.data, qo.ctypes.data, qo.size - 1, offered_qps,
               duration_s, max_request_queries, thr_lo, thr_hi, seed, out)
        det = (ctypes.c_double * 5)()
        N.call("hibf_gpu_server_open_loop_detail", self._s, det)
        return dict(offered_qps=offered_qps, achieved_qps=out[0], p50_ms=out[1] * 1e3, p99_ms=out[2] * 1e3,
                    p999_ms=out[3] * 1e3, requests=int(out[4]), queries=int(out[5]), rejected=int(out[6]),
                    mean_batch_queries=out[7], duration_s=duration_s,
                    # the load generator: how late it submitted, and latency counted from the actual submission
                    generator_late_max_ms=det[0] * 1e3, generator_late_p999_ms=det[1] * 1e3,
                    generator_late_over_1ms=int(det[2]), p99_from_submit_ms=det[3] * 1e3,
                    p999_from_submit_ms=det[4] * 1e3)
