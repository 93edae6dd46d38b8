"""ctypes bindings for the two CPU checkers (test infrastructure only).

``Oracle`` wraps oracle/_build/libhibf_oracle.so (the C restatement, hibf_oracle.c).
``Reference`` wraps oracle/_ref/libhibf_ref.so (the reference's own sources + ref_driver.cpp).
Both are built by oracle/Makefile; ``build_oracle()`` / ``build_reference()`` run it.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "_build" / "libhibf_oracle.so"
REF_SO = HERE / "_ref" / "libhibf_ref.so"
# The seqan/hibf source tree: HIBF_REFERENCE_DIR, else a checkout named `reference` beside this repository.
DEFAULT_REF_DIR = os.environ.get("HIBF_REFERENCE_DIR", str(Path(__file__).resolve().parents[2] / "reference"))

u64 = ctypes.c_uint64
vp = ctypes.c_void_p
MERGED = np.uint64(0xFFFFFFFFFFFFFFFF)
DELETED = np.uint64(0xFFFFFFFFFFFFFFFE)


def _ptr(a: np.ndarray | None) -> int | None:
    return None if a is None else a.ctypes.data


def _u64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint64))


def build_oracle() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE), "oracle"], check=True)
    return ORACLE_SO


def reference_available(ref_dir: str = DEFAULT_REF_DIR) -> bool:
    return REF_SO.exists() or (Path(ref_dir) / "src" / "interleaved_bloom_filter.cpp").exists()


def build_reference(ref_dir: str = DEFAULT_REF_DIR, jobs: int = 8) -> Path | None:
    if not (Path(ref_dir) / "src" / "interleaved_bloom_filter.cpp").exists():
        return REF_SO if REF_SO.exists() else None
    subprocess.run(["make", "-s", "-C", str(HERE), f"-j{jobs}", "ref", f"REF_DIR={ref_dir}"], check=True)
    return REF_SO


_WIDTH_DTYPE = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}


# --------------------------------------------------------------------------------------------------------------
# C restatement
# --------------------------------------------------------------------------------------------------------------
class QuerySpec(ctypes.Structure):
    """hg_query_spec (include/hibf_gb300_synthetic.h)."""
    _fields_ = [("seed", u64), ("law", ctypes.c_int), ("len_lo", u64), ("len_hi", u64), ("mix_pct", ctypes.c_uint32),
                ("noise_pct", ctypes.c_uint32), ("thr_num", ctypes.c_uint32), ("thr_den", ctypes.c_uint32),
                ("n_user_bins", u64)]


class Oracle:
    def __init__(self, path: Path = ORACLE_SO):
        if not Path(path).exists():
            build_oracle()
        L = self.lib = ctypes.CDLL(str(path))
        L.orc_ibf_new.restype = vp
        L.orc_ibf_new.argtypes = [u64, u64, u64, ctypes.c_int]
        L.orc_ibf_delete.argtypes = [vp]
        L.orc_ibf_data.restype = ctypes.POINTER(u64)
        L.orc_ibf_data.argtypes = [vp]
        L.orc_ibf_nwords.restype = u64
        L.orc_ibf_nwords.argtypes = [vp]
        L.orc_ibf_emplace_many.argtypes = [vp, vp, vp, u64]
        L.orc_ibf_emplace_one_bin.argtypes = [vp, vp, u64, u64]
        L.orc_ibf_clear.argtypes = [vp, u64]
        L.orc_ibf_clear_range.argtypes = [vp, vp, u64]
        L.orc_ibf_try_increase_bin_number_to.restype = ctypes.c_int
        L.orc_ibf_try_increase_bin_number_to.argtypes = [vp, u64]
        L.orc_ibf_increase_bin_number_to.restype = ctypes.c_int
        L.orc_ibf_increase_bin_number_to.argtypes = [vp, u64]
        L.orc_ibf_bulk_contains_many.argtypes = [vp, vp, u64, vp]
        L.orc_ibf_bulk_count.argtypes = [vp, vp, u64, ctypes.c_int, vp]
        L.orc_ibf_bulk_count_mt.argtypes = [vp, vp, u64, ctypes.c_int, vp, ctypes.c_int]
        L.orc_ibf_bulk_contains_many_mt.argtypes = [vp, vp, u64, vp, ctypes.c_int]
        L.orc_ibf_membership.restype = u64
        L.orc_ibf_membership.argtypes = [vp, vp, u64, ctypes.c_uint16, vp]
        L.orc_hibf_new.restype = vp
        L.orc_hibf_new.argtypes = [u64, u64, vp, vp, vp, vp, vp]
        L.orc_hibf_delete.argtypes = [vp]
        L.orc_hibf_ibf.restype = vp
        L.orc_hibf_ibf.argtypes = [vp, u64]
        L.orc_hibf_membership.restype = u64
        L.orc_hibf_membership.argtypes = [vp, vp, u64, ctypes.c_uint16, ctypes.c_int, vp]
        L.orc_hibf_count.argtypes = [vp, vp, u64, u64, ctypes.c_int, vp]
        L.orc_hibf_query_batch.argtypes = [vp, vp, vp, u64, vp, vp, ctypes.c_int, vp, vp, vp, vp, vp]
        L.orc_hibf_membership_batch.argtypes = [vp, vp, vp, u64, vp, ctypes.c_int, vp, vp, vp]
        L.orc_hibf_run_queries.restype = u64
        L.orc_hibf_run_queries.argtypes = [vp, vp, vp, u64, vp, vp, ctypes.c_int, ctypes.c_int, vp]
        L.orc_hibf_fill_synthetic.restype = ctypes.c_int
        L.orc_hibf_fill_synthetic.argtypes = [vp, u64, vp, u64, vp, vp, vp, vp, vp, vp, vp, ctypes.c_int]
        L.orc_hibf_digests.argtypes = [vp, vp, ctypes.c_int]
        L.orc_synth_user_bin_offsets.argtypes = [u64, ctypes.c_int, ctypes.c_double, ctypes.c_double, u64, u64, u64,
                                                 vp]
        L.orc_synth_queries.argtypes = [ctypes.POINTER(QuerySpec), vp, u64, u64, vp, vp, vp, ctypes.c_int]

    # -- synthetic workloads (include/hibf_gb300_synthetic.h) ---------------------------------------------
    def synth_user_bin_offsets(self, seed, law, p0, p1, lo, hi, n) -> np.ndarray:
        out = np.zeros(n + 1, np.uint64)
        self.lib.orc_synth_user_bin_offsets(seed, law, p0, p1, lo, hi, n, _ptr(out))
        return out

    def synth_query_offsets(self, spec, first, n):
        """(query offsets, thresholds) of queries first .. first+n-1."""
        q = QuerySpec(spec.seed, spec.law, spec.len_lo, spec.len_hi, spec.mix_pct, spec.noise_pct, spec.thr_num,
                      spec.thr_den, spec.n_user_bins)
        qo, thr = np.zeros(n + 1, np.uint64), np.zeros(max(n, 1), np.uint64)
        self.lib.orc_synth_queries(ctypes.byref(q), None, first, n, _ptr(qo), _ptr(thr), None, 0)
        return qo, thr[:n]

    def synth_queries(self, spec, ub_offsets, first, n, threads=0):
        """(values, query offsets, thresholds) of queries first .. first+n-1; `spec` has the fields of
        hg_query_spec (hibf_gb300.synthetic.query_spec)."""
        q = QuerySpec(spec.seed, spec.law, spec.len_lo, spec.len_hi, spec.mix_pct, spec.noise_pct, spec.thr_num,
                      spec.thr_den, spec.n_user_bins)
        o = _u64(ub_offsets)
        qo, thr = np.zeros(n + 1, np.uint64), np.zeros(max(n, 1), np.uint64)
        self.lib.orc_synth_queries(ctypes.byref(q), _ptr(o), first, n, _ptr(qo), _ptr(thr), None, 0)
        v = np.zeros(max(int(qo[-1]), 1), np.uint64)
        self.lib.orc_synth_queries(ctypes.byref(q), _ptr(o), first, n, _ptr(qo), _ptr(thr), _ptr(v),
                                   threads or os.cpu_count())
        return v[:int(qo[-1])], qo, thr[:n]

    # -- IBF ---------------------------------------------------------------------------------------------
    def ibf(self, bins, bin_size, hash_funs=2, track_occupancy=False) -> "OracleIBF":
        return OracleIBF(self, bins, bin_size, hash_funs, track_occupancy)

    def hibf(self, tables: dict) -> "OracleHIBF":
        return OracleHIBF(self, tables)


class OracleIBF:
    def __init__(self, o: Oracle, bins, bin_size, hash_funs, track_occupancy):
        self.o, self.L = o, o.lib
        self.h = self.L.orc_ibf_new(bins, bin_size, hash_funs, int(track_occupancy))
        if not self.h:
            raise ValueError("invalid IBF parameters")
        self.bins = bins
        self.bin_size = bin_size
        self.hash_funs = hash_funs

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_ibf_delete(self.h)
            self.h = None

    @property
    def bin_words(self) -> int:
        return (self.bins + 63) // 64

    def words(self) -> np.ndarray:
        n = self.L.orc_ibf_nwords(self.h)
        p = self.L.orc_ibf_data(self.h)
        return np.ctypeslib.as_array(p, shape=(n,)).copy()

    def set_words(self, w: np.ndarray):
        n = self.L.orc_ibf_nwords(self.h)
        w = _u64(w)
        assert w.size == n
        ctypes.memmove(self.L.orc_ibf_data(self.h), w.ctypes.data, n * 8)

    def emplace(self, values, bins):
        v = _u64(values)
        b = _u64(np.broadcast_to(np.asarray(bins, dtype=np.uint64), v.shape))
        self.L.orc_ibf_emplace_many(self.h, _ptr(v), _ptr(b), v.size)

    def clear(self, bin_):
        self.L.orc_ibf_clear(self.h, int(bin_))

    def clear_range(self, bins):
        b = _u64(bins)
        self.L.orc_ibf_clear_range(self.h, _ptr(b), b.size)

    def try_increase_bin_number_to(self, n) -> bool:
        ok = bool(self.L.orc_ibf_try_increase_bin_number_to(self.h, n))
        if ok:
            self.bins = n
        return ok

    def increase_bin_number_to(self, n):
        rc = self.L.orc_ibf_increase_bin_number_to(self.h, n)
        if rc == -1:
            raise ValueError("The number of new bins must be >= the current number of bins.")
        if rc != 0:
            raise MemoryError
        self.bins = n

    def occupancy(self) -> np.ndarray:
        L = self.L
        L.orc_ibf_occupancy.restype = ctypes.POINTER(u64)
        L.orc_ibf_occupancy.argtypes = [vp]
        return np.ctypeslib.as_array(L.orc_ibf_occupancy(self.h), shape=((self.bins + 63) // 64 * 64,)).copy()

    def data_ptr(self) -> tuple[int, int]:
        """(address, words) of the bit store, to fill it in place (e.g. from a device download)."""
        return ctypes.cast(self.L.orc_ibf_data(self.h), ctypes.c_void_p).value, self.L.orc_ibf_nwords(self.h)

    def bulk_contains(self, values, threads=1) -> np.ndarray:
        v = _u64(values)
        out = np.zeros((v.size, self.bin_words), np.uint64)
        if threads > 1:
            self.L.orc_ibf_bulk_contains_many_mt(self.h, _ptr(v), v.size, _ptr(out), threads)
        else:
            self.L.orc_ibf_bulk_contains_many(self.h, _ptr(v), v.size, _ptr(out))
        return out

    def bulk_count(self, values, width=2, threads=1) -> np.ndarray:
        v = _u64(values)
        out = np.zeros(self.bins, _WIDTH_DTYPE[width])
        if threads > 1:
            self.L.orc_ibf_bulk_count_mt(self.h, _ptr(v), v.size, width, _ptr(out), threads)
        else:
            self.L.orc_ibf_bulk_count(self.h, _ptr(v), v.size, width, _ptr(out))
        return out

    def membership_for(self, values, threshold) -> np.ndarray:
        v = _u64(values)
        out = np.zeros(self.bins, np.uint64)
        m = self.L.orc_ibf_membership(self.h, _ptr(v), v.size, threshold, _ptr(out))
        return out[:m]


class OracleHIBF:
    """tables: n_user_bins, bins[k], bin_size[k], hash_funs[k], next_ibf (flat), user_bin (flat), words[k]."""

    def __init__(self, o: Oracle, t: dict):
        self.o, self.L = o, o.lib
        bins = _u64(t["bins"])
        self.n_ibfs = bins.size
        self.n_user_bins = int(t["n_user_bins"])
        self._keep = [bins, _u64(t["bin_size"]), _u64(t["hash_funs"]), _u64(t["next_ibf"]), _u64(t["user_bin"])]
        self.h = self.L.orc_hibf_new(self.n_ibfs, self.n_user_bins, *[_ptr(a) for a in self._keep])
        if not self.h:
            raise ValueError("invalid HIBF tables")
        if "words" in t:
            for k, w in enumerate(t["words"]):
                self.set_words(k, w)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_hibf_delete(self.h)
            self.h = None

    def _ibf_ptr(self, k):
        return self.L.orc_hibf_ibf(self.h, k)

    def set_words(self, k, w):
        p = self._ibf_ptr(k)
        n = self.L.orc_ibf_nwords(p)
        w = _u64(w)
        assert w.size == n, (w.size, n)
        ctypes.memmove(self.L.orc_ibf_data(p), w.ctypes.data, n * 8)

    def data_ptr(self, k) -> tuple[int, int]:
        """(address, word count) of IBF k's bit store, for filling it in place."""
        p = self._ibf_ptr(k)
        return ctypes.cast(self.L.orc_ibf_data(p), ctypes.c_void_p).value, int(self.L.orc_ibf_nwords(p))

    def words(self, k) -> np.ndarray:
        p = self._ibf_ptr(k)
        n = self.L.orc_ibf_nwords(p)
        return np.ctypeslib.as_array(self.L.orc_ibf_data(p), shape=(n,)).copy()

    def emplace(self, k, values, bin_):
        v = _u64(values)
        self.L.orc_ibf_emplace_one_bin(self._ibf_ptr(k), _ptr(v), v.size, int(bin_))

    def fill_synthetic(self, seed, offsets, split, threads=0):
        """Every synthetic user bin into its technical bins (split ones chunked by the split-table arrays `split`,
        the fields of hibf_gb300.build.SPLIT_TABLE_FIELDS) and into every ancestor's merged bin."""
        o = _u64(offsets)
        a = {k: _u64(split[k]) for k in ("user_bin", "mult", "mask", "bnd_off", "bnd_home", "before_off", "before")}
        rc = self.L.orc_hibf_fill_synthetic(self.h, int(seed), _ptr(o), a["user_bin"].size,
                                            *[_ptr(a[k]) for k in ("user_bin", "mult", "mask", "bnd_off",
                                                                   "bnd_home", "before_off", "before")],
                                            threads or os.cpu_count())
        if rc != 0:
            raise ValueError(f"orc_hibf_fill_synthetic: {rc}")

    def digests(self, threads=0) -> np.ndarray:
        out = np.zeros(max(self.n_ibfs, 1), np.uint64)
        self.L.orc_hibf_digests(self.h, _ptr(out), threads or os.cpu_count())
        return out[:self.n_ibfs]

    def membership_for(self, values, threshold, sort=True) -> np.ndarray:
        v = _u64(values)
        out = np.zeros(self.n_user_bins, np.uint64)
        m = self.L.orc_hibf_membership(self.h, _ptr(v), v.size, threshold, int(sort), _ptr(out))
        return out[:m]

    def bulk_count(self, values, threshold, width=2) -> np.ndarray:
        v = _u64(values)
        out = np.zeros(self.n_user_bins, _WIDTH_DTYPE[width])
        self.L.orc_hibf_count(self.h, _ptr(v), v.size, threshold, width, _ptr(out))
        return out

    def query_batch(self, values, qoffsets, mem_t, cnt_t, threads=0):
        v, qo = _u64(values), _u64(qoffsets)
        nq = qo.size - 1
        mt = np.ascontiguousarray(np.asarray(mem_t, dtype=np.uint16))
        ct = _u64(cnt_t)
        res = {k: np.zeros(nq, np.uint64) for k in ("mem_len", "mem_digest", "cnt_nnz", "cnt_digest", "visits")}
        self.L.orc_hibf_query_batch(self.h, _ptr(v), _ptr(qo), nq, _ptr(mt), _ptr(ct), threads or os.cpu_count(),
                                    *[_ptr(res[k]) for k in ("mem_len", "mem_digest", "cnt_nnz", "cnt_digest",
                                                             "visits")])
        return res

    def membership_batch(self, values, qoffsets, thresholds, threads=0):
        v, qo = _u64(values), _u64(qoffsets)
        nq = qo.size - 1
        t = np.ascontiguousarray(np.asarray(thresholds, dtype=np.uint16))
        lengths = np.zeros(nq, np.uint64)
        th = threads or os.cpu_count()
        self.L.orc_hibf_membership_batch(self.h, _ptr(v), _ptr(qo), nq, _ptr(t), th, _ptr(lengths), None, None)
        offs = np.zeros(nq + 1, np.uint64)
        np.cumsum(lengths, out=offs[1:])
        ids = np.zeros(int(offs[-1]), np.uint64)
        self.L.orc_hibf_membership_batch(self.h, _ptr(v), _ptr(qo), nq, _ptr(t), th, _ptr(lengths), _ptr(offs),
                                         _ptr(ids))
        return offs, ids

    def run_queries(self, values, qoffsets, mem_t, cnt_t, mode=1, threads=0):
        v, qo = _u64(values), _u64(qoffsets)
        mt = np.ascontiguousarray(np.asarray(mem_t, dtype=np.uint16))
        ct = _u64(cnt_t)
        chk = np.zeros(1, np.uint64)
        pairs = self.L.orc_hibf_run_queries(self.h, _ptr(v), _ptr(qo), qo.size - 1, _ptr(mt), _ptr(ct), mode,
                                            threads or os.cpu_count(), _ptr(chk))
        return int(pairs), int(chk[0])


# --------------------------------------------------------------------------------------------------------------
# The reference itself
# --------------------------------------------------------------------------------------------------------------
class RefCfg(ctypes.Structure):
    _fields_ = [("number_of_user_bins", u64), ("number_of_hash_functions", u64), ("maximum_fpr", ctypes.c_double),
                ("relaxed_fpr", ctypes.c_double), ("threads", u64), ("sketch_bits", u64), ("tmax", u64),
                ("alpha", ctypes.c_double), ("max_rearrangement_ratio", ctypes.c_double),
                ("disable_estimate_union", ctypes.c_int), ("disable_rearrangement", ctypes.c_int),
                ("track_occupancy", ctypes.c_int), ("empty_bin_fraction", ctypes.c_double)]


def ref_cfg(n_user_bins, h=2, fpr=0.05, relaxed_fpr=0.3, threads=1, sketch_bits=12, tmax=0, alpha=1.2,
            max_rearrangement_ratio=0.5, disable_estimate_union=False, disable_rearrangement=False,
            track_occupancy=False, empty_bin_fraction=0.0) -> RefCfg:
    return RefCfg(n_user_bins, h, fpr, relaxed_fpr, threads, sketch_bits, tmax, alpha, max_rearrangement_ratio,
                  int(disable_estimate_union), int(disable_rearrangement), int(track_occupancy),
                  float(empty_bin_fraction))


class Reference:
    def __init__(self, path: Path = REF_SO):
        if not Path(path).exists():
            if build_reference() is None:
                raise FileNotFoundError("reference library not available")
        L = self.lib = ctypes.CDLL(str(path))
        cfgp = ctypes.POINTER(RefCfg)
        L.ref_free.argtypes = [vp]
        L.ref_ibf_new.restype = vp
        L.ref_ibf_new.argtypes = [u64, u64, u64, ctypes.c_int]
        L.ref_ibf_from_config.restype = vp
        L.ref_ibf_from_config.argtypes = [cfgp, vp, vp, u64]
        L.ref_ibf_free.argtypes = [vp]
        L.ref_ibf_params.argtypes = [vp, vp]
        L.ref_ibf_emplace.argtypes = [vp, vp, vp, u64]
        L.ref_ibf_clear.argtypes = [vp, u64]
        L.ref_ibf_clear_range.argtypes = [vp, vp, u64]
        L.ref_ibf_try_increase_bin_number_to.restype = ctypes.c_int
        L.ref_ibf_try_increase_bin_number_to.argtypes = [vp, u64]
        L.ref_ibf_increase_bin_number_to.restype = ctypes.c_int
        L.ref_ibf_increase_bin_number_to.argtypes = [vp, u64]
        L.ref_ibf_nwords.restype = u64
        L.ref_ibf_nwords.argtypes = [vp]
        L.ref_ibf_words.argtypes = [vp, vp]
        L.ref_ibf_occupancy.restype = u64
        L.ref_ibf_occupancy.argtypes = [vp, vp]
        L.ref_ibf_bulk_contains.argtypes = [vp, vp, u64, vp]
        L.ref_ibf_bulk_count.argtypes = [vp, vp, u64, ctypes.c_int, vp]
        L.ref_ibf_membership.restype = u64
        L.ref_ibf_membership.argtypes = [vp, vp, u64, ctypes.c_uint16, vp]
        L.ref_layout.restype = ctypes.c_void_p
        L.ref_layout.argtypes = [cfgp, vp, vp, u64, ctypes.c_int]
        L.ref_hibf_new.restype = vp
        L.ref_hibf_new.argtypes = [cfgp, vp, vp, u64, ctypes.c_int, ctypes.c_char_p]
        L.ref_hibf_free.argtypes = [vp]
        L.ref_hibf_num_ibfs.restype = u64
        L.ref_hibf_num_ibfs.argtypes = [vp]
        L.ref_hibf_ibf_params.argtypes = [vp, u64, vp]
        L.ref_hibf_ibf_words.argtypes = [vp, u64, vp]
        L.ref_hibf_ibf_digest.restype = u64
        L.ref_hibf_ibf_digest.argtypes = [vp, u64]
        L.ref_hibf_tables.argtypes = [vp, u64, vp, vp]
        L.ref_hibf_membership.restype = u64
        L.ref_hibf_membership.argtypes = [vp, vp, u64, ctypes.c_uint16, ctypes.c_int, vp]
        L.ref_hibf_count.argtypes = [vp, vp, u64, u64, ctypes.c_int, vp]
        L.ref_hibf_query_batch.argtypes = [vp, vp, vp, u64, vp, vp, ctypes.c_int, vp, vp, vp, vp, vp]

    # -- IBF ---------------------------------------------------------------------------------------------
    def ibf(self, bins, bin_size, hash_funs=2, track_occupancy=False) -> "RefIBF":
        return RefIBF(self, self.lib.ref_ibf_new(bins, bin_size, hash_funs, int(track_occupancy)))

    def ibf_from_config(self, cfg: RefCfg, values, offsets, max_bin_elements=0) -> "RefIBF":
        v, o = _u64(values), _u64(offsets)
        return RefIBF(self, self.lib.ref_ibf_from_config(ctypes.byref(cfg), _ptr(v), _ptr(o), max_bin_elements))

    # -- layout / HIBF -----------------------------------------------------------------------------------
    def ibf_load(self, data: bytes) -> "RefIBF":
        """The reference's load of bytes in that encoding (its serialize() with an input archive)."""
        L = self.lib
        L.ref_ibf_load.restype = vp
        L.ref_ibf_load.argtypes = [ctypes.c_char_p, u64]
        return RefIBF(self, L.ref_ibf_load(data, len(data)))

    def hll(self, values, bits):
        """The reference's hyperloglog over `values`: (registers, estimate)."""
        L = self.lib
        L.ref_hll.restype = ctypes.c_int
        L.ref_hll.argtypes = [vp, u64, ctypes.c_uint32, vp, ctypes.POINTER(ctypes.c_double)]
        v = _u64(values)
        regs = np.zeros(1 << bits, np.uint8)
        e = ctypes.c_double(0)
        if L.ref_hll(_ptr(v), v.size, bits, _ptr(regs), ctypes.byref(e)) != 0:
            raise RuntimeError("reference hyperloglog failed")
        return regs, e.value

    def layout(self, cfg: RefCfg, values=None, offsets=None, seed=0, synthetic=False) -> str:
        v = None if values is None else _u64(values)
        o = _u64(offsets)
        p = self.lib.ref_layout(ctypes.byref(cfg), _ptr(v), _ptr(o), seed, int(synthetic))
        if not p:
            raise RuntimeError("reference layout computation failed")
        s = ctypes.string_at(p).decode()
        self.lib.ref_free(p)
        return s

    def hibf(self, cfg: RefCfg, values=None, offsets=None, seed=0, synthetic=False, layout: str | None = None):
        v = None if values is None else _u64(values)
        o = _u64(offsets)
        p = self.lib.ref_hibf_new(ctypes.byref(cfg), _ptr(v), _ptr(o), seed, int(synthetic),
                                  None if layout is None else layout.encode())
        if not p:
            raise RuntimeError("reference HIBF construction failed")
        return RefHIBF(self, p, int(cfg.number_of_user_bins))


class RefIBF:
    def __init__(self, r: Reference, h):
        if not h:
            raise ValueError("invalid IBF parameters")
        self.r, self.L, self.h = r, r.lib, h
        p = np.zeros(4, np.uint64)
        self.L.ref_ibf_params(h, _ptr(p))
        self.bins, self.bin_size, self.hash_funs, self.bit_size = (int(x) for x in p)

    def save(self) -> bytes:
        """The reference's serialize() through a cereal-binary-encoding byte archive (oracle/ref_driver.cpp)."""
        return _ref_bytes(self.L, "ref_ibf_save", self.h)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.ref_ibf_free(self.h)
            self.h = None

    @property
    def bin_words(self):
        return (self.bins + 63) // 64

    def _refresh(self):
        p = np.zeros(4, np.uint64)
        self.L.ref_ibf_params(self.h, _ptr(p))
        self.bins, self.bin_size, self.hash_funs, self.bit_size = (int(x) for x in p)

    def words(self):
        out = np.zeros(self.L.ref_ibf_nwords(self.h), np.uint64)
        self.L.ref_ibf_words(self.h, _ptr(out))
        return out

    def occupancy(self):
        n = self.L.ref_ibf_occupancy(self.h, None)
        out = np.zeros(n, np.uint64)
        self.L.ref_ibf_occupancy(self.h, _ptr(out))
        return out

    def emplace(self, values, bins):
        v = _u64(values)
        b = _u64(np.broadcast_to(np.asarray(bins, dtype=np.uint64), v.shape))
        self.L.ref_ibf_emplace(self.h, _ptr(v), _ptr(b), v.size)

    def clear(self, b):
        self.L.ref_ibf_clear(self.h, int(b))

    def clear_range(self, bins):
        b = _u64(bins)
        self.L.ref_ibf_clear_range(self.h, _ptr(b), b.size)

    def try_increase_bin_number_to(self, n):
        ok = bool(self.L.ref_ibf_try_increase_bin_number_to(self.h, n))
        self._refresh()
        return ok

    def increase_bin_number_to(self, n):
        rc = self.L.ref_ibf_increase_bin_number_to(self.h, n)
        self._refresh()
        if rc != 0:
            raise ValueError("The number of new bins must be >= the current number of bins.")

    def bulk_contains(self, values):
        v = _u64(values)
        out = np.zeros((v.size, self.bin_words), np.uint64)
        self.L.ref_ibf_bulk_contains(self.h, _ptr(v), v.size, _ptr(out))
        return out

    def bulk_count(self, values, width=2):
        v = _u64(values)
        out = np.zeros(self.bins, _WIDTH_DTYPE[width])
        self.L.ref_ibf_bulk_count(self.h, _ptr(v), v.size, width, _ptr(out))
        return out

    def membership_for(self, values, threshold):
        v = _u64(values)
        out = np.zeros(self.bins, np.uint64)
        m = self.L.ref_ibf_membership(self.h, _ptr(v), v.size, threshold, _ptr(out))
        return out[:m]


def _ref_bytes(L, fn, h) -> bytes:
    f = getattr(L, fn)
    f.restype = vp
    f.argtypes = [vp, ctypes.POINTER(u64)]
    n = u64(0)
    p = f(h, ctypes.byref(n))
    if not p:
        raise RuntimeError(f"{fn} failed")
    out = ctypes.string_at(p, n.value)
    L.ref_free(p)
    return out


class RefHIBF:
    def __init__(self, r: Reference, h, n_user_bins):
        self.r, self.L, self.h, self.n_user_bins = r, r.lib, h, n_user_bins

    def save(self) -> bytes:
        """The reference's serialize() through a cereal-binary-encoding byte archive (oracle/ref_driver.cpp)."""
        return _ref_bytes(self.L, "ref_hibf_save", self.h)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.ref_hibf_free(self.h)
            self.h = None

    def tables(self, with_words=True) -> dict:
        """Flat tables in the reference's own IBF numbering."""
        n = self.L.ref_hibf_num_ibfs(self.h)
        bins, bsz, hf, prev_ibf, prev_bin, digests, words, nxt, ub = [], [], [], [], [], [], [], [], []
        p = np.zeros(6, np.uint64)
        for k in range(n):
            self.L.ref_hibf_ibf_params(self.h, k, _ptr(p))
            bins.append(int(p[0]))
            bsz.append(int(p[1]))
            hf.append(int(p[2]))
            prev_ibf.append(int(p[4]))
            prev_bin.append(int(p[5]))
            digests.append(self.L.ref_hibf_ibf_digest(self.h, k))
            a, b = np.zeros(int(p[0]), np.uint64), np.zeros(int(p[0]), np.uint64)
            self.L.ref_hibf_tables(self.h, k, _ptr(a), _ptr(b))
            nxt.append(a)
            ub.append(b)
            if with_words:
                w = np.zeros(int(p[3]), np.uint64)
                self.L.ref_hibf_ibf_words(self.h, k, _ptr(w))
                words.append(w)
        t = dict(n_user_bins=self.n_user_bins, bins=np.array(bins, np.uint64), bin_size=np.array(bsz, np.uint64),
                 hash_funs=np.array(hf, np.uint64), next_ibf=np.concatenate(nxt), user_bin=np.concatenate(ub),
                 digests=np.array(digests, np.uint64), prev_ibf=np.array(prev_ibf, np.uint64),
                 prev_bin=np.array(prev_bin, np.uint64))
        if with_words:
            t["words"] = words
        return t

    def membership_for(self, values, threshold, sort=True):
        v = _u64(values)
        out = np.zeros(self.n_user_bins, np.uint64)
        m = self.L.ref_hibf_membership(self.h, _ptr(v), v.size, threshold, int(sort), _ptr(out))
        return out[:m]

    def bulk_count(self, values, threshold, width=2):
        v = _u64(values)
        out = np.zeros(self.n_user_bins, _WIDTH_DTYPE[width])
        self.L.ref_hibf_count(self.h, _ptr(v), v.size, threshold, width, _ptr(out))
        return out

    def query_batch(self, values, qoffsets, mem_t, cnt_t, threads=0, with_lists=False):
        v, qo = _u64(values), _u64(qoffsets)
        nq = qo.size - 1
        mt = np.ascontiguousarray(np.asarray(mem_t, dtype=np.uint16))
        ct = _u64(cnt_t)
        res = {k: np.zeros(nq, np.uint64) for k in ("mem_len", "mem_digest", "cnt_nnz", "cnt_digest")}
        lists = np.zeros(nq * self.n_user_bins, np.uint64) if with_lists else None
        self.L.ref_hibf_query_batch(self.h, _ptr(v), _ptr(qo), nq, _ptr(mt), _ptr(ct), threads or os.cpu_count(),
                                    *[_ptr(res[k]) for k in ("mem_len", "mem_digest", "cnt_nnz", "cnt_digest")],
                                    _ptr(lists))
        if with_lists:
            res["lists"] = lists.reshape(nq, self.n_user_bins)
        return res
