"""ctypes binding of the C ABI in include/hibf_gb300.h (libhibf_gb300.so, built in-tree by hibf_gb300._build).

There is no CPU fallback: ``lib()`` raises when the shared library is missing, and every entry point that needs a
GPU returns HIBF_GPU_ERR_NO_DEVICE, which ``check`` turns into an exception.
"""

from __future__ import annotations

import ctypes
import os
from pathlib import Path

LIB_PATH = Path(os.environ.get("HIBF_GB300_LIB", Path(__file__).resolve().parent / "_lib" / "libhibf_gb300.so"))

u64 = ctypes.c_uint64
u64p = ctypes.POINTER(ctypes.c_uint64)
vp = ctypes.c_void_p
ci = ctypes.c_int

OK = 0
ERR_INVALID_ARG = 1
ERR_LOGIC = 2
ERR_OUT_OF_MEMORY = 3
ERR_NO_DEVICE = 4
ERR_CUDA = 5
ERR_OVERFLOW = 6
ERR_TIMEOUT = 7
ERR_ADMISSION = 8
ERR_CYCLE = 9

QUERY_MEMBERSHIP = 1
QUERY_COUNT = 2
SCHEDULE_QUEUE = 0
SCHEDULE_LEVELS = 1
EARLY_EXIT_ADAPTIVE = 0xFFFFFFFF  # hibf_gpu_tuning.early_exit_stages: checks where the outcome can first change

BIN_MERGED = (1 << 64) - 1
BIN_DELETED = (1 << 64) - 2


class HibfGpuError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"[status {status}] {msg}")
        self.status = status


class LogicError(HibfGpuError, ValueError):
    """std::logic_error of the reference (invalid IBF construction arguments)."""


class InvalidArgument(HibfGpuError, ValueError):
    """std::invalid_argument of the reference."""


class BuildConfig(ctypes.Structure):
    """hibf_gpu_build_config (the fields of seqan::hibf::config the build uses)."""

    _fields_ = [("number_of_user_bins", u64), ("number_of_hash_functions", u64), ("maximum_fpr", ctypes.c_double),
                ("relaxed_fpr", ctypes.c_double), ("threads", u64), ("user_bins_disjoint", ci)]


INPUT_FN = ctypes.CFUNCTYPE(None, vp, u64, vp)


class Tuning(ctypes.Structure):
    """hibf_gpu_tuning: schedule of the persistent query kernel (results never depend on it)."""

    _fields_ = [(n, ctypes.c_uint32) for n in ("values_per_lane", "fetch_bytes", "counter_bits", "blocks_per_sm",
                                                 "early_exit_first", "early_exit_step", "early_exit_stages",
                                                 "early_exit_min", "block_queries", "schedule",
                                                 "level_values_per_lane")]

    def as_dict(self) -> dict:
        return {n: int(getattr(self, n)) for n, _ in self._fields_}

    @classmethod
    def from_dict(cls, d: dict) -> "Tuning":
        t = cls()
        lib().hibf_gpu_tuning_default(ctypes.byref(t))
        for k, v in d.items():
            setattr(t, k, int(v))
        return t


class Timer(ctypes.Structure):
    """hibf_gpu_timer: one build phase's seconds, longest interval and interval count."""

    _fields_ = [("seconds", ctypes.c_double), ("max_seconds", ctypes.c_double), ("count", u64)]


TIMER_NAMES = ("index_allocation", "user_bin_io", "merge_kmers", "fill_ibf")


class TuneTrial(ctypes.Structure):
    _fields_ = [("tuning", Tuning), ("kernel_ms", ctypes.c_double)]


TUNE_MEASURE_FN = ctypes.CFUNCTYPE(ci, ctypes.POINTER(Tuning), vp, ctypes.POINTER(ctypes.c_double))

# (name, restype, argtypes); restype None means the int status convention, "void" no result.
_SIGS = [
    ("hibf_gpu_last_error", ctypes.c_char_p, []),
    ("hibf_gpu_abi_version", ci, []),
    ("hibf_gpu_device_count", None, [ctypes.POINTER(ci)]),
    ("hibf_gpu_ibf_create", None, [u64, u64, u64, ci, ctypes.POINTER(vp)]),
    ("hibf_gpu_ibf_destroy", None, [vp]),
    ("hibf_gpu_ibf_info", None, [vp, u64p]),
    ("hibf_gpu_ibf_emplace", None, [vp, vp, u64, u64]),
    ("hibf_gpu_ibf_emplace_binned", None, [vp, vp, vp, u64]),
    ("hibf_gpu_ibf_emplace_d", None, [vp, vp, vp, u64, u64, vp]),
    ("hibf_gpu_ibf_clear", None, [vp, u64]),
    ("hibf_gpu_ibf_clear_range", None, [vp, vp, u64]),
    ("hibf_gpu_ibf_try_increase_bin_number_to", None, [vp, u64, ctypes.POINTER(ci)]),
    ("hibf_gpu_ibf_increase_bin_number_to", None, [vp, u64]),
    ("hibf_gpu_ibf_bulk_contains", None, [vp, vp, u64, vp]),
    ("hibf_gpu_ibf_bulk_contains_d", None, [vp, vp, u64, vp, vp]),
    ("hibf_gpu_ibf_bulk_count", None, [vp, vp, u64, ci, vp]),
    ("hibf_gpu_ibf_bulk_count_d", None, [vp, vp, u64, ci, vp, vp]),
    ("hibf_gpu_ibf_bulk_count_noalloc_d", None, [vp, vp, u64, ci, vp, vp]),
    ("hibf_gpu_ibf_membership_for", None, [vp, vp, u64, ctypes.c_uint16, vp, u64p]),
    ("hibf_gpu_ibf_upload_words", None, [vp, vp, u64]),
    ("hibf_gpu_ibf_download_words", None, [vp, vp, u64]),
    ("hibf_gpu_ibf_download_occupancy", None, [vp, vp, u64]),
    ("hibf_gpu_ibf_track_occupancy", None, [vp, vp]),
    ("hibf_gpu_ibf_status", None, [vp]),
    ("hibf_gpu_hibf_create", None, [u64, u64, vp, vp, vp, vp, vp, ctypes.POINTER(vp)]),
    ("hibf_gpu_hibf_destroy", None, [vp]),
    ("hibf_gpu_hibf_info", None, [vp, u64p]),
    ("hibf_gpu_hibf_ibf_info", None, [vp, u64, u64p]),
    ("hibf_gpu_hibf_emplace", None, [vp, u64, vp, u64, u64]),
    ("hibf_gpu_hibf_emplace_d", None, [vp, u64, vp, vp, u64, u64, vp]),
    ("hibf_gpu_hibf_get_tables", None, [vp, vp, vp, vp, vp, vp]),
    ("hibf_gpu_sink_push", None, [vp, vp, u64]),
    ("hibf_gpu_hibf_build", None, [ctypes.POINTER(BuildConfig), ctypes.c_char_p, INPUT_FN, vp, ctypes.POINTER(vp)]),
    ("hibf_gpu_ibf_build", None, [ctypes.POINTER(BuildConfig), u64, ctypes.c_uint32, ci, INPUT_FN, vp,
                                  ctypes.POINTER(vp)]),
    ("hibf_gpu_hibf_set_prev", None, [vp, vp, vp]),
    ("hibf_gpu_hibf_get_prev", None, [vp, vp, vp]),
    ("hibf_gpu_ibf_save", None, [vp, ctypes.c_char_p]),
    ("hibf_gpu_ibf_load", None, [ctypes.c_char_p, ctypes.POINTER(vp)]),
    ("hibf_gpu_hibf_save", None, [vp, ctypes.c_char_p]),
    ("hibf_gpu_hibf_load", None, [ctypes.c_char_p, ctypes.POINTER(vp)]),
    ("hibf_gpu_hll_sketch", None, [vp, u64, ctypes.c_uint32, vp]),
    ("hibf_gpu_hll_estimate", None, [vp, ctypes.c_uint32, ctypes.POINTER(ctypes.c_double)]),
    ("hibf_gpu_hll_sketch_d", None, [vp, u64, vp, u64, ctypes.c_uint32, vp, vp]),
    ("hibf_gpu_hibf_build_inputs", None, [ctypes.POINTER(BuildConfig), ctypes.c_char_p, INPUT_FN, vp, vp, vp]),
    ("hibf_gpu_ibf_plan", None, [ctypes.POINTER(BuildConfig), u64, ctypes.c_uint32, INPUT_FN, vp, u64p, u64p]),
    ("hibf_gpu_hibf_build_synthetic", None, [ctypes.POINTER(BuildConfig), ctypes.c_char_p, u64, vp, vp,
                                             ctypes.POINTER(vp)]),
    ("hibf_gpu_split_table_synthetic", None, [ctypes.POINTER(BuildConfig), ctypes.c_char_p, u64, vp,
                                              ctypes.POINTER(vp)]),
    ("hibf_gpu_split_table_inputs", None, [ctypes.POINTER(BuildConfig), ctypes.c_char_p, INPUT_FN, vp,
                                           ctypes.POINTER(vp)]),
    ("hibf_gpu_split_table_sizes", None, [vp, u64p, u64p, u64p]),
    ("hibf_gpu_split_table_export", None, [vp, vp, vp, vp, vp, vp, vp, vp, vp]),
    ("hibf_gpu_split_table_import", None, [u64, u64, u64, vp, vp, vp, vp, vp, vp, vp, vp, ctypes.POINTER(vp)]),
    ("hibf_gpu_split_table_chunks", None, [vp, u64, vp, u64, vp]),
    ("hibf_gpu_split_table_destroy", "void", [vp]),
    ("hibf_gpu_plan_disjoint", None, [ctypes.POINTER(BuildConfig), ctypes.c_char_p, vp, u64p, u64p, vp, vp, vp,
                                      vp, vp, vp]),
    ("hibf_gpu_hibf_upload_words", None, [vp, u64, vp, u64]),
    ("hibf_gpu_hibf_download_words", None, [vp, u64, vp, u64]),
    ("hibf_gpu_hibf_digests", None, [vp, vp, ctypes.c_uint32]),
    ("hibf_gpu_hibf_build_timers", None, [vp, ctypes.POINTER(Timer)]),
    ("hibf_gpu_agent_create", None, [vp, ctypes.POINTER(vp)]),
    ("hibf_gpu_agent_destroy", None, [vp]),
    ("hibf_gpu_agent_set_stream", None, [vp, vp]),
    ("hibf_gpu_agent_reserve", None, [vp, u64, u64, u64, u64]),
    ("hibf_gpu_agent_membership_for", None, [vp, vp, u64, ctypes.c_uint16, ctypes.POINTER(u64p), u64p]),
    ("hibf_gpu_agent_membership_for_unsorted", None, [vp, vp, u64, ctypes.c_uint16, ctypes.POINTER(u64p), u64p]),
    ("hibf_gpu_agent_bulk_count", None, [vp, vp, u64, u64, ci, ctypes.POINTER(vp)]),
    ("hibf_gpu_agent_query_batch", None,
     [vp, ci, vp, vp, u64, vp, ci, ctypes.POINTER(u64p), ctypes.POINTER(u64p), ctypes.POINTER(vp)]),
    ("hibf_gpu_agent_query_batch_d", None,
     [vp, ci, vp, vp, u64, vp, ci, ctypes.POINTER(u64p), ctypes.POINTER(u64p), ctypes.POINTER(vp)]),
    ("hibf_gpu_agent_query_plain_d", None, [vp, ci, vp, vp, u64, vp, ci]),
    ("hibf_gpu_agent_fetch_results", None,
     [vp, u64, ci, ci, ctypes.POINTER(u64p), ctypes.POINTER(u64p), ctypes.POINTER(vp)]),
    ("hibf_gpu_agent_status", None, [vp]),
    ("hibf_gpu_set_l2_fetch_granularity", None, [ci]),
    ("hibf_gpu_agent_selftest_wait_limit", None, [vp, ctypes.c_double]),
    ("hibf_gpu_agent_last_work", None, [vp, u64p, u64p]),
    ("hibf_gpu_agent_last_work_executed", None, [vp, u64p]),
    ("hibf_gpu_agent_capture_batch_d", None, [vp, ci, vp, vp, u64, vp, ci]),
    ("hibf_gpu_agent_replay", None, [vp]),
    ("hibf_gpu_agent_kernel_ms", None, [vp, ctypes.POINTER(ctypes.c_float)]),
    ("hibf_gpu_agent_level_ms", None, [vp, ctypes.POINTER(ctypes.c_float), ctypes.c_uint32,
                                       ctypes.POINTER(ctypes.c_uint32)]),
    ("hibf_gpu_agent_level_work", None, [vp, vp, vp, vp, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32)]),
    ("hibf_gpu_agent_set_host_read", None, [vp, ci]),
    ("hibf_gpu_agent_last_in_place", None, [vp, ctypes.POINTER(ci)]),
    ("hibf_gpu_agent_input_chunks", None, [vp, ctypes.POINTER(ctypes.c_uint32)]),
    ("hibf_gpu_agent_last_timeline", None, [vp, ctypes.POINTER(ctypes.c_double), ctypes.c_uint32,
                                            ctypes.POINTER(ctypes.c_uint32)]),
    ("hibf_gpu_stream_plan", None, [vp, u64, vp, u64, ctypes.POINTER(ctypes.c_uint64)]),
    ("hibf_gpu_tuning_default", "void", [ctypes.POINTER(Tuning)]),
    ("hibf_gpu_agent_set_tuning", None, [vp, ctypes.POINTER(Tuning)]),
    ("hibf_gpu_agent_get_tuning", None, [vp, ctypes.POINTER(Tuning)]),
    ("hibf_gpu_tune_search", None, [ctypes.c_uint32, ctypes.c_uint32, TUNE_MEASURE_FN, vp,
                                    ctypes.POINTER(TuneTrial), u64, u64p, ctypes.POINTER(Tuning)]),
    ("hibf_gpu_agent_set_order_d", None, [vp, vp, u64]),
    ("hibf_gpu_agent_set_work_out_d", None, [vp, vp, u64]),
    ("hibf_gpu_agent_query_features_d", None, [vp, vp, vp, u64, vp, ctypes.c_uint32, vp]),
    ("hibf_gpu_cost_model_create", None, [u64, ctypes.POINTER(vp)]),
    ("hibf_gpu_cost_model_destroy", None, [vp]),
    ("hibf_gpu_cost_model_get_params", None, [vp, vp]),
    ("hibf_gpu_cost_model_set_params", None, [vp, vp]),
    ("hibf_gpu_cost_model_loss_grad_d", None, [vp, vp, vp, u64, vp, ctypes.POINTER(ctypes.c_double)]),
    ("hibf_gpu_cost_model_train_d", None, [vp, vp, vp, u64, ctypes.c_uint32, ctypes.c_float,
                                           ctypes.POINTER(ctypes.c_double)]),
    ("hibf_gpu_cost_model_predict_d", None, [vp, vp, u64, vp, vp]),
    ("hibf_gpu_cost_model_order_d", None, [vp, vp, u64, vp, vp]),
    ("hibf_gpu_sort_desc_d", None, [vp, vp, u64, vp, vp]),
    ("hibf_gpu_agent_autotune", None, [vp, ci, vp, vp, u64, vp, ci, ci, ctypes.POINTER(TuneTrial), u64, u64p]),
    ("hibf_gpu_server_create", None, [vp, ci, u64, u64, u64, ctypes.POINTER(vp)]),
    ("hibf_gpu_server_destroy", None, [vp]),
    ("hibf_gpu_server_submit", None, [vp, vp, vp, u64, vp, ctypes.c_double, ci, u64p]),
    ("hibf_gpu_server_wait", None, [vp, u64, ctypes.c_double, ctypes.POINTER(ci), ctypes.POINTER(u64p),
                                    ctypes.POINTER(u64p), ctypes.POINTER(ctypes.c_double)]),
    ("hibf_gpu_server_release", None, [vp, u64]),
    ("hibf_gpu_server_register_host", None, [vp, vp, u64, ci]),
    ("hibf_gpu_server_set_zero_copy", None, [vp, ci]),
    ("hibf_gpu_server_unregister_host", None, [vp, vp]),
    ("hibf_gpu_server_now", ctypes.c_double, []),
    ("hibf_gpu_server_stats", None, [vp, u64p]),
    ("hibf_gpu_server_phase_times", None, [vp, ctypes.POINTER(ctypes.c_double)]),
    ("hibf_gpu_server_batch_log", None, [vp, ctypes.POINTER(ctypes.c_double), u64, u64p]),
    ("hibf_gpu_server_open_loop", None, [vp, vp, vp, u64, ctypes.c_double, ctypes.c_double, u64, ctypes.c_double,
                                         ctypes.c_double, u64, ctypes.POINTER(ctypes.c_double)]),
    ("hibf_gpu_server_open_loop_detail", None, [vp, vp]),
    ("hibf_gpu_probe_random_reads", None, [u64, u64, ctypes.POINTER(ctypes.c_double)]),
    ("hibf_gpu_synth_user_bin_offsets", None, [u64, ci, ctypes.c_double, ctypes.c_double, u64, u64, u64, vp]),
    ("hibf_gpu_synth_query_offsets", None, [u64, ci, u64, u64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                            ctypes.c_uint32, u64, u64, u64, vp, vp]),
    ("hibf_gpu_synth_queries", None, [u64, ci, u64, u64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                      ctypes.c_uint32, u64, vp, u64, u64, vp, vp]),
    ("hibf_gpu_synth_ibf_emplace", None, [vp, u64, u64, u64, u64, vp]),
    ("hibf_gpu_synth_ibf_queries", None, [u64, u64, u64, u64, u64, vp]),
    ("hibf_gpu_synth_ibf_queries_d", None, [u64, u64, u64, u64, u64, vp, vp]),
    ("hibf_gpu_synth_queries_d", None, [u64, ci, u64, u64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                        ctypes.c_uint32, u64, vp, u64, u64, vp, vp, vp]),
]

_lib = None


def declared_symbols() -> list[str]:
    return [name for name, _, _ in _SIGS]


def lib() -> ctypes.CDLL:
    """Loads libhibf_gb300.so (building it first when HIBF_GB300_AUTOBUILD=1)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        if os.environ.get("HIBF_GB300_AUTOBUILD") == "1":
            from . import _build

            _build.build()
        else:
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -m hibf_gb300._build` "
                              "(the library has no CPU fallback)")
    L = ctypes.CDLL(str(LIB_PATH))
    for name, res, args in _SIGS:
        f = getattr(L, name)
        f.restype = ci if res is None else (None if res == "void" else res)
        f.argtypes = args
    _lib = L
    return L


def last_error() -> str:
    return (lib().hibf_gpu_last_error() or b"").decode(errors="replace")


def check(status: int) -> None:
    if status == OK:
        return
    msg = last_error()
    if status == ERR_LOGIC:
        raise LogicError(status, msg)
    if status == ERR_INVALID_ARG:
        raise InvalidArgument(status, msg)
    if status == ERR_OUT_OF_MEMORY:
        raise MemoryError(msg)
    raise HibfGpuError(status, msg)


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args))


def device_count() -> int:
    n = ci(0)
    call("hibf_gpu_device_count", ctypes.byref(n))
    return n.value
