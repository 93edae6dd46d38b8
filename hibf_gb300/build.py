"""HIBF construction from a layout: the seqan::hibf::config mirror and the build entry points.

    cfg = config(input_fn=fn, number_of_user_bins=3)            # fn(user_bin, it): it.push(values) / it(value)
    hibf = hierarchical_interleaved_bloom_filter(cfg, layout_text)
    hibf = build_synthetic(cfg, layout_text, seed, offsets)    # user bins from the seeded splitmix64 stream

The layout is the reference's layout file text (its DP and HyperLogLog sketches stay on the host, unchanged, so the
same layout gives the same filter sizes and tables).  Sizes and tables are computed on the host; all inserts run on
the device.
"""

from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field
from typing import Callable

import numpy as np

from . import _native as N


@dataclass
class config:
    """Mirror of seqan::hibf::config (include/hibf/config.hpp:75-413)."""

    input_fn: Callable | None = None
    number_of_user_bins: int = 0
    number_of_hash_functions: int = 2
    maximum_fpr: float = 0.05
    relaxed_fpr: float = 0.3
    threads: int = 1
    sketch_bits: int = 12
    tmax: int = 0
    empty_bin_fraction: float = 0.0
    track_occupancy: bool = False
    alpha: float = 1.2
    max_rearrangement_ratio: float = 0.5
    disable_estimate_union: bool = False
    disable_rearrangement: bool = False
    warnings: list = field(default_factory=list)

    def validate_and_set_defaults(self) -> None:
        """config::validate_and_set_defaults (src/config.cpp:64-130): same checks, messages and defaults."""
        E = N.InvalidArgument
        if self.input_fn is None:
            raise E(N.ERR_INVALID_ARG, "[HIBF CONFIG ERROR] You did not set the required config::input_fn.")
        if self.number_of_user_bins == 0:
            raise E(N.ERR_INVALID_ARG,
                    "[HIBF CONFIG ERROR] You did not set the required config::number_of_user_bins.")
        if self.number_of_user_bins >= 18446744073709551614:
            raise E(N.ERR_INVALID_ARG, "[HIBF CONFIG ERROR] The maximum possible config::number_of_user_bins "
                                       "is 18446744073709551613.")
        if self.number_of_hash_functions == 0 or self.number_of_hash_functions > 5:
            raise E(N.ERR_INVALID_ARG, "[HIBF CONFIG ERROR] config::number_of_hash_functions must be in [1,5].")
        if not (0.0 < self.maximum_fpr < 1.0):
            raise E(N.ERR_INVALID_ARG, "[HIBF CONFIG ERROR] config::maximum_fpr must be in (0.0,1.0).")
        if not (0.0 < self.relaxed_fpr < 1.0):
            raise E(N.ERR_INVALID_ARG, "[HIBF CONFIG ERROR] config::relaxed_fpr must be in (0.0,1.0).")
        if self.relaxed_fpr < self.maximum_fpr:
            raise E(N.ERR_INVALID_ARG, "[HIBF CONFIG ERROR] config::relaxed_fpr must be "
                                       "greater than or equal to config::maximum_fpr.")
        if self.threads == 0:
            raise E(N.ERR_INVALID_ARG, "[HIBF CONFIG ERROR] config::threads must be greater than 0.")
        if self.sketch_bits < 5 or self.sketch_bits > 32:
            raise E(N.ERR_INVALID_ARG, "[HIBF CONFIG ERROR] config::sketch_bits must be in [5,32].")
        if self.tmax == 0:
            self.tmax = ((math.ceil(math.sqrt(self.number_of_user_bins)) + 63) >> 6) << 6
        elif self.tmax > 18446744073709551552:
            raise E(N.ERR_INVALID_ARG, "[HIBF CONFIG ERROR] The maximum possible config::tmax is "
                                       "18446744073709551552.")
        elif self.tmax % 64 != 0:
            self.tmax = ((self.tmax + 63) >> 6) << 6
            self.warnings.append("[HIBF CONFIG WARNING]: Your requested number of technical bins was not a multiple "
                                 f"of 64. Due to the architecture of the HIBF, it will use up space equal to the next "
                                 f"multiple of 64 anyway, so we increased your number of technical bins to "
                                 f"{self.tmax}.")
        if not (0.0 <= self.empty_bin_fraction < 1.0):
            raise E(N.ERR_INVALID_ARG, "[HIBF CONFIG ERROR] config::empty_bin_fraction must be in [0.0,1.0).")
        if self.empty_bin_fraction != 0.0:
            self.track_occupancy = True
        if self.alpha < 0.0:
            raise E(N.ERR_INVALID_ARG, "[HIBF CONFIG ERROR] config::alpha must be positive.")
        if not (0.0 <= self.max_rearrangement_ratio <= 1.0):
            raise E(N.ERR_INVALID_ARG, "[HIBF CONFIG ERROR] config::max_rearrangement_ratio must be in [0.0,1.0].")
        if self.disable_estimate_union or self.max_rearrangement_ratio == 0.0:
            self.disable_rearrangement = True


def _cfg(c: config, disjoint: bool) -> N.BuildConfig:
    return N.BuildConfig(c.number_of_user_bins, c.number_of_hash_functions, c.maximum_fpr, c.relaxed_fpr, c.threads,
                         int(disjoint))


class insert_iterator:
    """What input_fn receives: `it(value)`, `it.push(values)` or `it = value`-style `it.emplace(value)`."""

    def __init__(self, sink):
        self._sink = sink

    def push(self, values) -> None:
        v = np.ascontiguousarray(np.asarray(values, dtype=np.uint64).reshape(-1))
        if v.size:
            N.call("hibf_gpu_sink_push", self._sink, v.ctypes.data, v.size)

    def __call__(self, value) -> None:
        self.push([int(value)])

    emplace = __call__


def _adopt_handle(h: ctypes.c_void_p, n_user_bins: int):
    from .hibf import hierarchical_interleaved_bloom_filter

    info = (ctypes.c_uint64 * 4)()
    N.call("hibf_gpu_hibf_info", h, info)
    n_ibfs = int(info[1])
    bins = np.zeros(n_ibfs, np.uint64)
    N.call("hibf_gpu_hibf_get_tables", h, bins.ctypes.data, None, None, None, None)
    total = int(bins.sum())
    bsz, hf = np.zeros(n_ibfs, np.uint64), np.zeros(n_ibfs, np.uint64)
    nxt, ub = np.zeros(total, np.uint64), np.zeros(total, np.uint64)
    N.call("hibf_gpu_hibf_get_tables", h, None, bsz.ctypes.data, hf.ctypes.data, nxt.ctypes.data, ub.ctypes.data)
    obj = hierarchical_interleaved_bloom_filter.__new__(hierarchical_interleaved_bloom_filter)
    obj._h = h
    obj.number_of_user_bins = int(n_user_bins)
    obj.bins, obj.bin_size, obj.hash_funs = bins, bsz, hf
    obj.next_ibf_id, obj.ibf_bin_to_user_bin_id = nxt, ub
    obj._rank = None
    return obj


def build_from_layout(configuration: config, layout_text: str, user_bins_disjoint: bool = False):
    """hierarchical_interleaved_bloom_filter(config&, layout const&) with config.input_fn as the data source."""
    configuration.validate_and_set_defaults()
    fn = configuration.input_fn

    def trampoline(_user, ub, sink):
        fn(int(ub), insert_iterator(sink))

    cb = N.INPUT_FN(trampoline)
    h = ctypes.c_void_p()
    N.call("hibf_gpu_hibf_build", ctypes.byref(_cfg(configuration, user_bins_disjoint)), layout_text.encode(), cb,
           None, ctypes.byref(h))
    return _adopt_handle(h, configuration.number_of_user_bins)


SPLIT_TABLE_FIELDS = ("user_bin", "n_values", "mult", "mask", "bnd_off", "bnd_home", "before_off", "before")


class split_table:
    """How the reference chunks every split user bin of one layout and one set of user bin sizes (see
    hibf_gpu_split_table_* in include/hibf_gb300.h): computed by replaying the reference's hash-set history, or
    imported from the arrays of an earlier export (a dict with SPLIT_TABLE_FIELDS)."""

    def __init__(self, handle: ctypes.c_void_p):
        self._h = handle

    @classmethod
    def synthetic(cls, configuration: config, layout_text: str, seed: int, user_bin_offsets) -> "split_table":
        if configuration.input_fn is None:
            configuration.input_fn = lambda ub, it: None
        configuration.validate_and_set_defaults()
        off = np.ascontiguousarray(np.asarray(user_bin_offsets, dtype=np.uint64))
        h = ctypes.c_void_p()
        N.call("hibf_gpu_split_table_synthetic", ctypes.byref(_cfg(configuration, True)), layout_text.encode(),
               int(seed), off.ctypes.data, ctypes.byref(h))
        return cls(h)

    @classmethod
    def inputs(cls, configuration: config, layout_text: str) -> "split_table":
        """The table of build_from_layout's inputs (configuration.input_fn read once per user bin)."""
        configuration.validate_and_set_defaults()
        fn = configuration.input_fn

        def trampoline(_user, ub, sink):
            fn(int(ub), insert_iterator(sink))

        cb = N.INPUT_FN(trampoline)
        h = ctypes.c_void_p()
        N.call("hibf_gpu_split_table_inputs", ctypes.byref(_cfg(configuration, False)), layout_text.encode(), cb,
               None, ctypes.byref(h))
        return cls(h)

    @classmethod
    def from_arrays(cls, a: dict) -> "split_table":
        arr = {k: np.ascontiguousarray(np.asarray(a[k], dtype=np.uint64)) for k in SPLIT_TABLE_FIELDS}
        h = ctypes.c_void_p()
        N.call("hibf_gpu_split_table_import", arr["user_bin"].size, arr["bnd_home"].size, arr["before"].size,
               *[arr[k].ctypes.data for k in SPLIT_TABLE_FIELDS], ctypes.byref(h))
        return cls(h)

    def arrays(self) -> dict:
        ns, nb, nv = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        N.call("hibf_gpu_split_table_sizes", self._h, ctypes.byref(ns), ctypes.byref(nb), ctypes.byref(nv))
        n = dict(user_bin=ns.value, n_values=ns.value, mult=ns.value, mask=ns.value, bnd_off=ns.value + 1,
                 bnd_home=nb.value, before_off=nb.value + 1, before=nv.value)
        out = {k: np.zeros(max(n[k], 1), np.uint64) for k in SPLIT_TABLE_FIELDS}
        N.call("hibf_gpu_split_table_export", self._h, *[out[k].ctypes.data for k in SPLIT_TABLE_FIELDS])
        return {k: out[k][:n[k]] for k in SPLIT_TABLE_FIELDS}

    def chunks(self, user_bin: int, values) -> np.ndarray:
        v = np.ascontiguousarray(np.asarray(values, dtype=np.uint64))
        out = np.zeros(max(v.size, 1), np.uint64)
        N.call("hibf_gpu_split_table_chunks", self._h, int(user_bin), v.ctypes.data, v.size, out.ctypes.data)
        return out[:v.size]

    def __del__(self):
        if getattr(self, "_h", None):
            N.lib().hibf_gpu_split_table_destroy(self._h)
            self._h = None


def build_synthetic(configuration: config, layout_text: str, seed: int, user_bin_offsets,
                    table: split_table | None = None):
    """The same build for the seeded synthetic user bins (values generated on the device).  Split user bins are
    chunked in the reference's order, from `table` when given (it must belong to this layout and these offsets),
    else from a replay of the reference's hash-set history run first on the host."""
    if configuration.input_fn is None:
        configuration.input_fn = lambda ub, it: None  # contents come from the stream, not from a callback
    configuration.validate_and_set_defaults()
    off = np.ascontiguousarray(np.asarray(user_bin_offsets, dtype=np.uint64))
    h = ctypes.c_void_p()
    N.call("hibf_gpu_hibf_build_synthetic", ctypes.byref(_cfg(configuration, True)), layout_text.encode(), int(seed),
           off.ctypes.data, table._h if table is not None else None, ctypes.byref(h))
    return _adopt_handle(h, configuration.number_of_user_bins)


def plan_disjoint(configuration: config, layout_text: str, user_bin_sizes) -> dict:
    """Host-only sizes and tables for pairwise disjoint user bins (no device needed)."""
    if configuration.input_fn is None:
        configuration.input_fn = lambda ub, it: None
    configuration.validate_and_set_defaults()
    sizes = np.ascontiguousarray(np.asarray(user_bin_sizes, dtype=np.uint64))
    c = _cfg(configuration, True)
    n, t = ctypes.c_uint64(0), ctypes.c_uint64(0)
    args = [None] * 6
    N.call("hibf_gpu_plan_disjoint", ctypes.byref(c), layout_text.encode(), sizes.ctypes.data, ctypes.byref(n),
           ctypes.byref(t), *args)
    out = dict(bins=np.zeros(n.value, np.uint64), bin_size=np.zeros(n.value, np.uint64),
               next_ibf=np.zeros(t.value, np.uint64), user_bin=np.zeros(t.value, np.uint64),
               parent_ibf=np.zeros(n.value, np.uint64), parent_bin=np.zeros(n.value, np.uint64))
    N.call("hibf_gpu_plan_disjoint", ctypes.byref(c), layout_text.encode(), sizes.ctypes.data, ctypes.byref(n),
           ctypes.byref(t), *[out[k].ctypes.data for k in ("bins", "bin_size", "next_ibf", "user_bin", "parent_ibf",
                                                              "parent_bin")])
    out["hash_funs"] = np.full(n.value, configuration.number_of_hash_functions, np.uint64)
    out["n_user_bins"] = configuration.number_of_user_bins
    return out


def ibf_from_config(configuration: config, max_bin_elements: int = 0):
    """interleaved_bloom_filter(config&, max_bin_elements) (include/hibf/interleaved_bloom_filter.hpp:241)."""
    from .ibf import interleaved_bloom_filter

    configuration.validate_and_set_defaults()
    fn = configuration.input_fn

    def trampoline(_user, ub, sink):
        fn(int(ub), insert_iterator(sink))

    cb = N.INPUT_FN(trampoline)
    h = ctypes.c_void_p()
    N.call("hibf_gpu_ibf_build", ctypes.byref(_cfg(configuration, False)), int(max_bin_elements),
           configuration.sketch_bits, int(configuration.track_occupancy), cb, None, ctypes.byref(h))
    obj = interleaved_bloom_filter.__new__(interleaved_bloom_filter)
    obj._h = h
    obj._pending_v, obj._pending_b = [], []
    return obj


def ibf_plan(configuration: config, max_bin_elements: int = 0) -> tuple[int, int]:
    """Host part of interleaved_bloom_filter(config&, max_bin_elements): (bin size in bits, biggest user bin)."""
    configuration.validate_and_set_defaults()
    fn = configuration.input_fn

    def trampoline(_user, ub, sink):
        fn(int(ub), insert_iterator(sink))

    cb = N.INPUT_FN(trampoline)
    size, best = ctypes.c_uint64(0), ctypes.c_uint64(0)
    N.call("hibf_gpu_ibf_plan", ctypes.byref(_cfg(configuration, False)), int(max_bin_elements),
           configuration.sketch_bits, cb, None, ctypes.byref(size), ctypes.byref(best))
    return size.value, best.value


def build_inputs(configuration: config, layout_text: str) -> tuple[np.ndarray, np.ndarray]:
    """Host part of the build alone: (offsets, values) of every user bin's distinct values in insertion order, split
    user bins in the reference's chunk order (chunk k of ceil(n / tbs) values -> technical bin storage + k)."""
    configuration.validate_and_set_defaults()
    fn = configuration.input_fn

    def trampoline(_user, ub, sink):
        fn(int(ub), insert_iterator(sink))

    cb = N.INPUT_FN(trampoline)
    c = _cfg(configuration, False)
    offs = np.zeros(configuration.number_of_user_bins + 1, np.uint64)
    N.call("hibf_gpu_hibf_build_inputs", ctypes.byref(c), layout_text.encode(), cb, None, offs.ctypes.data, None)
    vals = np.zeros(int(offs[-1]), np.uint64)
    N.call("hibf_gpu_hibf_build_inputs", ctypes.byref(c), layout_text.encode(), cb, None, offs.ctypes.data,
           vals.ctypes.data)
    return offs, vals
