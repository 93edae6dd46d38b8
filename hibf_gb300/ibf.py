"""interleaved_bloom_filter -- the single-level IBF, device-resident (reference:
include/hibf/interleaved_bloom_filter.hpp, src/interleaved_bloom_filter.cpp).

Same names, argument meanings and error behaviour as the reference:

    ibf = interleaved_bloom_filter(bin_count(64), bin_size(1024), hash_function_count(2))
    ibf.emplace(value, bin_index(3))
    ibf.containment_agent().bulk_contains(value)        -> bit vector of bin_count bits
    ibf.counting_agent(width=2).bulk_count(values)      -> counting vector (uint16 by default, wraps like value_t)
    ibf.membership_agent().membership_for(values, t)    -> ascending bin ids with count >= t

Construction errors raise ``LogicError`` (std::logic_error), ``increase_bin_number_to`` below the current count
raises ``InvalidArgument`` (std::invalid_argument).  Single emplace() calls are buffered on the host and flushed to
the device in batches before any other operation, so the per-value API stays cheap.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _native as N


@dataclass(frozen=True)
class bin_count:
    value: int


@dataclass(frozen=True)
class bin_size:
    value: int


@dataclass(frozen=True)
class hash_function_count:
    value: int


@dataclass(frozen=True)
class bin_index:
    value: int


_DT = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}


def _u64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint64).reshape(-1))


def _val(x):
    return x.value if hasattr(x, "value") else int(x)


class interleaved_bloom_filter:
    _FLUSH = 1 << 20

    def __init__(self, bins, size, funs=hash_function_count(2), track_occupancy: bool = False):
        self._h = None
        h = ctypes.c_void_p()
        N.call("hibf_gpu_ibf_create", _val(bins), _val(size), _val(funs), int(track_occupancy), ctypes.byref(h))
        self._h = h
        self._pending_v: list[int] = []
        self._pending_b: list[int] = []

    def save(self, path) -> None:
        """Serialises the device store in the reference's byte layout (cereal binary encoding)."""
        self.flush()
        N.call("hibf_gpu_ibf_save", self._h, str(path).encode())

    @classmethod
    def load(cls, path) -> "interleaved_bloom_filter":
        """Reads a serialised IBF (as the reference writes it) into a new device store."""
        h = ctypes.c_void_p()
        N.call("hibf_gpu_ibf_load", str(path).encode(), ctypes.byref(h))
        obj = cls.__new__(cls)
        obj._h = h
        obj._pending_v, obj._pending_b = [], []
        return obj

    def __del__(self):
        if getattr(self, "_h", None):
            try:
                N.lib().hibf_gpu_ibf_destroy(self._h)
            except Exception:
                pass
            self._h = None

    def __eq__(self, other) -> bool:
        """Equal shape, tracking flag, occupancy and bits (the reference's defaulted operator==,
        interleaved_bloom_filter.hpp:433); the stores are compared through host copies."""
        if not isinstance(other, interleaved_bloom_filter):
            return NotImplemented
        a, b = self._info(), other._info()
        return (a[:3] == b[:3] and self.track_occupancy == other.track_occupancy and
                np.array_equal(self.occupancy, other.occupancy) and np.array_equal(self.words(), other.words()))

    __hash__ = None  # mutable, compared by content

    # -- properties ------------------------------------------------------------------------------------------
    def _info(self):
        out = (ctypes.c_uint64 * 5)()
        N.call("hibf_gpu_ibf_info", self._h, out)
        return [int(x) for x in out]

    def bin_count(self) -> int:
        return self._info()[0]

    def bin_size(self) -> int:
        return self._info()[1]

    def hash_function_count(self) -> int:
        return self._info()[2]

    def bit_size(self) -> int:
        return self._info()[3]

    @property
    def bin_words(self) -> int:
        return (self.bin_count() + 63) // 64

    # -- modifiers -------------------------------------------------------------------------------------------
    def emplace(self, value: int, bin: bin_index) -> None:
        self._pending_v.append(int(value))
        self._pending_b.append(_val(bin))
        if len(self._pending_v) >= self._FLUSH:
            self.flush()

    def emplace_many(self, values, bin) -> None:
        """Bulk emplace: every value into `bin` (an int / bin_index) or values[i] into bins[i] (an array)."""
        self.flush()
        v = _u64(values)
        if np.ndim(bin) == 0 and not isinstance(bin, np.ndarray):
            N.call("hibf_gpu_ibf_emplace", self._h, v.ctypes.data, v.size, _val(bin))
        else:
            b = _u64(bin)
            N.call("hibf_gpu_ibf_emplace_binned", self._h, v.ctypes.data, b.ctypes.data, v.size)

    def flush(self) -> None:
        if self._pending_v:
            v = np.array(self._pending_v, dtype=np.uint64)
            b = np.array(self._pending_b, dtype=np.uint64)
            self._pending_v, self._pending_b = [], []
            N.call("hibf_gpu_ibf_emplace_binned", self._h, v.ctypes.data, b.ctypes.data, v.size)

    def clear(self, bin) -> None:
        self.flush()
        if isinstance(bin, (list, tuple, np.ndarray)):
            b = _u64([_val(x) for x in bin])
            N.call("hibf_gpu_ibf_clear_range", self._h, b.ctypes.data, b.size)
        else:
            N.call("hibf_gpu_ibf_clear", self._h, _val(bin))

    def try_increase_bin_number_to(self, new_bins) -> bool:
        self.flush()
        ok = ctypes.c_int(0)
        N.call("hibf_gpu_ibf_try_increase_bin_number_to", self._h, _val(new_bins), ctypes.byref(ok))
        return bool(ok.value)

    def increase_bin_number_to(self, new_bins) -> None:
        self.flush()
        N.call("hibf_gpu_ibf_increase_bin_number_to", self._h, _val(new_bins))

    # -- words / occupancy -----------------------------------------------------------------------------------
    def words(self) -> np.ndarray:
        self.flush()
        out = np.zeros(self.bin_words * self.bin_size(), np.uint64)
        N.call("hibf_gpu_ibf_download_words", self._h, out.ctypes.data, out.size)
        return out

    def set_words(self, w) -> None:
        self.flush()
        w = _u64(w)
        N.call("hibf_gpu_ibf_upload_words", self._h, w.ctypes.data, w.size)

    @property
    def track_occupancy(self) -> bool:
        v = ctypes.c_int(0)
        N.call("hibf_gpu_ibf_track_occupancy", self._h, ctypes.byref(v))
        return bool(v.value)

    @property
    def occupancy(self) -> np.ndarray:
        self.flush()
        out = np.zeros(self.bin_words * 64, np.uint64)
        N.call("hibf_gpu_ibf_download_occupancy", self._h, out.ctypes.data, out.size)
        return out

    # -- agents ----------------------------------------------------------------------------------------------
    def containment_agent(self) -> "containment_agent_type":
        self.flush()
        return containment_agent_type(self)

    def counting_agent(self, width: int = 2) -> "counting_agent_type":
        self.flush()
        return counting_agent_type(self, width)

    def membership_agent(self) -> "membership_agent_type":
        self.flush()
        return membership_agent_type(self)


class containment_agent_type:
    def __init__(self, ibf: interleaved_bloom_filter):
        self.ibf = ibf

    def bulk_contains(self, value) -> np.ndarray:
        """Bit vector (bool array of bin_count entries) for one value."""
        words = self.bulk_contains_words(np.array([int(value)], np.uint64))[0]
        bits = np.unpackbits(words.view(np.uint8), bitorder="little")
        return bits[: self.ibf.bin_count()].astype(bool)

    def bulk_contains_words(self, values) -> np.ndarray:
        """For many values: the bit_vector words of every result, shape (n, ceil(bins/64))."""
        self.ibf.flush()
        v = _u64(values)
        out = np.zeros((v.size, self.ibf.bin_words), np.uint64)
        N.call("hibf_gpu_ibf_bulk_contains", self.ibf._h, v.ctypes.data, v.size, out.ctypes.data)
        return out


class counting_agent_type:
    def __init__(self, ibf: interleaved_bloom_filter, width: int = 2):
        self.ibf = ibf
        self.width = width

    def bulk_count(self, values) -> np.ndarray:
        self.ibf.flush()
        v = _u64(values)
        out = np.zeros(self.ibf.bin_count(), _DT[self.width])
        N.call("hibf_gpu_ibf_bulk_count", self.ibf._h, v.ctypes.data, v.size, self.width, out.ctypes.data)
        return out


class membership_agent_type:
    def __init__(self, ibf: interleaved_bloom_filter):
        self.ibf = ibf

    def membership_for(self, values, threshold: int) -> np.ndarray:
        self.ibf.flush()
        v = _u64(values)
        out = np.zeros(self.ibf.bin_count(), np.uint64)
        n = ctypes.c_uint64(0)
        N.call("hibf_gpu_ibf_membership_for", self.ibf._h, v.ctypes.data, v.size, int(threshold), out.ctypes.data,
               ctypes.byref(n))
        return out[: n.value]

    def sort_results(self) -> None:
        """No-op, as in the reference: IBF results are already ascending."""
