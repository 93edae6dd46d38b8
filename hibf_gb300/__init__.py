"""hibf_gb300 -- GB300-native build and query path of the Hierarchical Interleaved Bloom Filter.

A drop-in for seqan::hibf's IBF/HIBF hot path: the bit stores live in HBM, construction and queries run as
hand-written sm_103a CUDA kernels behind the C ABI in include/hibf_gb300.h (libhibf_gb300.so).  This package is the
Python mirror of the reference's interface over that ABI; it never computes results on the CPU.
"""

from ._native import (BIN_DELETED, BIN_MERGED, QUERY_COUNT, QUERY_MEMBERSHIP, HibfGpuError, InvalidArgument,
                      LogicError, device_count)
from .ibf import bin_count, bin_index, bin_size, hash_function_count, interleaved_bloom_filter
from .hibf import hierarchical_interleaved_bloom_filter

__all__ = [
    "BIN_DELETED", "BIN_MERGED", "QUERY_COUNT", "QUERY_MEMBERSHIP", "HibfGpuError", "InvalidArgument", "LogicError",
    "device_count", "bin_count", "bin_index", "bin_size", "hash_function_count", "interleaved_bloom_filter",
    "hierarchical_interleaved_bloom_filter",
]
