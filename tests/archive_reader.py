"""A reader of the serialised filter layout (the reference's serialize functions in cereal's binary encoding), used by
the tests to look inside the reference's own archives."""

import struct

import numpy as np


class _Bytes:
    def __init__(self, data: bytes):
        self.b, self.i = data, 0

    def take(self, n):
        out = self.b[self.i:self.i + n]
        if len(out) != n:
            raise ValueError("archive truncated")
        self.i += n
        return out

    def u8(self):
        return self.take(1)[0]

    def u32(self):
        return struct.unpack("<I", self.take(4))[0]

    def u64(self):
        return struct.unpack("<Q", self.take(8))[0]

    def u64s(self, n=None):
        n = self.u64() if n is None else n
        return np.frombuffer(self.take(8 * n), np.uint64).copy()


def read_ibf(r: _Bytes) -> dict:
    d = dict(version=r.u32(), bins=r.u64(), technical_bins=r.u64(), bin_size=r.u64(), hash_shift=r.u64(),
             bin_words=r.u64(), hash_funs=r.u64(), bits=r.u64())
    d["words"] = r.u64s((d["bits"] + 63) // 64)
    d["occupancy"] = r.u64s()
    d["track_occupancy"] = r.u8()
    return d


def ibf(data: bytes) -> dict:
    r = _Bytes(data)
    d = read_ibf(r)
    assert r.i == len(data)
    return d


def hibf(data: bytes) -> dict:
    r = _Bytes(data)
    d = dict(version=r.u32(), n_user_bins=r.u64())
    d["ibfs"] = [read_ibf(r) for _ in range(r.u64())]
    d["next_ibf"] = [r.u64s() for _ in range(r.u64())]
    d["prev"] = [(r.u64(), r.u64()) for _ in range(r.u64())]
    d["user_bin"] = [r.u64s() for _ in range(r.u64())]
    assert r.i == len(data)
    return d
