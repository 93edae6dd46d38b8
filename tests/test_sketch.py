"""HyperLogLog sketches (seqan::hibf::sketch::hyperloglog): the host restatement against the reference's registers
(golden vectors, CPU) and the device sketching of many user bins against the host (GPU)."""

import ctypes

import numpy as np
import pytest

from hibf_gb300 import _build, _native as N
from hibf_gb300 import synthetic as S
from tests import golden_io as G


@pytest.fixture(scope="module")
def lib():
    _build.build()
    return N.lib()


def host_sketch(values, bits):
    v = np.ascontiguousarray(np.asarray(values, dtype=np.uint64))
    out = np.zeros(1 << bits, np.uint8)
    N.call("hibf_gpu_hll_sketch", v.ctypes.data if v.size else None, v.size, bits, out.ctypes.data)
    return out


def estimate(regs, bits):
    e = ctypes.c_double(0)
    r = np.ascontiguousarray(regs, dtype=np.uint8)
    N.call("hibf_gpu_hll_estimate", r.ctypes.data, bits, ctypes.byref(e))
    return e.value


@pytest.mark.skipif(not (G.GOLDEN / "hll_cases.npz").exists(), reason="golden sketches not generated")
def test_host_sketch_matches_reference(lib):
    z = np.load(G.GOLDEN / "hll_cases.npz")
    for i in range(int(z["n_cases"][0])):
        bits = int(z[f"c{i}_bits"][0])
        kind, seed, n = (int(x) for x in z[f"c{i}_source"])
        values = (S.stream_range(seed, 0, n), np.arange(n, dtype=np.uint64), z.get(f"c{i}_values"))[kind]
        regs = host_sketch(values, bits)
        np.testing.assert_array_equal(regs, z[f"c{i}_registers"], err_msg=f"case {i}")
        assert estimate(regs, bits) == z[f"c{i}_estimate"][0]


def test_estimate_tracks_cardinality(lib):
    for n, bits in ((100, 12), (50_000, 12), (2_000_000, 14)):
        e = estimate(host_sketch(S.stream_range(9, 0, n), bits), bits)
        assert abs(e - n) / n < 0.05


@pytest.mark.gpu
@pytest.mark.parametrize("bits", [5, 12, 15])
def test_device_sketches_match_host(gpu_lib, bits):
    import torch

    sizes = S.user_bin_sizes(5, 40, S.SIZES_LOG_UNIFORM, 0, 0, 1, 300_000)
    sizes[3] = 0  # an empty user bin
    offs = S.offsets_of(sizes)
    size = 1 << bits
    # synthetic stream user bins
    d = torch.empty(40 * size, dtype=torch.uint8, device="cuda")
    N.call("hibf_gpu_hll_sketch_d", None, 5, offs.ctypes.data, 40, bits, d.data_ptr(), None)
    got = d.cpu().numpy().reshape(40, size)
    vals = S.stream_range(5, 0, int(offs[-1]))
    for u in range(40):
        np.testing.assert_array_equal(got[u], host_sketch(vals[offs[u]:offs[u + 1]], bits), err_msg=f"ub {u}")
    # values in device memory (duplicates and overlaps between user bins)
    rng = np.random.default_rng(bits)
    v = rng.integers(0, 1 << 40, int(offs[-1]), dtype=np.uint64)
    v[: v.size // 3] = v[v.size // 3: 2 * (v.size // 3)]
    dv = torch.from_numpy(v.view(np.int64)).cuda()
    N.call("hibf_gpu_hll_sketch_d", dv.data_ptr(), 0, offs.ctypes.data, 40, bits, d.data_ptr(), None)
    got = d.cpu().numpy().reshape(40, size)
    for u in range(40):
        np.testing.assert_array_equal(got[u], host_sketch(v[offs[u]:offs[u + 1]], bits), err_msg=f"ub {u}")
