"""Serialised filters in the reference's byte layout: what the reference's serialize functions write (golden archives
from the reference, read here on the CPU), and the device stores saved and loaded through it (GPU)."""

import numpy as np
import pytest

from hibf_gb300 import synthetic as S
from tests import archive_reader as A
from tests import golden_io as G
from tests.hibf_canon import canonical


def test_reference_ibf_archive_layout(oracle):
    """The reference's IBF archive: header fields, the bit_vector words of the same emplaces in the oracle, occupancy."""
    d = A.ibf((G.GOLDEN / "serial_ibf.bin").read_bytes())
    assert (d["version"], d["bins"], d["technical_bins"], d["bin_size"], d["hash_shift"], d["bin_words"],
            d["hash_funs"], d["bits"]) == (1, 130, 192, 1000, 54, 3, 3, 192000)
    O = oracle.ibf(130, 1000, 3, True)
    v = S.stream_range(3, 0, 4000)
    O.emplace(v, np.arange(4000, dtype=np.uint64) % np.uint64(130))
    np.testing.assert_array_equal(d["words"], O.words())
    assert d["track_occupancy"] == 1 and d["occupancy"].size == 192
    assert int(d["occupancy"][:130].sum()) <= 4000 and int(d["occupancy"][130:].sum()) == 0


@pytest.mark.parametrize("name", ["snippet", "synth64"])
def test_reference_hibf_archive_layout(name):
    """The reference's HIBF archive holds the same IBFs (by path of merged bins), sizes, tables and bit words as the
    golden HIBF, and prev_ibf_id as its build leaves it."""
    d = A.hibf((G.GOLDEN / f"serial_hibf_{name}.bin").read_bytes())
    g = G.hibf_case(name)
    assert d["version"] == 1 and d["n_user_bins"] == g["n_ub"]
    t = dict(bins=np.array([x["bins"] for x in d["ibfs"]], np.uint64),
             bin_size=np.array([x["bin_size"] for x in d["ibfs"]], np.uint64),
             next_ibf=np.concatenate(d["next_ibf"]), user_bin=np.concatenate(d["user_bin"]))
    ref, got = canonical(G.tables(g)), canonical(t)
    assert set(ref) == set(got)
    for path, (bins, size, row, k_ref) in ref.items():
        k = got[path][3]
        assert (bins, size) == got[path][:2], path
        assert S.digest(d["ibfs"][k]["words"].tolist()) == int(g["digests"][k_ref]), path
    assert d["prev"][0] == (0, 0)


# ---------------------------------------------------------------------------------------------------------------- GPU
@pytest.mark.gpu
def test_device_ibf_archive_round_trip(gpu_lib, tmp_path):
    """The same emplaces on the device save to the reference's bytes; its archive loads into an equal device store."""
    import hibf_gb300 as hg

    ibf = hg.interleaved_bloom_filter(hg.bin_count(130), hg.bin_size(1000), hg.hash_function_count(3), True)
    v = S.stream_range(3, 0, 4000)
    ibf.emplace_many(v, np.arange(4000, dtype=np.uint64) % np.uint64(130))
    ibf.save(tmp_path / "a.bin")
    ref = (G.GOLDEN / "serial_ibf.bin").read_bytes()
    assert (tmp_path / "a.bin").read_bytes() == ref
    loaded = hg.interleaved_bloom_filter.load(G.GOLDEN / "serial_ibf.bin")
    np.testing.assert_array_equal(loaded.words(), ibf.words())
    np.testing.assert_array_equal(loaded.occupancy[:130], ibf.occupancy[:130])
    assert loaded == ibf  # the reference's operator==: shape, occupancy, bits
    loaded.save(tmp_path / "b.bin")
    assert (tmp_path / "b.bin").read_bytes() == ref
    loaded.clear(hg.bin_index(0))
    assert not loaded == ibf


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["snippet", "synth64"])
def test_device_hibf_archive_round_trip(gpu_lib, tmp_path, name):
    """A reference HIBF archive loads into device stores that answer the golden queries and save to the same bytes."""
    import hibf_gb300 as hg

    src = G.GOLDEN / f"serial_hibf_{name}.bin"
    H = hg.hierarchical_interleaved_bloom_filter.load(src)
    H.save(tmp_path / "h.bin")
    assert (tmp_path / "h.bin").read_bytes() == src.read_bytes()
    np.testing.assert_array_equal(H.prev_ibf_id, np.array(A.hibf(src.read_bytes())["prev"], np.uint64))
    assert hg.hierarchical_interleaved_bloom_filter.load(tmp_path / "h.bin") == H
    g = G.hibf_case(name)
    offs, ids, _ = H.membership_agent().query_batch(g["q_values"], g["q_offsets"], g["mem_t"])
    for i, e in enumerate(G.mem_lists(g, "mem_sorted")):
        np.testing.assert_array_equal(ids[offs[i]:offs[i + 1]], e, err_msg=f"query {i}")


@pytest.mark.gpu
def test_malformed_archives_are_rejected(gpu_lib, tmp_path):
    import hibf_gb300 as hg

    ref = (G.GOLDEN / "serial_ibf.bin").read_bytes()
    (tmp_path / "short.bin").write_bytes(ref[:-9])
    (tmp_path / "version.bin").write_bytes(bytes([2]) + ref[1:])
    (tmp_path / "fields.bin").write_bytes(ref[:12] + (7).to_bytes(8, "little") + ref[20:])
    for bad in ("short.bin", "version.bin", "fields.bin"):
        with pytest.raises(hg.InvalidArgument):
            hg.interleaved_bloom_filter.load(tmp_path / bad)
    with pytest.raises(hg.InvalidArgument):
        hg.hierarchical_interleaved_bloom_filter.load(tmp_path / "short.bin")
