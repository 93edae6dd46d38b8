"""The C++20 facade (include/hibf_gb300.hpp): it compiles against the C ABI (CPU), and a C++ program that
re-expresses the reference's IBF/HIBF unit tests and snippets passes on the device (GPU)."""

import subprocess
from pathlib import Path

import pytest

from hibf_gb300 import _build, _native as N
from tests import golden_io as G

ROOT = Path(__file__).resolve().parents[1]


def _compile(out: Path) -> Path:
    _build.build()
    exe = out / "test_facade"
    cmd = ["g++", "-std=c++20", "-O1", "-Wall", "-Wextra", f"-I{ROOT / 'include'}",
           str(ROOT / "tests" / "cpp" / "test_facade.cpp"), "-o", str(exe), f"-L{N.LIB_PATH.parent}",
           "-lhibf_gb300", f"-Wl,-rpath,{N.LIB_PATH.parent}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_facade_compiles(tmp_path):
    assert _compile(tmp_path).exists()


@pytest.mark.gpu
def test_facade_reference_unit_tests(gpu_lib, tmp_path):
    exe = _compile(tmp_path)
    for name in ("snippet", "readme"):
        (tmp_path / f"layout_{name}.txt").write_text(G.hibf_case(name)["layout_text"])
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all facade checks passed" in r.stdout
