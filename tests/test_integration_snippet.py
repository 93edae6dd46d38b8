"""The seqan::hibf-side binding shown in INTEGRATION.md compiles against the reference's own headers (with the
cereal/simde stand-ins in oracle/shim) and this repository's C ABI header.  Skipped where the reference sources are
not present."""

import re
import subprocess
from pathlib import Path

import pytest

from oracle.bindings import DEFAULT_REF_DIR

ROOT = Path(__file__).resolve().parents[1]
REF_INCLUDE = Path(DEFAULT_REF_DIR) / "include"


@pytest.mark.skipif(not (REF_INCLUDE / "hibf").is_dir(), reason="seqan/hibf headers not present")
def test_integration_snippet_compiles(tmp_path):
    text = (ROOT / "INTEGRATION.md").read_text()
    blocks = re.findall(r"```cpp\n(.*?)```", text, flags=re.S)
    assert blocks, "INTEGRATION.md has no C++ snippet"
    src = tmp_path / "snippet.cpp"
    src.write_text("\n".join(blocks) + "\nint main() { return 0; }\n")
    cmd = ["g++", "-std=c++23", "-fsyntax-only", "-w", f"-I{REF_INCLUDE}",
           f"-I{ROOT / 'oracle' / 'shim'}", f"-I{ROOT / 'include'}", str(src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
