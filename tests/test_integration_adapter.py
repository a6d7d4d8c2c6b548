"""The GpuModelData adapter shown in INTEGRATION.md compiles against the
reference's headers and this repository's C ABI header (where the reference
sources are present; nothing is run)."""
import os
import re
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_SRC = "/root/reference/src"


@pytest.mark.skipif(not os.path.isdir(REF_SRC) or shutil.which("g++") is None,
                    reason="reference sources not present")
def test_adapter_compiles_against_reference_headers():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    blocks = re.findall(r"```cpp\n(.*?)```", text, flags=re.S)
    assert blocks, "no C++ block in INTEGRATION.md"
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "gpu_model_data.cc")
        with open(src, "w") as f:
            f.write(blocks[0] + "\nint main() { nimble::GpuModelData m; return 0; }\n")
        r = subprocess.run(["g++", "-std=c++14", "-fsyntax-only", "-I" + REF_SRC, "-I" + os.path.join(ROOT, "include"),
                            "-include", os.path.join(ROOT, "oracle", "ref_shim.h"), src],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
