"""The FP64 element kernel forms the diagonal of F = I + H with integer
operations (hex_math.cuh: one_plus), off the FP64 pipe.  This compiles the
same function for the host and checks it against the FP64 add bit for bit."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_one_plus_matches_the_fp64_add(tmp_path):
    nvcc = shutil.which(os.environ.get("NVCC", "nvcc"))
    if nvcc is None:
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "one_plus_check")
    subprocess.run([nvcc, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "nimblesm_gb300", "csrc"),
                    "-I", os.path.join(ROOT, "include"), os.path.join(HERE, "one_plus_check.cu"), "-o", exe],
                   check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " 0 mismatches" in r.stdout
