"""The reference-side adapter (integration/gpu_model_data.h) run inside the
reference's own DataManager and explicit loop, on the CPU.

The reference is built from its sources (oracle/Makefile -> oracle/_ref) with
its one ModelData hook pointed at nimble::GpuModelData
(tests/adapter/adapter_shim.h, the line a maintainer changes in
DataManager::Initialize), and the engine's C ABI is replaced by a TEST-ONLY
stand-in built on the CPU oracle (tests/adapter/nsm_abi_stub.cc), which is
bitwise the reference's element arithmetic.  So a run through the adapter must
equal a plain reference run bit for bit: u, v, a and f_int after every output
step, and the deformation gradient and stress of every integration point that
the adapter copies into the reference's element data on output steps.  That
pins the adapter's marshalling: the [N][3] node views, the block order, the
element-data offsets and the elastic / neo-Hookean material mapping.

Runs where the reference sources are present (NIMBLESM_REFERENCE)."""
import ctypes as C
import glob
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ADAPTER_DIR = os.path.join(ROOT, "tests", "adapter")
OUT = os.path.join(ROOT, "oracle", "_ref", "adapter")
LIB = os.path.join(OUT, "libnimble_ref_adapter.so")

pytestmark = pytest.mark.skipif(not os.path.isdir(O.REF_SRC) or shutil.which("g++") is None,
                                reason="reference sources not present")


def _build():
    O.build(ref=True)
    os.makedirs(OUT, exist_ok=True)
    flags = ["-std=c++14", "-O3", "-DNDEBUG", "-fPIC", "-ffp-contract=off", "-I" + O.REF_SRC,
             "-I" + os.path.join(ROOT, "integration"), "-I" + os.path.join(ROOT, "include"),
             "-I" + os.path.join(ROOT, "oracle")]
    shim = ["-include", os.path.join(ADAPTER_DIR, "adapter_shim.h")]
    jobs = [
        ["g++"] + flags + shim + ["-c", os.path.join(O.REF_SRC, "nimble_data_manager.cc"),
                                  "-o", os.path.join(OUT, "nimble_data_manager.o")],
        ["g++"] + flags + shim + ["-c", os.path.join(ROOT, "oracle", "ref_harness.cc"),
                                  "-o", os.path.join(OUT, "ref_harness.o")],
        ["g++"] + flags + ["-c", os.path.join(ADAPTER_DIR, "nsm_abi_stub.cc"), "-o", os.path.join(OUT, "stub.o")],
        ["gcc", "-std=c11", "-O3", "-fPIC", "-ffp-contract=off", "-fopenmp", "-c",
         os.path.join(ROOT, "oracle", "nsm_oracle.c"), "-o", os.path.join(OUT, "nsm_oracle.o")],
    ]
    procs = [subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True) for j in jobs]
    for j, p in zip(jobs, procs):
        _, err = p.communicate()
        assert p.returncode == 0, " ".join(j[-3:]) + "\n" + err[-3000:]
    ref_objs = [o for o in sorted(glob.glob(os.path.join(ROOT, "oracle", "_ref", "obj", "*.o")))
                if os.path.basename(o) not in ("nimble_data_manager.o", "ref_harness.o")]
    objs = [os.path.join(OUT, f) for f in ("nimble_data_manager.o", "ref_harness.o", "stub.o", "nsm_oracle.o")]
    r = subprocess.run(["g++", "-shared", "-fopenmp", "-o", LIB] + objs + ref_objs, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    lib = C.CDLL(LIB)
    _dp, _ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
    lib.nimref_run_blocks.argtypes = [C.c_int, _dp, C.c_int, _ip, C.c_int, _ip, C.c_char_p, C.c_int, _ip, _ip,
                                      C.c_char_p, C.c_char_p, C.c_double, C.c_int, C.c_int, _dp, C.c_int,
                                      _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _ip]
    lib.nimref_last_error.restype = C.c_char_p
    return lib


@pytest.fixture(scope="module")
def adapter_lib():
    return _build()


def _cases():
    from nimblesm_gb300.mesh import cube_problem, critical_time_step
    from tests.goldens import gold_problem

    p = cube_problem(5, jitter=0.2, seed=4)
    dt = 0.5 * critical_time_step(p)
    yield "jittered 5^3 cube", p, 30 * dt, 30, 7
    for deck in ("brick_with_fibers", "notched_plate_native_hypoelastic"):
        fx = np.load(os.path.join(ROOT, "tests", "golden", f"gold_{deck}.npz"))
        q = gold_problem(fx)
        steps = min(int(fx["num_steps"]), 60)
        yield deck, q, float(fx["final_time"]) * steps / int(fx["num_steps"]), steps, 20


def test_adapter_runs_inside_the_reference_loop_bitwise(adapter_lib):
    for name, p, final_time, steps, of in _cases():
        plain = O.run_ref_outputs(p, final_time, steps, of)
        via = O.run_ref_outputs(p, final_time, steps, of, lib=adapter_lib)
        assert len(plain) == len(via) >= 3, name
        for t, (a, b) in enumerate(zip(plain, via)):
            for k in ("u", "v", "a", "f_int", "F", "sigma", "mass"):
                assert np.array_equal(a[k], b[k]), f"{name}: {k} differs at output {t}"
            assert a["dt_crit"] == b["dt_crit"], name
        # the copy is not vacuous: the stresses of the last output are not zero
        assert np.abs(via[-1]["sigma"]).max() > 0, name
