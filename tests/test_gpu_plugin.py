"""Block materials computed by callbacks (the plugin path of the reference's
BlockMaterialInterface): the split step (kinematics, the callback's stress,
forces from the recorded stress), the n / n+1 record and state buffers, the
request a callback receives, and failure reporting.  The library's example
callbacks compute the neo-Hookean stress with the engine's own arithmetic,
so a run through them must match the built-in material."""
import ctypes as C

import numpy as np
import pytest

from nimblesm_gb300 import engine as E
from nimblesm_gb300.mesh import Material, cube_problem, critical_time_step
from oracle import oracle as O
from tests.gpu_util import rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from nimblesm_gb300 import build as B
    B.build()
    O.build(ref=False)


class Request(C.Structure):
    """nsm_stress_request (include/nimble_gb300.h)."""
    _fields_ = [("block", C.c_int), ("elem_begin", C.c_int), ("elem_end", C.c_int), ("precision", C.c_int),
                ("ld_e", C.c_long), ("records_n", C.c_void_p), ("records_np1", C.c_void_p), ("num_state", C.c_int),
                ("state_n", C.c_void_p), ("state_np1", C.c_void_p), ("time_n", C.c_double), ("time_np1", C.c_double),
                ("density", C.c_double), ("bulk_modulus", C.c_double), ("shear_modulus", C.c_double),
                ("stream", C.c_void_p)]


def _run(p, steps, precision="fp64", callback=None, block=0, num_state=0):
    m = E.Model(p, precision=precision)
    if callback is not None:
        m.set_block_material_callback(block, callback, num_state)
    dt = 0.5 * critical_time_step(p)
    m.begin(steps * dt, steps, 0)
    m.advance(steps)
    st = m.state()
    m.close()
    return st


def test_example_callback_matches_the_builtin_material_and_the_oracle():
    p = cube_problem(8, jitter=0.2, seed=11)
    steps = 40
    a = _run(p, steps)
    b = _run(p, steps, callback=E.example_callback("neohookean"))
    r = O.run_port(p, steps * 0.5 * critical_time_step(p), steps, 0)
    for k in ("u", "v", "sigma"):
        assert rel(b[k], a[k]) <= 1e-10, (k, rel(b[k], a[k]))
        assert rel(b[k], r[k]) <= 1e-10, (k, rel(b[k], r[k]))
    assert rel(b["F"], a["F"]) <= 1e-10  # the records the kinematics pass wrote


def test_example_callback_in_the_fp32_form():
    p = cube_problem(8, jitter=0.2, seed=12)
    steps = 40
    ref = _run(p, steps)  # FP64, built-in
    b = _run(p, steps, precision="fp32", callback=E.example_callback("neohookean"))
    assert rel(b["u"], ref["u"]) < 1e-3


def test_callback_on_one_block_of_two():
    p = cube_problem(6, jitter=0.2, seed=13)
    p.elem_block = (np.arange(p.num_elem) >= p.num_elem // 2).astype(np.int32)
    p.blocks = [Material("elastic", 7800.0, 1.6e11, 0.793e11), Material("neohookean", 7800.0, 1.6e11, 0.793e11)]
    steps = 30
    a = _run(p, steps)
    b = _run(p, steps, callback=E.example_callback("neohookean"), block=1)
    for k in ("u", "v", "sigma"):
        assert rel(b[k], a[k]) <= 1e-10, (k, rel(b[k], a[k]))


def _det(F):
    """det of [..., 9] full tensors in the reference's K_F slot order (xx yy zz xy yz zx yx zy xz)."""
    xx, yy, zz, xy, yz, zx, yx, zy, xz = (F[..., k] for k in range(9))
    return xx * (yy * zz - yz * zy) - xy * (yx * zz - yz * zx) + xz * (yx * zy - yy * zx)


def test_history_state_follows_the_step_records():
    """One state variable per point, state_np1 = state_n + |det F_np1 - det F_n|:
    after each step it equals the same sum over the F records read back."""
    p = cube_problem(5, jitter=0.2, seed=14)
    m = E.Model(p)
    m.set_block_material_callback(0, E.example_callback("history"), 1)
    dt = 0.5 * critical_time_step(p)
    m.begin(12 * dt, 12, 0)
    J_prev = np.ones((p.num_elem, 8))
    expect = np.zeros((p.num_elem, 8))
    for _ in range(12):
        m.advance(1)
        F, _ = m.GetIntegrationPointData()
        J = _det(F)
        expect += np.abs(J - J_prev)
        J_prev = J
        s = m.get_state_data()[..., 0]
        assert np.allclose(s, expect, rtol=1e-9, atol=1e-15)
    assert expect.max() > 0
    m.close()


def test_request_contents_and_failures():
    """A Python callback sees each step's block range, times and alternating
    record buffers, delegates the stress to the library's example, and a
    nonzero return fails the step with NSM_ERR_STATE."""
    p = cube_problem(4, jitter=0.2, seed=15)
    seen = []
    example = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p)(E.example_callback("neohookean"))

    def probe(user, req):
        r = Request.from_address(req)
        seen.append((r.block, r.elem_begin, r.elem_end, r.time_n, r.time_np1, r.records_n, r.records_np1,
                     r.bulk_modulus, r.shear_modulus))
        return example(user, req)

    cb = E.STRESS_CALLBACK(probe)
    m = E.Model(p)
    m.set_block_material_callback(0, cb)
    dt = 0.5 * critical_time_step(p)
    m.begin(5 * dt, 5, 0)
    m.advance(5)
    assert [s[:3] for s in seen] == [(0, 0, p.num_elem)] * 5
    for i, s in enumerate(seen):
        assert np.isclose(s[3], i * dt, rtol=1e-12, atol=0) and np.isclose(s[4], (i + 1) * dt, rtol=1e-12)
        assert s[7] == p.bulk_modulus and s[8] == p.shear_modulus
    assert seen[0][5] == seen[1][6] and seen[0][6] == seen[1][5]  # the buffers alternate
    m.close()

    fail = E.STRESS_CALLBACK(lambda user, req: 1)
    m = E.Model(p)
    m.set_block_material_callback(0, fail)
    m.begin(5 * dt, 5, 0)
    with pytest.raises(E.EngineError) as ei:
        m.advance(1)
    assert ei.value.code == 5  # NSM_ERR_STATE
    m.close()
