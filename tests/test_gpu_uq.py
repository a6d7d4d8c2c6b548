"""The reference's UQ mode on the GPU (nsm_create_uq / UqModel): nominal, exact
and approximate trajectories with the linear force closure, against the
reference's own UQ run of its uq_wave deck and against the oracle."""
import numpy as np
import pytest

from nimblesm_gb300 import engine as E
from nimblesm_gb300.mesh import BoundaryCondition, Material, cube_problem, critical_time_step
from nimblesm_gb300.uq import UqSpec
from oracle import oracle as O
from tests.goldens import load, output_steps, uq_problem
from tests.gpu_util import rel

pytestmark = pytest.mark.gpu
TOL = 1e-10


@pytest.fixture(scope="module", autouse=True)
def _built():
    from nimblesm_gb300 import build as B
    B.build()
    O.build(ref=False)


def force_floor(p, K):
    """The FP64 resolution of a nodal force at this modulus and mesh: 64 ulps
    of F = I times K times a typical element face area, normwise over the
    nodes (where the exact stress is zero -- a rigidly moving part of the
    mesh -- the reference's force is round-off of this size)."""
    ext = p.coords.max(axis=0) - p.coords.min(axis=0)
    area = (np.prod(ext) / p.num_elem) ** (2.0 / 3.0)
    return 64 * np.finfo(np.float64).eps * K * area * np.sqrt(3 * p.num_nodes)


def close(ours, ref, floor=0.0):
    return np.linalg.norm(ours - ref) <= max(TOL * np.linalg.norm(ref), floor)


def check_trajectories(m, ref, t, p):
    u, v, f = m.trajectories("displacement"), m.trajectories("velocity"), m.trajectories("internal_force")
    K = max(mt.bulk_modulus for mt in p.materials())
    for ours, key_nom, key_s, floor in ((u, "u", "su", 0.0), (v, "v", "sv", 0.0), (f, "f", "sf", force_floor(p, K))):
        assert close(ours[0], ref[key_nom][t], floor), (key_nom, t, rel(ours[0], ref[key_nom][t]))
        for s in range(ours.shape[0] - 1):
            assert close(ours[1 + s], ref[key_s][t][s], floor), (key_s, s, t, rel(ours[1 + s], ref[key_s][t][s]))


def test_uq_wave_against_reference():
    """uq_wave (100 elements, 2 exact + 5 approximate trajectories, 10,000
    steps): every trajectory within 1e-10 of the reference's UQ run."""
    fx = load("ref_uq_wave")
    p, spec = uq_problem(fx)
    steps, of = int(fx["num_steps"]), int(fx["output_frequency"])
    m = E.UqModel(p, spec, graph_steps=100)
    m.begin(float(fx["final_time"]), steps, of)
    done = 0
    for t, s_end in enumerate(fx["out_steps"]):
        m.advance(int(s_end) - done)
        done = int(s_end)
        check_trajectories(m, fx, t, p)
    m.close()


def jittered_uq():
    p = cube_problem(10, jitter=0.2, seed=9)
    p.blocks = [Material("neohookean", 7800.0, 160e9, 79.3e9), Material("elastic", 7800.0, 140e9, 60e9)]
    p.elem_block = (np.arange(p.num_elem) >= p.num_elem // 2).astype(np.int32)
    p.bcs = p.bcs + [BoundaryCondition.parse("prescribed_displacement nodelist_2 z 1e-5")]
    spec = UqSpec([(0, "bulk_modulus", 2.0e10), (1, "shear_modulus", 1.0e10), (0, "shear_modulus", 5.0e9)],
                  [[-1.0, 0.5, 0.2], [1.0, -0.5, -0.2], [0.3, 0.9, -0.6]],
                  [[0.0, 0.0, 0.0], [-0.5, 0.2, 0.1], [0.4, 0.4, 0.4], [0.9, -0.9, 0.3]],
                  [[1.0, 0.0, 0.0, 0.0], [0.3, 0.3, 0.2, 0.2], [0.1, 0.5, 0.2, 0.2], [0.0, 0.25, 0.25, 0.5]])
    return p, spec


def test_uq_cube_against_oracle():
    """A jittered cube of two element blocks (neo-Hookean and elastic), three
    uncertain parameters, 3 exact and 4 approximate trajectories, a prescribed
    displacement (nominal only): every trajectory within 1e-10 of the
    oracle's restatement of the reference's UQ mode."""
    p, spec = jittered_uq()
    dt = 0.5 * critical_time_step(p)
    steps, of = 240, 60
    ref = O.run_port_uq(p, spec, steps * dt, steps, of, threads=8)
    m = E.UqModel(p, spec, graph_steps=50)
    m.begin(steps * dt, steps, of)
    done = 0
    for t, s_end in enumerate(output_steps(steps, of)):
        m.advance(s_end - done)
        done = s_end
        check_trajectories(m, ref, t, p)
    m.close()


def test_uq_nominal_is_the_plain_run():
    """The nominal trajectory of a UQ handle is bitwise the plain run of the
    same problem (same kernels, same assembly order)."""
    p, spec = jittered_uq()
    dt = 0.5 * critical_time_step(p)
    m = E.UqModel(p, spec)
    m.begin(100 * dt, 100, 0)
    m.advance(100)
    plain = E.Model(p)
    plain.begin(100 * dt, 100, 0)
    plain.advance(100)
    assert np.array_equal(m.trajectories("displacement")[0], plain.GetVectorNodeData("displacement"))
    assert np.array_equal(m.trajectories("velocity")[0], plain.GetVectorNodeData("velocity"))
    m.close()
    plain.close()


def test_uq_fp32_mixed():
    """The FP32-mixed form of the UQ mode within 1e-3 of the FP64 form."""
    p, spec = jittered_uq()
    dt = 0.5 * critical_time_step(p)
    out = {}
    for prec in ("fp64", "fp32"):
        m = E.UqModel(p, spec, precision=prec)
        m.begin(200 * dt, 200, 0)
        m.advance(200)
        out[prec] = m.trajectories("displacement")
        m.close()
    assert rel(out["fp32"], out["fp64"]) < 1e-3
