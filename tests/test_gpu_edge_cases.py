"""Edge cases of the engine's inputs: an empty model, an empty sample inside an
ensemble, nodes with more element incidences than a structured mesh has (the
gather's general path), and element counts that leave partial warps and
chunks at every boundary of the kernels' tilings.  Parity against the CPU
oracle (1e-10) or bitwise against the single runs, as the case allows."""
import numpy as np
import pytest

from nimblesm_gb300 import engine as E
from nimblesm_gb300.mesh import Problem, cube_problem, critical_time_step
from oracle import oracle as O
from tests.gpu_util import rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from nimblesm_gb300 import build as B
    B.build()
    O.build(ref=False)


def empty_problem():
    return Problem(coords=np.zeros((0, 3)), conn=np.zeros((0, 8), np.int32))


def oracle_sensitivity(p, final_time, steps):
    """The reference's own sensitivity on this run (the oracle is bitwise the
    reference): its u, v, sigma after the initial velocity is perturbed by
    one ulp (relative 2^-52, seeded signs)."""
    r0 = O.run_port(p, final_time, steps, 0)
    q = Problem(**{**p.__dict__})
    rng = np.random.default_rng(77)
    q.v_init = p.v_init * (1.0 + rng.choice([-1.0, 1.0], size=p.v_init.shape) * 2.0 ** -52)
    r1 = O.run_port(q, final_time, steps, 0)
    return r0, {k: rel(r1[k], r0[k]) for k in ("u", "v", "sigma")}


def test_empty_model_runs():
    """No nodes and no elements: creation, the schedule, stepping, the
    host-buffer call and every read-back work on empty arrays."""
    m = E.Model(empty_problem())
    assert m.GetCriticalTimeStep() == np.finfo(np.float64).max
    m.begin(1.0e-6, 10, 5)
    m.advance(10)
    st = m.state()
    assert st["u"].shape == (0, 3) and st["sigma"].shape == (0, 8, 6) and st["mass"].shape == (0,)
    assert m.ComputeInternalForceHost(np.zeros((0, 3))).shape == (0, 3)
    assert m.ComputeDerivedElementData()[0].shape == (0,)
    m.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_empty_sample_in_an_ensemble(precision):
    """A sample with no nodes and no elements between two others: the others
    are bitwise their single runs."""
    probs = [cube_problem(3, jitter=0.2, seed=1), empty_problem(), cube_problem(4, jitter=0.2, seed=2)]
    steps = 30
    ens = E.Model(probs, precision=precision)
    dts = ens.sample_time_steps()
    assert dts[1] == np.finfo(np.float64).max
    final = [steps * 0.5 * d for d in (dts[0], dts[0], dts[2])]
    ens.begin(final, steps, 0)
    ens.advance(steps)
    st = ens.state()
    for g in (0, 2):
        single = E.Model(probs[g], precision=precision)
        single.begin(final[g], steps, 0)
        single.advance(steps)
        s1 = single.state()
        sl = ens.sample_slice(g)
        es = slice(int(ens.elem_offsets[g]), int(ens.elem_offsets[g + 1]))
        for k in ("u", "v", "a", "f_int"):
            assert np.array_equal(st[k][sl], s1[k]), (g, k)
        assert np.array_equal(st["sigma"][es], s1["sigma"]), g
        single.close()
    ens.close()


def test_nodes_with_sixteen_incidences_against_the_oracle():
    """Every element listed twice: interior nodes gather 16 element
    contributions (the gather's general path past the first eight), in
    increasing element order as the reference's serial scatter does."""
    p = cube_problem(4, jitter=0.2, seed=3)
    p.conn = np.ascontiguousarray(np.concatenate([p.conn, p.conn]))
    dt = 0.5 * critical_time_step(p)
    steps = 40
    g = E.run(p, steps * dt, steps)
    r = O.run_port(p, steps * dt, steps, 0)
    assert np.array_equal(g["mass"], r["mass"]) and g["dt_crit"] == r["dt_crit"]
    for k in ("u", "v"):
        assert rel(g[k], r[k]) <= 1e-10, (k, rel(g[k], r[k]))
    assert rel(g["sigma"], r["sigma"]) <= 1e-10


@pytest.mark.parametrize("dims", [(1, 1, 1), (3, 1, 1), (31, 1, 1), (33, 1, 1), (129, 1, 1), (5, 7, 3)])
def test_partial_warps_and_chunks_against_the_oracle(dims):
    """Element counts around the tilings' boundaries: 1, 3, 31, 33 (warps of
    32), 129 (blocks of 128), 105; FP64 against the oracle, and the host
    pipeline at 7 chunks bitwise the one-launch path."""
    nx, ny, nz = dims
    xs, ys, zs = (np.linspace(0.0, d / 4.0, d + 1) for d in dims)
    X, Y, Z = np.meshgrid(xs, ys, zs, indexing="ij")
    coords = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    rng = np.random.default_rng(sum(dims))
    coords = coords + rng.uniform(-0.02, 0.02, coords.shape)
    idx = lambda i, j, k: (i * (ny + 1) + j) * (nz + 1) + k
    conn = np.array([[idx(i, j, k), idx(i + 1, j, k), idx(i + 1, j + 1, k), idx(i, j + 1, k),
                      idx(i, j, k + 1), idx(i + 1, j, k + 1), idx(i + 1, j + 1, k + 1), idx(i, j + 1, k + 1)]
                     for i in range(nx) for j in range(ny) for k in range(nz)], np.int32)
    p = Problem(coords=coords, conn=conn, v_init=rng.uniform(-1.0, 1.0, coords.shape))
    dt = 0.5 * critical_time_step(p)
    steps = 25
    g = E.run(p, steps * dt, steps)
    # a random velocity per node is all high-frequency content, to which a
    # 1-ulp change of the input moves the reference itself by ~1e-10 in v:
    # the bound is 1e-10 or twice that sensitivity
    r, env = oracle_sensitivity(p, steps * dt, steps)
    for k in ("u", "v", "sigma"):
        assert rel(g[k], r[k]) <= max(1e-10, 2 * env[k]), (dims, k, rel(g[k], r[k]), env[k])
    m = E.Model(p)
    u = rng.normal(0, 1e-4, size=(p.num_nodes, 3))
    m.SetVectorNodeData("displacement", u)
    m.ComputeInternalForce()
    ref = m.GetVectorNodeData("internal_force")
    m.set_host_chunks(min(7, p.num_elem))
    assert np.array_equal(m.ComputeInternalForceHost(u), ref)
    m.close()


def test_a_traction_line_applies_nothing():
    """The reference parses prescribed_traction lines and applies nothing
    (ApplyTractionBC is empty): the run is bitwise the run without the line,
    also when the line's set name is a node set's."""
    from nimblesm_gb300.mesh import BoundaryCondition
    p = cube_problem(4, jitter=0.2, seed=9)
    q = cube_problem(4, jitter=0.2, seed=9)
    q.bcs = q.bcs + [BoundaryCondition.parse("prescribed_traction nodelist_2 z 1.0e6")]
    dt = 0.5 * critical_time_step(p)
    a, b = E.run(p, 20 * dt, 20), E.run(q, 20 * dt, 20)
    for k in ("u", "v", "sigma"):
        assert np.array_equal(a[k], b[k]), k


def test_external_force_is_zero():
    """ModelData::ComputeExternalForce zeroes the external force every step:
    the field reads as zero and writing it is refused."""
    p = cube_problem(3, jitter=0.2, seed=10)
    m = E.Model(p)
    dt = 0.5 * critical_time_step(p)
    m.begin(5 * dt, 5, 0)
    m.advance(5)
    assert not np.any(m.GetVectorNodeData("external_force"))
    with pytest.raises(E.EngineError):
        m.SetVectorNodeData("external_force", np.ones((p.num_nodes, 3)))
    m.close()
