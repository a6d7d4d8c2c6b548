"""Parity of the CUDA engine (through the C ABI) with the CPU oracle and the
reference's gold files.

Tolerance for the FP64 form: 1e-10 relative (normwise over the field) in
nodal displacement, velocity and integration-point stress after N steps; the
lumped mass and the critical time step are bit-exact (same arithmetic order,
no FMA contraction).  FP32-mixed form: 1e-3 relative displacement error
against the FP64 form."""
import numpy as np
import pytest

from nimblesm_gb300 import engine as E
from nimblesm_gb300.mesh import BC_PRESCRIBED_DISPLACEMENT, BoundaryCondition, cube_problem, critical_time_step
from oracle import oracle as O
from tests.goldens import GOLD_DECKS, exodiff_ok, gold_checks, gold_problem, load, output_steps
from tests.gpu_util import rel

pytestmark = pytest.mark.gpu
TOL = 1e-10  # FP64 parity target, relative (normwise over the field)


@pytest.fixture(scope="module", autouse=True)
def _built():
    from nimblesm_gb300 import build as B
    B.build()
    O.build(ref=False)


def compare(gpu, ref, keys=("u", "v", "sigma"), tol=TOL, sigma_tol=None, v_tol=None):
    """u, v within 1e-10 of the reference.  sigma (and, on long schedules, v)
    within 1e-10 or, where the reference itself is less reproducible than
    that, within twice its measured sensitivity (sigma_tol / v_tol, from the
    reference: a 1-ulp input perturbation or its stress-evaluation error
    against extended precision)."""
    for k in keys:
        t = tol
        if k == "sigma" and sigma_tol:
            t = max(tol, sigma_tol)
        if k == "v" and v_tol:
            t = max(tol, v_tol)
        e = rel(gpu[k], ref[k])
        assert e <= t, f"{k}: relative error {e:.3e} > {t:.3e}"


def sigma_floor(problem, state, sample=4096, seed=0):
    """Twice the reference's stress-evaluation error on a sample of elements,
    against the extended-precision stress of the same displacement."""
    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(problem.num_elem, min(sample, problem.num_elem), replace=False)).astype(np.int32)
    exact = O.stress_exact(problem, state["u"], idx)
    return 2.0 * rel(state["sigma"][idx], exact), idx


def test_single_element_known_answers():
    """Each reference element of the known-answer fixture, as a one-element
    mesh: F, sigma and nodal forces against the reference's values."""
    fx = load("ref_points")
    for k in range(fx["elem_X"].shape[0]):
        p = cube_problem(1)
        p.coords = fx["elem_X"][k].copy()  # corner order
        p.conn = np.arange(8, dtype=np.int32)[None, :]
        p.bcs, p.v_init = [], None
        p.bulk_modulus, p.shear_modulus = float(fx["K"]), float(fx["G"])
        m = E.Model(p)
        m.SetVectorNodeData("displacement", fx["elem_u"][k])
        m.ComputeInternalForce()
        f = m.GetVectorNodeData("internal_force")
        F, s = m.GetIntegrationPointData()
        assert rel(F, fx["elem_F"][k]) < 1e-13
        assert rel(s, fx["elem_sigma"][k]) < 1e-9
        assert rel(f, fx["elem_f"][k]) < 1e-9
        m.close()


@pytest.mark.parametrize("name", ["cube4_jitter", "cube16_cfg0"])
def test_cube_against_reference_fixture(name):
    fx = load("ref_" + name)
    p = cube_problem(int(fx["n"]), jitter=float(fx["jitter"]), seed=int(fx["seed"]))
    g = E.run(p, float(fx["final_time"]), int(fx["steps"]), int(fx["output_frequency"]))
    assert g["dt_crit"] == float(fx["dt_crit"])
    assert np.array_equal(g["mass"], fx["mass"])
    idx = fx.get("elem_index")
    ref = {k: fx[k] for k in ("u", "v", "a", "f_int")}
    ref["sigma"] = fx["sigma"]
    gs = g["sigma"] if idx is None else g["sigma"][idx]
    # sampled elements: allow 3x the reference's 1-ulp envelope (subset statistics)
    compare({"u": g["u"], "v": g["v"], "sigma": gs}, ref, sigma_tol=3.0 * float(fx["envelope_sigma"]))
    assert rel(g["a"], fx["a"]) < 1e-9 and rel(g["f_int"], fx["f_int"]) < 1e-9
    if idx is not None:
        e = rel(g["sigma"].mean(axis=1), fx["sigma_elem"])
        assert e <= max(TOL, 2.0 * float(fx["envelope_sigma_elem"])), e


@pytest.mark.parametrize("name", GOLD_DECKS)
def test_gold_decks(name):
    """The reference's regression decks (neo-Hookean and elastic materials,
    one and two element blocks) at every output time: exodiff tolerances
    against the gold files, including the derived element output; 1e-10
    against the reference run; lumped mass bit for bit."""
    fx, rf = load("gold_" + name), load("ref_" + name)
    p = gold_problem(fx)
    steps, of = int(fx["num_steps"]), int(fx["output_frequency"])
    m = E.Model(p)
    assert np.array_equal(m.ComputeLumpedMass(), rf["mass"])
    m.begin(float(fx["final_time"]), steps, of)
    done = 0
    for t, s_end in enumerate(output_steps(steps, of)):
        m.advance(s_end - done)
        done = s_end
        st = m.state()
        vol, sig_avg, F_avg = m.ComputeDerivedElementData()
        gold_checks(fx, t, st, vol, sig_avg, F_avg)
        K = float(np.max(fx["block_params"][:, 1]))
        assert stress_close(st["sigma"], rf["sigma"][t], K)
        assert stress_close(sig_avg, rf["sigma_avg"][t], K)
        compare(st, {"u": rf["u"][t], "v": rf["v"][t]}, keys=("u", "v"))
        assert rel(vol, rf["volume"][t]) < TOL and rel(F_avg, rf["F_avg"][t]) < TOL
    m.close()


def stress_close(ours, ref, K):
    """Normwise 1e-10 relative, with the FP64 resolution of a stress at this
    modulus as the floor: a few ulps of F = I times K per component (the
    rigid-motion deck's exact stress is zero and the reference's is
    round-off of that size)."""
    floor = 64 * np.finfo(np.float64).eps * K * np.sqrt(ours.size)
    return np.linalg.norm(ours - ref) <= max(TOL * np.linalg.norm(ref), floor)


def test_jittered_cube_against_oracle_with_output_steps():
    p = cube_problem(12, jitter=0.2, seed=21)
    dt = 0.5 * critical_time_step(p)
    steps = 300
    ref = O.run_port(p, steps * dt, steps, 70, threads=8)
    g = E.run(p, steps * dt, steps, 70)
    compare(g, ref)
    assert np.array_equal(g["mass"], ref["mass"])
    assert abs(g["kinetic_energy"] - ref["kinetic_energy"]) <= 1e-9 * ref["kinetic_energy"]
    assert abs(g["internal_energy"] - ref["internal_energy"]) <= 1e-8 * ref["internal_energy"]


def test_prescribed_displacement_and_initial_velocity():
    p = cube_problem(6, jitter=0.15, seed=3)
    p.bcs = [BoundaryCondition.parse("initial_velocity nodelist_2 x 2.5"),
             BoundaryCondition.parse("prescribed_velocity nodelist_1 x 0.0"),
             BoundaryCondition.parse("prescribed_velocity nodelist_1 y 0.0"),
             BoundaryCondition.parse("prescribed_displacement nodelist_1 z 1.0e-4"),
             BoundaryCondition(BC_PRESCRIBED_DISPLACEMENT, "nodelist_2", 1, -2.0e-5)]
    p.v_init = None
    dt = 0.5 * critical_time_step(p)
    ref = O.run_port(p, 150 * dt, 150, 40)
    g = E.run(p, 150 * dt, 150, 40)
    compare(g, ref)


def test_advance_in_pieces_equals_one_advance():
    p = cube_problem(8, jitter=0.2, seed=4)
    dt = 0.5 * critical_time_step(p)
    a = E.Model(p, graph_steps=7)
    a.begin(90 * dt, 90, 25)
    for k in (1, 13, 50, 26):
        a.advance(k)
    sa = a.state()
    b = E.Model(p)
    b.begin(90 * dt, 90, 25)
    b.advance(90)
    sb = b.state()
    for k in ("u", "v", "a", "f_int", "F", "sigma"):
        assert np.array_equal(sa[k], sb[k]), k


def test_runs_are_bitwise_deterministic():
    p = cube_problem(10, jitter=0.2, seed=8)
    dt = 0.5 * critical_time_step(p)
    r1 = E.run(p, 40 * dt, 40)
    r2 = E.run(p, 40 * dt, 40)
    for k in ("u", "v", "a", "f_int", "F", "sigma"):
        assert np.array_equal(r1[k], r2[k]), k


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_every_launch_shape_gives_the_same_bits(precision):
    """Every launch shape the autotuner may pick (one pass, register-bounded,
    persistent, and in the FP32 form the cp.async-staged persistent grid)
    runs the same element arithmetic: a 40-step run is bitwise the same, on
    one mesh and on an ensemble of uneven meshes with per-sample materials."""
    meshes = [cube_problem(13, jitter=0.2, seed=21)]
    ens = [cube_problem(n, jitter=0.2, seed=30 + n) for n in (5, 9, 7)]
    for i, q in enumerate(ens):
        q.bulk_modulus *= 1.0 + 0.1 * i
        q.shear_modulus *= 1.0 - 0.05 * i
    steps = 40
    for probs in (meshes, ens):
        dts = [0.5 * critical_time_step(q) for q in probs]
        ref = None
        count = len(E.Model(probs if len(probs) > 1 else probs[0], precision=precision).launch_candidate_times(1))
        for c in range(count):
            m = E.Model(probs if len(probs) > 1 else probs[0], precision=precision)
            m.set_launch_candidate(c)
            if len(probs) > 1:
                m.begin([steps * d for d in dts], steps, 0)
            else:
                m.begin(steps * dts[0], steps, 0)
            m.advance(steps)
            st = m.state()
            m.close()
            if ref is None:
                ref = st
                continue
            for k in ("u", "v", "f_int", "F", "sigma"):
                assert np.array_equal(st[k], ref[k]), (len(probs), c, k)


def test_host_buffer_internal_force_matches_device_path():
    p = cube_problem(6, jitter=0.2, seed=9)
    rng = np.random.default_rng(0)
    u = rng.normal(0, 1e-4, size=(p.num_nodes, 3))
    m = E.Model(p)
    pinned = E.PinnedArray((p.num_nodes, 3))
    pinned.array[:] = u
    out = E.PinnedArray((p.num_nodes, 3))
    f_host = m.ComputeInternalForceHost(pinned.array, out.array).copy()
    m.SetVectorNodeData("displacement", u)
    m.ComputeInternalForce()
    assert np.array_equal(f_host, m.GetVectorNodeData("internal_force"))
    # against the oracle's element arithmetic, assembled in element order
    fo = np.zeros((p.num_nodes, 3))
    for e in range(p.num_elem):
        X, ue = p.coords[p.conn[e]], u[p.conn[e]]
        _, _, f = O.element(X, ue, p.bulk_modulus, p.shear_modulus)
        for c in range(8):
            fo[p.conn[e, c]] += f[c]
    assert rel(f_host, fo) < 1e-10


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_host_pipeline_chunks_give_the_same_bits(precision):
    """The host-buffer call as a pipeline of element ranges (u copied in
    ahead of them, f_int copied out behind them) equals the one-launch device
    path bit for bit, at any chunk count: on a mesh in its natural order, on
    one whose elements are shuffled (few nodes are complete before the last
    chunk) and on an ensemble."""
    rng = np.random.default_rng(5)
    p = cube_problem(12, jitter=0.2, seed=31)
    shuffled = cube_problem(10, jitter=0.2, seed=32)
    shuffled.conn = np.ascontiguousarray(shuffled.conn[rng.permutation(shuffled.num_elem)])
    ens = [cube_problem(n, jitter=0.2, seed=40 + n) for n in (6, 9, 4)]
    for probs in ([p], [shuffled], ens):
        m = E.Model(probs if len(probs) > 1 else probs[0], precision=precision)
        N = m.problem.num_nodes
        u = rng.normal(0, 1e-4, size=(N, 3))
        m.SetVectorNodeData("displacement", u)
        m.ComputeInternalForce()
        ref = m.GetVectorNodeData("internal_force")
        ref_F, ref_s = m.GetIntegrationPointData()
        pin_u, pin_f = E.PinnedArray((N, 3)), E.PinnedArray((N, 3))
        pin_u.array[:] = u
        for k in (1, 2, 3, 7, 16):
            m.set_host_chunks(k)
            assert m.host_chunks() == k
            pin_f.array[:] = np.nan
            m.ComputeInternalForceHost(pin_u.array, pin_f.array)
            assert np.array_equal(pin_f.array, ref), (len(probs), k)
            F, sig = m.GetIntegrationPointData()
            assert np.array_equal(F, ref_F) and np.array_equal(sig, ref_s), (len(probs), k)
        m.set_host_chunks(0)
        m.close()


def test_host_loop_equals_device_loop():
    """The reference integrator's loop on host arrays around the host-buffer
    force call (the drop-in step, nsm_host_loop_steps) against the engine's
    device loop (nsm_advance) on the same schedule: bitwise the same u, v, a and
    f_int, with output steps in between (kinematic conditions on them)."""
    p = cube_problem(9, jitter=0.2, seed=21)
    dt = 0.5 * critical_time_step(p)
    steps, of = 37, 10
    dev = E.Model(p)
    dev.begin(steps * dt, steps, of)
    dev.advance(steps)
    g = dev.state(with_ip=False)
    dev.close()
    m = E.Model(p)
    m.begin(steps * dt, steps, of)  # initial and kinematic conditions at t = 0, as the reference's loop sets them
    mass = m.ComputeLumpedMass()
    pins = {k: E.PinnedArray((p.num_nodes, 3)) for k in ("u", "v", "a", "f")}
    pins["u"].array[:] = m.GetVectorNodeData("displacement")
    pins["v"].array[:] = m.GetVectorNodeData("velocity")
    pins["a"].array[:] = 0.0
    pins["f"].array[:] = 0.0
    t = 0.0
    for first, k in ((0, 13), (13, 24)):  # in two pieces
        t, host_s = m.HostLoopSteps(k, t, (steps * dt - 0.0) / steps, mass, pins["u"].array, pins["v"].array,
                                    pins["a"].array, pins["f"].array, output_frequency=of, first_step=first,
                                    num_load_steps=steps)
        assert host_s > 0.0
    for k, key in (("u", "u"), ("v", "v"), ("a", "a"), ("f", "f_int")):
        assert np.array_equal(pins[k].array, g[key]), key
    # a condition naming a node outside the model is refused before any step
    p.node_sets["nodelist_1"] = np.append(p.node_sets["nodelist_1"], p.num_nodes).astype(np.int32)
    with pytest.raises(E.EngineError, match="out of range"):
        m.HostLoopSteps(1, t, (steps * dt) / steps, mass, pins["u"].array, pins["v"].array, pins["a"].array,
                        pins["f"].array)
    m.close()


def test_fp32_mixed_within_1e3_of_fp64():
    p = cube_problem(16, jitter=0.2, seed=2)
    dt = 0.5 * critical_time_step(p)
    a = E.run(p, 500 * dt, 500, precision="fp64")
    b = E.run(p, 500 * dt, 500, precision="fp32")
    assert np.array_equal(a["mass"], b["mass"])
    e = rel(b["u"], a["u"])
    assert e < 1e-3, e
    assert rel(b["v"], a["v"]) < 1e-2


def test_fp32_point_records_match_fp64():
    """The FP32 form's F and sigma records, which whole warps write through a
    swizzled shared tile (partial warps lane by lane), agree entry by entry
    with the FP64 form's to FP32 accuracy; 1,331 elements give 41 whole warps
    and a partial one."""
    p = cube_problem(11, jitter=0.2, seed=4)
    dt = 0.5 * critical_time_step(p)
    out = {}
    for prec in ("fp64", "fp32"):
        m = E.Model(p, precision=prec)
        m.begin(30 * dt, 30, 0)
        m.advance(30)
        out[prec] = m.GetIntegrationPointData()
        m.close()
    (F64, S64), (F32, S32) = out["fp64"], out["fp32"]
    assert np.abs(F32 - F64).max() < 1e-5, np.abs(F32 - F64).max()
    scale = np.abs(S64).max()
    assert np.abs(S32 - S64).max() < 1e-3 * scale, np.abs(S32 - S64).max() / scale


def test_inverted_element_is_reported():
    """A mesh with an inverted element: the engine returns
    NSM_ERR_BAD_JACOBIAN at setup (the reference asserts,
    src/nimble_utils.h:1243-1255)."""
    p = cube_problem(2)
    c = p.conn.copy()
    c[0] = c[0][[4, 5, 6, 7, 0, 1, 2, 3]]  # swap top and bottom faces
    p.conn = c
    with pytest.raises(E.EngineError) as ei:
        E.Model(p)
    assert ei.value.code == 3


def test_large_deformation_reports_inversion_and_stays_usable():
    """Displacements that turn an element inside out flag the status word; the
    context stays usable for the next call."""
    p = cube_problem(3)
    m = E.Model(p)
    u = np.zeros((p.num_nodes, 3))
    u[p.conn[13, 6]] = [-0.8, -0.8, -0.8]  # push the centre element's (+,+,+) corner through
    m.SetVectorNodeData("displacement", u)
    with pytest.raises(E.EngineError) as ei:
        m.ComputeInternalForce()
    assert ei.value.code in (3, 4)
    m.SetVectorNodeData("displacement", np.zeros_like(u))
    m.ComputeInternalForce()
    assert np.all(m.GetVectorNodeData("internal_force") == 0.0)


def test_128_cube_first_steps_against_oracle():
    """The benchmark mesh (128^3 jittered, 2.1M nodes): the first steps
    against the oracle on all host cores, plus full-size invariants."""
    import os
    p = cube_problem(128, jitter=0.2, seed=0)
    dt = 0.5 * critical_time_step(p)
    steps = 4
    run = O.PortRun(p, threads=os.cpu_count())
    run.begin(2000 * dt, 2000, 0)
    run.advance(steps)
    ref = run.state()
    m = E.Model(p)
    assert m.GetCriticalTimeStep() == run.dt_crit
    m.begin(2000 * dt, 2000, 0)
    m.advance(steps)
    g = m.state()
    floor, idx = sigma_floor(p, ref)
    compare(g, ref, sigma_tol=floor)
    # the engine's stress is itself accurate: within 1e-10 of the
    # extended-precision stress of its own displacement
    assert rel(g["sigma"][idx], O.stress_exact(p, g["u"], idx)) < TOL
    m.close()


def test_full_schedule_against_oracle():
    """The workload's whole schedule, 2000 steps at dt = 0.5 dt_crit, on a
    40^3 jittered cube (the 128^3 benchmark mesh's construction, 512k
    integration points): FP64 parity with the oracle after the last step.
    Over 2000 steps the reference's own velocity and stress move by
    1.7e-10 / 1.1e-10 under a 1-ulp perturbation of the initial velocity
    (ref_cube40_schedule, measured on the reference), so v and sigma are held
    to twice that; u to 1e-10."""
    import os
    fx = load("ref_cube40_schedule")
    p = cube_problem(40, jitter=0.2, seed=0)
    dt = 0.5 * critical_time_step(p)
    steps = 2000
    run = O.PortRun(p, threads=os.cpu_count())
    run.begin(steps * dt, steps, 0)
    run.advance(steps)
    ref = run.state()
    assert run.dt_crit == float(fx["dt_crit"])
    m = E.Model(p, graph_steps=100)
    m.begin(steps * dt, steps, 0)
    m.advance(steps)
    g = m.state()
    floor, idx = sigma_floor(p, ref)
    compare(g, ref, sigma_tol=max(floor, 2.0 * float(fx["envelope_sigma"])), v_tol=2.0 * float(fx["envelope_v"]))
    m.close()


def test_128_cube_full_schedule_against_reference_fixture():
    """The benchmark configuration itself: the jittered 128^3 cube (2,097,152
    elements) over its whole 2000-step schedule at dt = 0.5 dt_crit, against
    the reference's result (ref_cube128_schedule: the oracle on 8 host
    threads, bitwise the reference's own code on this mesh, as the fixture
    script checks) on seeded subsets of 10,000 nodes (u, v, a, f_int) and
    2,048 elements (F and sigma of every point), on per-z-layer sums that
    every node and element enters, on the whole-field norms and on the kinetic
    and internal energy.

    u is held to 1e-10.  v, a, f_int, F and sigma are held to 1e-10 or twice
    the reference's own sensitivity at 128^3, measured on the same subset: its
    change when the initial velocity is perturbed by one ulp."""
    fx = load("ref_cube128_schedule")
    p = cube_problem(int(fx["n"]), jitter=float(fx["jitter"]), seed=int(fx["seed"]))
    steps = int(fx["steps"])
    dt = 0.5 * critical_time_step(p)
    m = E.Model(p, graph_steps=100)
    assert m.GetCriticalTimeStep() == float(fx["dt_crit"])
    m.begin(steps * dt, steps, 0)
    assert m.progress()[0] == 0
    m.advance(steps)
    g = m.state()
    ke, ie = m.GetEnergies()
    m.close()
    nodes, elems = fx["node_index"], fx["elem_index"]
    n = int(fx["n"])
    zl = np.rint(p.coords[:, 2] * n).astype(np.int64)
    ez = zl[p.conn].min(axis=1)
    got = {k: g[k][nodes] for k in ("u", "v", "a", "f_int")}
    got["F"], got["sigma"] = g["F"][elems], g["sigma"][elems]
    for k in ("u", "v"):
        sums = np.zeros((n + 1, 3))
        np.add.at(sums, zl, g[k])
        got[k + "_layer_sum"] = sums
    sums = np.zeros((n, 6))
    np.add.at(sums, ez, g["sigma"].mean(axis=1))
    got["sigma_layer_sum"] = sums
    report = {}
    for k in ("u", "v", "a", "f_int", "F", "sigma", "u_layer_sum", "v_layer_sum", "sigma_layer_sum"):
        e = rel(got[k], fx[k])
        env = float(fx["env_" + k])
        report[k] = (e, env)
        tol = TOL if k in ("u", "u_layer_sum") else max(TOL, 2.0 * env)
        assert e <= tol, f"{k}: relative error {e:.3e} > {tol:.3e} (reference's own 1-ulp sensitivity {env:.3e})"
    for k in ("u", "v", "a", "f_int", "F", "sigma"):
        e = abs(np.linalg.norm(g[k]) - float(fx[k + "_norm"])) / float(fx[k + "_norm"])
        report[k + "_norm"] = (e, float(fx["envelope_" + k]))
        assert e <= max(TOL, 2.0 * float(fx["envelope_" + k])), (k, e)
    for k, v in (("kinetic_energy", ke), ("internal_energy", ie)):
        e = abs(v - float(fx[k])) / abs(float(fx[k]))
        report[k] = (e, float(fx["env_" + k]))
        assert e <= max(TOL, 2.0 * float(fx["env_" + k])), (k, e)
    # the engine's own stress is accurate: within 1e-10 of the extended-precision
    # stress of its own displacement on the sampled elements
    e_exact = rel(got["sigma"], O.stress_exact(p, g["u"], np.asarray(elems, np.int32)))
    report["sigma_vs_extended_precision"] = (e_exact, 0.0)
    print("128^3 x 2000 steps, relative error (reference's 1-ulp sensitivity):",
          {k: f"{e:.2e} ({env:.2e})" for k, (e, env) in report.items()})
    assert e_exact < TOL


def test_derived_element_data():
    """Derived element output (element volume, volume-averaged stress and
    deformation gradient, Block::ComputeDerivedElementData): bitwise the oracle's restatement
    applied to the engine's own displacement and point stresses (same
    operations in the same order, no FMA contraction), and within the stress
    tolerance of the oracle run's derived output.  The FP32-mixed form's
    derived output is within 1e-3 of the FP64 form's."""
    p = cube_problem(8, jitter=0.2, seed=3)
    dt = 0.5 * critical_time_step(p)
    steps = 60
    ref = O.run_port(p, steps * dt, steps, 0)
    m = E.Model(p)
    m.begin(steps * dt, steps, 0)
    m.advance(steps)
    g = m.state()
    vol, avg, avg_F = m.ComputeDerivedElementData()
    v_own, a_own, f_own = O.derived_element_data(p, g["u"], g["sigma"], g["F"])
    assert np.array_equal(vol, v_own) and np.array_equal(avg, a_own) and np.array_equal(avg_F, f_own)
    v_ref, a_ref, f_ref = O.derived_element_data(p, ref["u"], ref["sigma"], ref["F"])
    floor, _ = sigma_floor(p, ref)
    assert rel(vol, v_ref) < TOL and rel(avg_F, f_ref) < TOL
    assert rel(avg, a_ref) < max(TOL, floor)
    m.close()
    m32 = E.Model(p, precision="fp32")
    m32.begin(steps * dt, steps, 0)
    m32.advance(steps)
    v32, a32, f32 = m32.ComputeDerivedElementData()
    assert rel(v32, vol) < 1e-6 and rel(a32, avg) < 1e-3 and rel(f32, avg_F) < 1e-6
    m32.close()
