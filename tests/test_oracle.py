"""The CPU oracle (oracle/nsm_oracle.c) pinned against the reference: its gold
files at the exodiff tolerances, and the reference's own outputs bit for bit."""
import numpy as np
import pytest

from nimblesm_gb300.mesh import cube_problem, critical_time_step
from oracle import oracle as O
from tests.goldens import GOLD_DECKS, exodiff_ok, gold_checks, gold_problem, load, output_steps, uq_problem


@pytest.fixture(scope="module", autouse=True)
def _build():
    O.build(ref=False)


def test_points_match_reference_bitwise():
    fx = load("ref_points")
    s = O.stress(fx["F"], float(fx["K"]), float(fx["G"]))
    assert np.array_equal(s, fx["sigma"])
    for k in range(fx["elem_X"].shape[0]):
        F, S, f = O.element(fx["elem_X"][k], fx["elem_u"][k], float(fx["K"]), float(fx["G"]))
        assert np.array_equal(F, fx["elem_F"][k])
        assert np.array_equal(S, fx["elem_sigma"][k])
        assert np.array_equal(f, fx["elem_f"][k])


def test_identity_stress_is_zero():
    F = np.array([[1.0, 1.0, 1.0, 0, 0, 0, 0, 0, 0]])
    assert np.all(O.stress(F, 160e9, 79.3e9) == 0.0)


@pytest.mark.parametrize("name", ["cube4_jitter", "cube16_cfg0"])
def test_cube_runs_match_reference_bitwise(name):
    fx = load("ref_" + name)
    p = cube_problem(int(fx["n"]), jitter=float(fx["jitter"]), seed=int(fx["seed"]))
    r = O.run_port(p, float(fx["final_time"]), int(fx["steps"]), int(fx["output_frequency"]), threads=4)
    assert r["dt_crit"] == float(fx["dt_crit"])
    for k in ("u", "v", "a", "f_int", "mass"):
        assert np.array_equal(r[k], fx[k]), k
    idx = fx.get("elem_index")
    F, S = (r["F"], r["sigma"]) if idx is None else (r["F"][idx], r["sigma"][idx])
    assert np.array_equal(F, fx["F"]) and np.array_equal(S, fx["sigma"])
    if idx is not None:
        assert np.linalg.norm(r["F"]) == float(fx["F_norm"])
        assert np.linalg.norm(r["sigma"]) == float(fx["sigma_norm"])


def test_derived_element_data_matches_reference_bitwise():
    """Element volume, volume-averaged stress and deformation gradient
    (Block::ComputeDerivedElementData)
    on the reference's final state of the 4^3 run, against the reference's own
    HexElement::ComputeVolumeAverage."""
    fx = load("ref_cube4_jitter")
    dx = load("ref_derived_cube4_jitter")
    p = cube_problem(int(fx["n"]), jitter=float(fx["jitter"]), seed=int(fx["seed"]))
    vol, avg, avg_F = O.derived_element_data(p, fx["u"], fx["sigma"], fx["F"])
    assert np.array_equal(vol, dx["volume"])
    assert np.array_equal(avg, dx["stress"])
    assert np.array_equal(avg_F, dx["deformation_gradient"])
    assert abs(vol.sum() - 1.0) < 1e-3  # the unit cube, slightly deformed


def test_uq_closure_matches_reference_bitwise():
    """The reference's UQ regression deck (uq_wave: nominal, 2 exact and 5
    approximate trajectories with the linear force closure, 10,000 steps):
    the oracle's restatement against the reference's own UQ mode, every
    trajectory, bit for bit."""
    fx = load("ref_uq_wave")
    p, spec = uq_problem(fx)
    steps, of = int(fx["num_steps"]), int(fx["output_frequency"])
    r = O.run_port_uq(p, spec, float(fx["final_time"]), steps, of)
    idx = [output_steps(steps, of).index(int(s)) for s in fx["out_steps"]]
    assert spec.num_exact == 2 and spec.num_approx == 5
    for k in ("u", "v", "f", "su", "sv", "sf"):
        assert np.array_equal(r[k][idx], fx[k]), k


def test_numpy_critical_time_step_matches_oracle():
    p = cube_problem(6, jitter=0.2, seed=11)
    keep = []
    assert critical_time_step(p) == O.PortRun(p).dt_crit


@pytest.mark.parametrize("name", GOLD_DECKS)
def test_gold_files(name):
    """The reference's regression decks (neo-Hookean and elastic materials,
    one and two element blocks) against their gold files, at the exodiff
    tolerances, at every output time, including the derived element output;
    and bit for bit against the reference run here on the same deck."""
    fx = load("gold_" + name)
    rf = load("ref_" + name)
    p = gold_problem(fx)
    steps, of = int(fx["num_steps"]), int(fx["output_frequency"])
    run = O.PortRun(p)
    run.begin(float(fx["final_time"]), steps, of)
    done = 0
    for t, s_end in enumerate(output_steps(steps, of)):
        run.advance(s_end - done)
        done = s_end
        st = run.state()
        assert np.isclose(st["time"], fx["times"][t + 1], rtol=1e-12, atol=0)
        vol, sig_avg, F_avg = O.derived_element_data(p, st["u"], st["sigma"], st["F"])
        gold_checks(fx, t, st, vol, sig_avg, F_avg)
        # the reference itself, same deck, same machine arithmetic
        for key in ("u", "v", "a", "f_int", "F", "sigma"):
            assert np.array_equal(st[key], rf[key][t]), key
        assert np.array_equal(st["mass"], rf["mass"])
        assert np.array_equal(vol, rf["volume"][t]) and np.array_equal(sig_avg, rf["sigma_avg"][t])
        assert np.array_equal(F_avg, rf["F_avg"][t])


def test_thread_count_does_not_change_results():
    p = cube_problem(5, jitter=0.2, seed=5)
    dt = 0.5 * critical_time_step(p)
    a = O.run_port(p, 30 * dt, 30, 0, threads=1)
    b = O.run_port(p, 30 * dt, 30, 0, threads=3)
    for k in ("u", "v", "a", "f_int", "F", "sigma"):
        assert np.array_equal(a[k], b[k])


def test_energy_is_bounded_to_integration_error():
    """KE + IE oscillates (central difference conserves a modified energy, and
    fixed nodes carry half a step of reaction velocity between output steps)
    but does not drift."""
    p = cube_problem(6, jitter=0.2, seed=1)
    dt = 0.5 * critical_time_step(p)
    run = O.PortRun(p)
    run.begin(400 * dt, 400, 0)
    run.advance(1)
    e0 = run.state()
    tot0 = e0["kinetic_energy"] + e0["internal_energy"]
    for _ in range(8):
        run.advance(50)
        e = run.state()
        assert e["internal_energy"] > 0
        assert abs(e["kinetic_energy"] + e["internal_energy"] - tot0) / tot0 < 5e-2


@pytest.mark.skipif(not O.reference_available(), reason="reference not built here")
def test_live_reference_bitwise_random_case():
    p = cube_problem(3, jitter=0.2, seed=99)
    dt = 0.5 * critical_time_step(p)
    a = O.run_port(p, 17 * dt, 17, 5)
    b = O.run_ref(p, 17 * dt, 17, 5)
    for k in ("u", "v", "a", "f_int", "mass", "F", "sigma"):
        assert np.array_equal(a[k], b[k]), k


def test_closure_base_is_the_material_to_second_order():
    """The learned closure's analytic base (oracle/mlp_oracle.py base_part,
    restated in nimblesm_gb300/csrc/mlp_common.cuh) is the reference's
    neo-Hookean stress to second order in H: the remainder falls as |H|^3
    (relative to the stress, as |H|^2), while the linear part's falls as |H|."""
    from oracle import mlp_oracle as M
    K, G = 160e9, 79.3e9
    slot = [0, 3, 8, 6, 1, 4, 5, 7, 2]
    rng = np.random.default_rng(0)
    errs = []
    for s in (1e-2, 1e-3):
        H = rng.normal(0, s, size=(2000, 9))
        F = np.zeros((H.shape[0], 9))
        for q in range(9):
            F[:, slot[q]] = H[:, q] + (1.0 if q % 4 == 0 else 0.0)
        exact = O.stress(F, K, G) / G
        e_b = np.linalg.norm(M.base_part(H, K / G) - exact) / np.linalg.norm(exact)
        e_l = np.linalg.norm(M.linear_part(H, K / G) - exact) / np.linalg.norm(exact)
        errs.append((e_b, e_l))
    (b2, l2), (b3, l3) = errs
    assert 50 < b2 / b3 < 200      # second-order remainder relative to the stress: |H|^2
    assert 5 < l2 / l3 < 20         # the linear part's: |H|
    assert b3 < 1e-5 and l3 > 1e-3
