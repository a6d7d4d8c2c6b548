"""Generates the golden fixtures in tests/golden/ (run in a container that has
the NimbleSM sources; the fixtures are committed so the tests need neither the
sources nor the reference build).

Two kinds of fixture:
  * gold_*.npz -- the reference's own regression gold files
    (test/dynamics/**/.gold.e, NetCDF-3, read with scipy), with the mesh they
    were made from (.g), the deck's material and boundary conditions (.in) and
    the per-variable exodiff tolerances (.exodiff).
  * ref_*.npz  -- outputs of the reference itself (oracle/_ref, NimbleSM's host
    sources compiled from where they lie) on seeded synthetic inputs.

Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import re
import sys

import numpy as np
import scipy.io

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from nimblesm_gb300.mesh import (CORNER_SIGNS, BoundaryCondition, Problem, cube_problem,  # noqa: E402
                                 critical_time_step)
from nimblesm_gb300.deck import read_deck as parse_deck  # noqa: E402
from nimblesm_gb300.deck import read_genesis  # noqa: E402
from oracle import oracle as O  # noqa: E402

REF = O.REF_ROOT  # the reference checkout (NIMBLESM_REFERENCE)


def read_exodus(path):
    """Mesh and results of an Exodus II (NetCDF-3) file (the engine's own
    reader, nimblesm_gb300.deck.read_genesis)."""
    return read_genesis(path)


def read_deck(path):
    """(materials {name: params}, blocks {block: material}, bc lines, other
    keys) of an input deck (the engine's own parser, nimblesm_gb300.deck)."""
    d = parse_deck(path)
    return d.materials, d.blocks, d.bcs, d.keys


def read_exodiff(path):
    """Per-variable absolute tolerances of an exodiff command file."""
    tol = {}
    for line in open(path):
        m = re.match(r"\s+(\w+)\s+absolute\s+([0-9.eE+-]+)", line)
        if m:
            tol[m.group(1)] = float(m.group(2))
    return tol


_VEC = ("x", "y", "z")
# Reference component order -> Exodus component names (src/nimble_data_utils.cc:158-207).
_FULL = ("xx", "yy", "zz", "xy", "yz", "zx", "yx", "zy", "xz")
_SYM = ("xx", "yy", "zz", "xy", "yz", "zx")


def gold_fixture(name, deck_dir, deck, genesis, gold, exodiff):
    base = os.path.join(REF, "test", "dynamics", deck_dir)
    mesh = read_exodus(os.path.join(base, genesis))
    res = read_exodus(os.path.join(base, gold))
    mats, blocks, bc_lines, keys = read_deck(os.path.join(base, deck))
    # the material of each mesh block, in the mesh's block order
    block_mats = [mats[blocks[f"block_{int(bid)}"]] for bid in mesh["block_ids"]]
    params = block_mats[0]
    tol = read_exodiff(os.path.join(base, exodiff))
    assert np.array_equal(mesh["coords"], res["coords"]), "gold file nodes are in mesh order"
    T = len(res["times"])
    N, E = mesh["coords"].shape[0], mesh["conn"].shape[0]
    fx = {
        "coords": mesh["coords"], "conn": mesh["conn"], "times": res["times"],
        "ns_names": np.array(list(mesh["node_sets"].keys())), "material_model": params["model"],
        "density": params["density"], "bulk_modulus": params["bulk_modulus"],
        "shear_modulus": params["shear_modulus"], "bc_lines": np.array(bc_lines),
        "elem_block": mesh["elem_block"], "block_ids": mesh["block_ids"],
        "output_fields": keys.get("output fields", ""),
        "block_models": np.array([bm["model"] for bm in block_mats]),
        "block_params": np.array([[bm["density"], bm["bulk_modulus"], bm["shear_modulus"]] for bm in block_mats]),
        "final_time": float(keys["final time"]), "num_steps": int(keys["number of load steps"]),
        "output_frequency": int(keys.get("output frequency", "1")),
    }
    for nm, ids in mesh["node_sets"].items():
        fx["ns:" + nm] = ids
    for field in ("displacement", "velocity", "acceleration", "internal_force"):
        if "nod:" + field + "_x" in res:
            fx["gold:" + field] = np.stack([res[f"nod:{field}_{c}"] for c in _VEC], axis=2)  # [T,N,3]
            fx["tol:" + field] = np.array([tol.get(f"{field}_{c}", 0.0) for c in _VEC])
    if "nod:lumped_mass" in res:
        fx["gold:lumped_mass"], fx["tol:lumped_mass"] = res["nod:lumped_mass"], tol.get("lumped_mass", 0.0)
    # per-point fields (ipt01..ipt08) where the deck writes them
    for key, comps, shape in (("deformation_gradient", _FULL, 9), ("stress", _SYM, 6)):
        if "elem:ipt01_" + key + "_xx" not in res:
            continue
        G, tG = np.zeros((T, E, 8, shape)), np.zeros((8, shape))
        for ip in range(8):
            for c, nm in enumerate(comps):
                k = f"ipt{ip + 1:02d}_{key}_{nm}"
                G[:, :, ip, c] = res["elem:" + k]
                tG[ip, c] = tol.get(k, 0.0)
        tag = "F" if key == "deformation_gradient" else "sigma"
        fx["gold:" + tag], fx["tol:" + tag] = G, tG
    # element fields without a point prefix are the volume averages
    # (Block::ComputeDerivedElementData); "volume" is the element volume
    for key, comps, tag in (("deformation_gradient", _FULL, "F_avg"), ("stress", _SYM, "sigma_avg")):
        if "elem:" + key + "_xx" in res:
            fx["gold:" + tag] = np.stack([res[f"elem:{key}_{c}"] for c in comps], axis=2)  # [T,E,k]
            fx["tol:" + tag] = np.array([tol.get(f"{key}_{c}", 0.0) for c in comps])
    if "elem:volume" in res:
        fx["gold:volume"], fx["tol:volume"] = res["elem:volume"], tol.get("volume", 0.0)
    np.savez_compressed(os.path.join(HERE, f"gold_{name}.npz"), **fx)
    print("wrote", name, {k: np.shape(v) for k, v in fx.items() if k.startswith("gold")})


def problem_from_fixture(fx) -> Problem:
    from tests.goldens import gold_problem
    return gold_problem(fx)


def ref_cube_fixture(name, n, jitter, seed, steps, output_frequency, sample_elems=None):
    p = cube_problem(n, jitter=jitter, seed=seed)
    dt = 0.5 * critical_time_step(p)
    final_time = steps * dt
    r = O.run_ref(p, final_time, steps, output_frequency)
    fx = {"n": n, "jitter": jitter, "seed": seed, "steps": steps, "output_frequency": output_frequency,
          "final_time": final_time, "dt_crit": r["dt_crit"]}
    for k in ("u", "v", "a", "f_int", "mass"):
        fx[k] = r[k]
    if sample_elems is None:
        fx["F"], fx["sigma"] = r["F"], r["sigma"]
    else:
        rng = np.random.default_rng(12345)
        idx = np.sort(rng.choice(p.num_elem, sample_elems, replace=False))
        fx["elem_index"] = idx
        fx["F"], fx["sigma"] = r["F"][idx], r["sigma"][idx]
        fx["F_norm"] = np.linalg.norm(r["F"])
        fx["sigma_norm"] = np.linalg.norm(r["sigma"])
        fx["sigma_elem"] = r["sigma"].mean(axis=1)  # volume-weighting aside, the element mean
    # The reference's own sensitivity: the same run with the initial velocity
    # perturbed by one ulp (relative 2^-52, seeded signs).  Two correct FP64
    # codes cannot be expected to agree more closely than this.
    q = cube_problem(n, jitter=jitter, seed=seed)
    rng = np.random.default_rng(77)
    q.v_init = q.v_init * (1.0 + rng.choice([-1.0, 1.0], size=q.v_init.shape) * 2.0 ** -52)
    rq = O.run_ref(q, final_time, steps, output_frequency)
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    fx["envelope_u"], fx["envelope_v"] = rel(rq["u"], r["u"]), rel(rq["v"], r["v"])
    fx["envelope_sigma"] = rel(rq["sigma"], r["sigma"])
    fx["envelope_sigma_elem"] = rel(rq["sigma"].mean(axis=1), r["sigma"].mean(axis=1))
    fx["sigma_elem_norm"] = np.linalg.norm(r["sigma"].mean(axis=1))
    np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **fx)
    print("wrote", name, r["loop_seconds"], "s", {k: fx[k] for k in fx if str(k).startswith("envelope")})


def ref_envelope_fixture(name, n, jitter, seed, steps):
    """Only the reference's own sensitivity on a long schedule (the state is
    too large to commit; the tests recompute it with the oracle): the run and
    the run with the initial velocity perturbed by one ulp (relative 2^-52,
    seeded signs, as in ref_cube_fixture), compared after the last step."""
    p = cube_problem(n, jitter=jitter, seed=seed)
    dt = 0.5 * critical_time_step(p)
    r = O.run_ref(p, steps * dt, steps, 0)
    q = cube_problem(n, jitter=jitter, seed=seed)
    rng = np.random.default_rng(77)
    q.v_init = q.v_init * (1.0 + rng.choice([-1.0, 1.0], size=q.v_init.shape) * 2.0 ** -52)
    rq = O.run_ref(q, steps * dt, steps, 0)
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    fx = {"n": n, "jitter": jitter, "seed": seed, "steps": steps, "dt_crit": r["dt_crit"],
          "envelope_u": rel(rq["u"], r["u"]), "envelope_v": rel(rq["v"], r["v"]),
          "envelope_sigma": rel(rq["sigma"], r["sigma"])}
    np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **fx)
    print("wrote", name, {k: fx[k] for k in fx if str(k).startswith("envelope")})


def ref_schedule_fixture(name, n, jitter, seed, steps, threads=8, node_sample=10_000, elem_sample=2_048):
    """The jittered n^3 cube over its whole schedule (Δt = 0.5 Δt_crit,
    `steps` steps), too large to commit whole, as seeded subsets plus
    whole-field figures:

      * u, v, a, f_int at `node_sample` seeded nodes; F and σ of every point of
        `elem_sample` seeded elements;
      * whole-field 2-norms of u, v, a, f_int, F and σ, per-z-layer sums of u and
        v (129 layers for n = 128: every node enters one) and of the element-mean
        σ (every element enters one), kinetic and internal energy;
      * the reference's own sensitivity: the same run with the initial velocity
        perturbed by one ulp (relative 2^-52, seeded signs, as in
        ref_cube_fixture), compared on the whole fields and on each stored
        subset and aggregate (`env_*`).

    The runs use the C restatement on `threads` host threads.  Its assembly
    order is the reference's serial order at any thread count, and it is
    bitwise the reference's own code on every committed fixture; on this mesh
    that is checked again here: the reference (oracle/_ref) and the restatement
    are run for 2 steps of the same schedule and must agree bit for bit."""
    p = cube_problem(n, jitter=jitter, seed=seed)
    dt = 0.5 * critical_time_step(p)
    final_time = steps * dt
    # the restatement is the reference on this mesh: 2 steps of Δt, both codes
    rs = O.run_ref(p, 2 * dt, 2, 0)
    ps = O.run_port(p, 2 * dt, 2, 0, threads=threads)
    for k in ("u", "v", "a", "f_int", "F", "sigma", "mass"):
        assert np.array_equal(ps[k], rs[k]), f"restatement differs from the reference in {k} at {n}^3"
    assert ps["dt_crit"] == rs["dt_crit"]
    dt_crit = rs["dt_crit"]
    del ps, rs
    print("restatement == reference after 2 steps at", n)

    def run(problem):
        pr = O.PortRun(problem, threads=threads)
        pr.begin(final_time, steps, 0)
        secs = pr.advance(steps)
        st = pr.state()
        print("  run", steps, "steps", secs, "s")
        return st

    r = run(p)
    q = cube_problem(n, jitter=jitter, seed=seed)
    rng = np.random.default_rng(77)
    q.v_init = q.v_init * (1.0 + rng.choice([-1.0, 1.0], size=q.v_init.shape) * 2.0 ** -52)
    rq = run(q)

    rng = np.random.default_rng(20261204)
    nodes = np.sort(rng.choice(p.num_nodes, node_sample, replace=False))
    elems = np.sort(rng.choice(p.num_elem, elem_sample, replace=False))
    zl = np.rint(p.coords[:, 2] * n).astype(np.int64)          # boundary planes stay planar
    ez = zl[p.conn].min(axis=1)                                 # element layer: its lowest node plane

    def aggregates(st):
        out = {}
        for k in ("u", "v", "a", "f_int"):
            out[k] = st[k][nodes]
            out[k + "_norm"] = np.linalg.norm(st[k])
        out["F"], out["sigma"] = st["F"][elems], st["sigma"][elems]
        out["F_norm"], out["sigma_norm"] = np.linalg.norm(st["F"]), np.linalg.norm(st["sigma"])
        for k in ("u", "v"):
            s = np.zeros((n + 1, 3))
            np.add.at(s, zl, st[k])
            out[k + "_layer_sum"] = s
        s = np.zeros((n, 6))
        np.add.at(s, ez, st["sigma"].mean(axis=1))
        out["sigma_layer_sum"] = s
        out["kinetic_energy"], out["internal_energy"] = st["kinetic_energy"], st["internal_energy"]
        return out

    a, b = aggregates(r), aggregates(rq)
    rel = lambda x, y: float(np.linalg.norm(np.asarray(x) - np.asarray(y)) / np.linalg.norm(y))
    fx = {"n": n, "jitter": jitter, "seed": seed, "steps": steps, "final_time": final_time,
          "dt_crit": dt_crit,
          "node_index": nodes, "elem_index": elems, **a}
    for k in ("u", "v", "a", "f_int", "F", "sigma"):
        fx["envelope_" + k] = rel(rq[k], r[k])          # whole field
        fx["env_" + k] = rel(b[k], a[k])                # the stored subset
    for k in ("u_layer_sum", "v_layer_sum", "sigma_layer_sum", "kinetic_energy", "internal_energy"):
        fx["env_" + k] = rel(b[k], a[k])
    np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **fx)
    print("wrote", name, {k: fx[k] for k in fx if str(k).startswith("env")})


def ref_derived_fixture(name="cube4_jitter"):
    """Derived element output of the reference (element volume and
    volume-averaged stress, HexElement::ComputeVolumeAverage through
    nimref_volume_average) on the final state of the ref_<name> fixture, with
    the current coordinates formed as Block::ComputeDerivedElementData forms
    them (reference coordinates + displacement, src/nimble_block.cc:477-483)."""
    fx = np.load(os.path.join(HERE, f"ref_{name}.npz"))
    p = cube_problem(int(fx["n"]), jitter=float(fx["jitter"]), seed=int(fx["seed"]))
    vol, avg, avg_F = np.zeros(p.num_elem), np.zeros((p.num_elem, 6)), np.zeros((p.num_elem, 9))
    for e in range(p.num_elem):
        ids = p.conn[e]
        x = p.coords[ids] + fx["u"][ids]
        vol[e], avg[e] = O.volume_average(x, fx["sigma"][e], which="ref")
        _, avg_F[e] = O.volume_average(x, fx["F"][e], which="ref")
    np.savez_compressed(os.path.join(HERE, f"ref_derived_{name}.npz"), volume=vol, stress=avg,
                        deformation_gradient=avg_F)
    print("wrote derived", name)


def ref_uq_fixture(name="uq_wave", keep_every=10):
    """The reference's UQ regression deck (test/uq/uq_wave: nominal, 2 exact and
    5 approximate trajectories, 10,000 steps; its gold file is not in the
    repository) run by the reference's own UQ mode (nimble_uq::ModelData
    through the harness): every keep_every-th output step of every
    trajectory, with the deck's mesh, materials, conditions and UQ input."""
    import tempfile
    from nimblesm_gb300.uq import UqSpec
    base = os.path.join(REF, "test", "uq", name)
    deck = parse_deck(os.path.join(base, f"{name}.in"))
    mesh = read_genesis(os.path.join(base, deck.genesis_file))
    p = deck.problem(mesh)
    uq_lines = [ln.split(":", 1)[1].strip() for ln in open(os.path.join(base, f"{name}.in"))
                if ln.split(":", 1)[0].strip() == "uq parameters"]
    samples = open(os.path.join(base, deck.keys["uq model"].split()[1])).read()
    mat_block = {deck.blocks[f"block_{int(b)}"]: i for i, b in enumerate(mesh["block_ids"])}
    spec = UqSpec.parse(uq_lines, samples, mat_block)
    with tempfile.TemporaryDirectory() as wd:
        r = O.run_ref_uq(p, spec, deck.final_time, deck.num_steps, deck.output_frequency, workdir=wd)
    out_steps = [s + 1 for s in range(deck.num_steps)
                 if deck.output_frequency != 0 and (s % deck.output_frequency == 0 or s == deck.num_steps - 1)]
    keep = list(range(0, len(out_steps), keep_every))
    if keep[-1] != len(out_steps) - 1:
        keep.append(len(out_steps) - 1)
    fx = {"coords": mesh["coords"], "conn": mesh["conn"], "ns_names": np.array(list(mesh["node_sets"])),
          "bc_lines": np.array(deck.bcs), "material_line": p.material_line(), "final_time": deck.final_time,
          "num_steps": deck.num_steps, "output_frequency": deck.output_frequency,
          "uq_parameters": np.array(uq_lines), "uq_samples": samples, "out_steps": np.array(out_steps)[keep]}
    for nm, ids in mesh["node_sets"].items():
        fx["ns:" + nm] = ids
    for k, v in r.items():
        fx[k] = v[keep]
    np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **fx)
    print("wrote UQ", name, fx["out_steps"])


def ref_points_fixture():
    """Stress and single-element known answers from the reference."""
    rng = np.random.default_rng(2024)
    K, G = 160e9, 79.3e9
    Fs = []
    for scale in (1e-6, 1e-4, 1e-3, 1e-2, 5e-2, 0.2):
        for _ in range(16):
            H = rng.normal(0.0, scale, size=(3, 3))
            M = np.eye(3) + H
            # reference storage order xx,yy,zz,xy,yz,zx,yx,zy,xz
            Fs.append([M[0, 0], M[1, 1], M[2, 2], M[0, 1], M[1, 2], M[2, 0], M[1, 0], M[2, 1], M[0, 2]])
    Fs.append([1.0, 1.0, 1.0, 0, 0, 0, 0, 0, 0])  # identity: the eigen solver's degenerate branch
    Fs = np.array(Fs)
    sig = O.stress(Fs, K, G, which="ref")
    X0 = CORNER_SIGNS.astype(np.float64)
    Xs, Us, Fe, Se, fe = [], [], [], [], []
    for k in range(24):
        h = 10.0 ** rng.uniform(-3, 0)
        X = 0.5 * h * X0 + rng.uniform(-0.15 * h, 0.15 * h, size=(8, 3)) + rng.uniform(-1, 1, size=3)
        U = rng.normal(0.0, h * 10.0 ** rng.uniform(-5, -1.5), size=(8, 3))
        F, S, f = O.element(X, U, K, G, which="ref")
        Xs.append(X), Us.append(U), Fe.append(F), Se.append(S), fe.append(f)
    np.savez_compressed(os.path.join(HERE, "ref_points.npz"), K=K, G=G, F=Fs, sigma=sig, elem_X=np.array(Xs),
                        elem_u=np.array(Us), elem_F=np.array(Fe), elem_sigma=np.array(Se), elem_f=np.array(fe))
    print("wrote points", Fs.shape)


GOLD_DECKS = (
    ("single_elem_native_neohookean", "single_elem_complex_displacement", "single_elem_native_neohookean.in",
     "single_elem.g", "single_elem_native_neohookean.gold.e", "single_elem_native_neohookean.exodiff"),
    ("wave_in_bar", "wave_in_bar", "wave_in_bar.in", "wave_in_bar.g", "wave_in_bar.gold.e", "wave_in_bar.exodiff"),
    ("rigid_body_motion", "rigid_body_motion", "rigid_body_motion.in", "rigid_body_motion.g",
     "rigid_body_motion.gold.e", "rigid_body_motion.exodiff"),
    ("simple_deformation_modes", "simple_deformation_modes", "simple_deformation_modes.in",
     "simple_deformation_modes.g", "simple_deformation_modes.gold.e", "simple_deformation_modes.exodiff"),
    ("notched_plate_native_neohookean", "notched_plate_native_neohookean", "notched_plate_native_neohookean.in",
     "notched_plate_native_neohookean.g", "notched_plate_native_neohookean.gold.e",
     "notched_plate_native_neohookean.exodiff"),
    ("notched_plate_native_hypoelastic", "notched_plate_native_hypoelastic", "notched_plate_native_hypoelastic.in",
     "notched_plate_native_hypoelastic.g", "notched_plate_native_hypoelastic.gold.e",
     "notched_plate_native_hypoelastic.exodiff"),
    ("brick_with_fibers", "brick_with_fibers", "brick_with_fibers.in", "brick_with_fibers.g",
     "brick_with_fibers.gold.e", "brick_with_fibers.exodiff"),
)


def _derived_ref(p, u, F, sigma):
    """The reference's derived element output of one state."""
    E = p.num_elem
    vol, avg_s, avg_F = np.zeros(E), np.zeros((E, 6)), np.zeros((E, 9))
    for e in range(E):
        ids = p.conn[e]
        x = p.coords[ids] + u[ids]
        vol[e], avg_s[e] = O.volume_average(x, sigma[e], which="ref")
        _, avg_F[e] = O.volume_average(x, F[e], which="ref")
    return vol, avg_s, avg_F


def ref_gold_rerun():
    """The reference itself on the gold decks, every output time, bitwise,
    with its derived element output (volume, volume-averaged F and sigma)."""
    for name, *_ in GOLD_DECKS:
        fx = dict(np.load(os.path.join(HERE, f"gold_{name}.npz")))
        p = problem_from_fixture(fx)
        steps, of = int(fx["num_steps"]), int(fx["output_frequency"])
        states = O.run_ref_outputs(p, float(fx["final_time"]), steps, of)
        out_steps = [s + 1 for s in range(steps) if of != 0 and (s % of == 0 or s == steps - 1)]
        assert len(states) == len(out_steps)
        res = {"out_steps": np.array(out_steps), "mass": states[0]["mass"]}
        for k in ("u", "v", "a", "f_int", "F", "sigma"):
            res[k] = np.array([st[k] for st in states])
        derived = [_derived_ref(p, st["u"], st["F"], st["sigma"]) for st in states]
        res["volume"] = np.array([d[0] for d in derived])
        res["sigma_avg"] = np.array([d[1] for d in derived])
        res["F_avg"] = np.array([d[2] for d in derived])
        np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **res)
        print("wrote ref rerun", name, out_steps)


# Boundary-condition expressions (written for these tests; they cover the
# reference grammar: precedence, associativity, unary minus, exponents,
# functions, constants, conditions) and points (x, y, z, t).
BC_EXPRESSIONS = [
    "1.5e-3 * t", "2.0*x - 0.5*y + z/4", "x^2 + y^3 - z^-2", "sqrt(x*x + y*y)", "exp(-t*1e5) * sin(2*pi*x)",
    "t < 5e-6 ? 1e3*t : 5e-3", "(x > 0.5 & y <= 0.5) | z == 0.25 ? 1 : -1",
    "abs(x - 0.5) + floor(y*3) + ceil(z*2.5) + round(x*7.3)", "log(1 + x) + log10(10 + y) + cbrt(z + 2)",
    "atan(x) + asin(y/2) + acos(z/3)", "erf(x) + erfc(y) + tan(z/2)", "10 % 4 + 1", "x % 0.3 + 1", "2^3^2",
    "-x - -y", "-(x + y) * -z", "e^x - tau*y + pi", "3*x/4*y/2", "x - y - z + t", "1e-3*sin(t*1.0e6)*x",
    "TAU*X + Sin(Y)", "((x))+(((y)))", "x*-2 + 1", "2e-3*x", "1.e2*y", ".5*z", "x ^ 0.5", "x^(1/3)",
    "!(x > 0.5) ? x : y", "x > 0.2 ^ y > 0.3 ? 1 : 0", "t >= 2e-6 ? (t <= 8e-6 ? 2*t : 3*t) : t/2",
    "8/2/2", "1 - 2 - 3", "x*y*z*t*1e6", "  ( x + 1 ) * ( y - 1 )  ", "exp(log(x+1)/2)", "-2^2", "(-2)^2",
    "x^2.5", "100*t - 0.001", "5 - -3", "sin(x)^2 + cos(x)^2", "1e-3 - x", "0.25*(1 - x)*(1 + y)",
]
# refused by the reference: an unknown name, an exponent's sign taken for an
# operator, an unclosed call, an unknown function, two operands
BC_EXPRESSIONS_BAD = ["a+1", "2*1e+5", "x - 1e-3", "sin(x", "foo(x)", "x y"]
BC_POINTS = [(0.0, 0.0, 0.25, 0.0), (0.3, 0.7, 0.25, 1.0e-6), (0.75, 0.2, 0.5, 5.0e-6), (1.0, 1.0, 1.0, 9.5e-6),
             (0.5, 0.5, 0.75, 2.0e-6), (0.125, 0.875, 0.375, 8.0e-6)]


def ref_bc_expressions_fixture():
    """The reference parser's values of BC_EXPRESSIONS at BC_POINTS, and the
    expressions it refuses."""
    vals = np.array([[O.ref_eval_expression(e, *pt) for pt in BC_POINTS] for e in BC_EXPRESSIONS])
    for e in BC_EXPRESSIONS_BAD:
        try:
            O.ref_eval_expression(e, *BC_POINTS[1])
            raise RuntimeError("the reference parsed " + e)
        except ValueError:
            pass
    np.savez_compressed(os.path.join(HERE, "ref_bc_expressions.npz"), expressions=np.array(BC_EXPRESSIONS),
                        bad=np.array(BC_EXPRESSIONS_BAD), points=np.array(BC_POINTS), values=vals)
    print("wrote bc expressions", vals.shape)


# A cube driven by expression conditions only (no initial velocity field):
# time- and position-dependent prescribed displacement and velocity on the
# bottom face, initial and prescribed velocity on the top face.
BC_EXPRESSION_RUN = [
    'initial_velocity nodelist_2 x "25.0*x*y"',
    'initial_velocity nodelist_2 z "-40.0*(1 + 0.5*sin(pi*x))"',
    'prescribed_displacement nodelist_1 z "1.0e-4*sin(t*2.0e5)*(1 + x*y)"',
    'prescribed_displacement nodelist_1 x "0.0"',
    'prescribed_velocity nodelist_1 y "t < 4.0e-6 ? 2.5e5*t*(1 - x) : 1.0 - x"',
    'prescribed_velocity nodelist_2 y "x > 0.5 ? 0.5 : -0.5"',
]


def bc_expression_problem(n=6, seed=3):
    p = cube_problem(n, jitter=0.2, seed=seed)
    p.v_init = None
    p.bcs = [BoundaryCondition.parse(line) for line in BC_EXPRESSION_RUN]
    return p


def ref_bc_expression_run_fixture(steps=300, output_frequency=50):
    p = bc_expression_problem()
    dt = 0.5 * critical_time_step(p)
    outs = O.run_ref_outputs(p, steps * dt, steps, output_frequency)
    fx = {"steps": steps, "output_frequency": output_frequency, "final_time": steps * dt,
          "bc_lines": np.array(BC_EXPRESSION_RUN)}
    for k in ("u", "v", "a", "f_int"):
        fx[k] = np.stack([o[k] for o in outs])
    fx["F"], fx["sigma"] = outs[-1]["F"], outs[-1]["sigma"]  # the last output's point data
    np.savez_compressed(os.path.join(HERE, "ref_bc_expression_cube6.npz"), **fx)
    print("wrote bc expression run", fx["u"].shape)


GENERATORS = {"bc_expressions": lambda: (ref_bc_expressions_fixture(), ref_bc_expression_run_fixture()),
              "cube128_schedule": lambda: ref_schedule_fixture("cube128_schedule", 128, 0.2, 0, 2000)}


if __name__ == "__main__":
    O.build(ref=True)
    if len(sys.argv) > 1:  # only the named fixture groups
        for name in sys.argv[1:]:
            GENERATORS[name]()
        sys.exit(0)
    for deck in GOLD_DECKS:
        gold_fixture(*deck)
    ref_points_fixture()
    ref_cube_fixture("cube4_jitter", 4, 0.2, 7, 20, 0)
    ref_cube_fixture("cube16_cfg0", 16, 0.0, 0, 500, 500, sample_elems=64)
    ref_gold_rerun()
    ref_envelope_fixture("cube40_schedule", 40, 0.2, 0, 2000)
    ref_derived_fixture("cube4_jitter")
    ref_uq_fixture("uq_wave")
    ref_schedule_fixture("cube128_schedule", 128, 0.2, 0, 2000)
