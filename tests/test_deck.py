"""Input decks, Genesis meshes and Exodus output (nimblesm_gb300/deck.py):
round trips on the CPU, and the reference's regression decks run end to end
on the GPU engine (deck + Genesis file in, Exodus file out) against their gold
files at the decks' exodiff tolerances."""
import numpy as np
import pytest

from nimblesm_gb300 import deck as D
from nimblesm_gb300.mesh import cube_problem
from tests.goldens import GOLD_DECKS, exodiff_ok, load


def two_block_mesh():
    p = cube_problem(3, jitter=0.1, seed=1)
    eb = (np.arange(p.num_elem) >= 10).astype(np.int32)
    return {"coords": p.coords, "conn": p.conn, "elem_block": eb, "block_ids": np.array([1, 2], np.int32),
            "node_sets": dict(p.node_sets)}


def test_exodus_round_trip(tmp_path):
    mesh = two_block_mesh()
    N, E = mesh["coords"].shape[0], mesh["conn"].shape[0]
    rng = np.random.default_rng(0)
    w = D.ExodusWriter(str(tmp_path / "r.e"), mesh, ["displacement_x", "lumped_mass"], ["volume", "stress_xy"])
    vals = []
    for t in (0.0, 1.5e-6, 3.0e-6):
        nv = {"displacement_x": rng.normal(size=N), "lumped_mass": rng.uniform(size=N)}
        ev = {"volume": rng.uniform(size=E), "stress_xy": rng.normal(size=E)}
        w.write(t, nv, ev)
        vals.append((nv, ev))
    w.close()
    r = D.read_genesis(str(tmp_path / "r.e"))
    assert np.array_equal(r["coords"], mesh["coords"]) and np.array_equal(r["conn"], mesh["conn"])
    assert np.array_equal(r["elem_block"], mesh["elem_block"]) and list(r["block_ids"]) == [1, 2]
    assert set(r["node_sets"]) == set(mesh["node_sets"])
    for nm, ids in mesh["node_sets"].items():
        assert np.array_equal(r["node_sets"][nm], ids)
    assert np.array_equal(r["times"], [0.0, 1.5e-6, 3.0e-6])
    for t, (nv, ev) in enumerate(vals):
        for k, v in nv.items():
            assert np.array_equal(r["nod:" + k][t], v)
        for k, v in ev.items():
            assert np.array_equal(r["elem:" + k][t], v)


def test_deck_round_trip(tmp_path):
    mesh = two_block_mesh()
    D.write_genesis(str(tmp_path / "m.g"), mesh)
    D.write_deck(str(tmp_path / "d.in"),
                 {"genesis input file": "m.g", "exodus output file": "o.e", "final time": repr(2.0e-6),
                  "number of load steps": "150", "output frequency": "30", "output fields": "displacement stress"},
                 {"material_1": "neohookean density 7.8 bulk_modulus 1.6e12 shear_modulus 0.8e12",
                  "material_2": "elastic density 5.0 bulk_modulus 1.333e12 shear_modulus 0.1379e12"},
                 {"block_1": "material_1", "block_2": "material_2"},
                 ["initial_velocity nodelist_1 x 1000.0", "prescribed_velocity nodelist_2 y 0.0"])
    deck = D.read_deck(str(tmp_path / "d.in"))
    assert deck.final_time == 2.0e-6 and deck.num_steps == 150 and deck.output_frequency == 30
    assert deck.output_fields == ["displacement", "stress"]
    p = deck.problem(D.read_genesis(str(tmp_path / "m.g")))
    assert [m.model for m in p.blocks] == ["neohookean", "elastic"]
    assert p.blocks[1].shear_modulus == 0.1379e12 and np.array_equal(p.elem_block, mesh["elem_block"])
    assert [b.line() for b in p.bcs] == ["initial_velocity nodelist_1 x 1000.0", "prescribed_velocity nodelist_2 y 0.0"]
    node, elem = D._output_vars(["displacement", "lumped_mass", "volume", "stress", "ipt03_deformation_gradient"])
    assert node == ["displacement_x", "displacement_y", "displacement_z", "lumped_mass"]
    assert elem[:2] == ["volume", "stress_xx"] and elem[-1] == "ipt03_deformation_gradient_xz"


def _deck_from_fixture(fx, tmp_path):
    """Writes the gold deck's mesh (Genesis) and input deck from the fixture."""
    mesh = {"coords": fx["coords"], "conn": fx["conn"], "elem_block": fx["elem_block"],
            "block_ids": fx["block_ids"], "node_sets": {str(n): fx["ns:" + str(n)] for n in fx["ns_names"]}}
    D.write_genesis(str(tmp_path / "mesh.g"), mesh)
    mats, blocks = {}, {}
    for b, (model, prm) in enumerate(zip(fx["block_models"], fx["block_params"])):
        mats[f"material_{b + 1}"] = (f"{model} density {float(prm[0])!r} bulk_modulus {float(prm[1])!r} "
                                     f"shear_modulus {float(prm[2])!r}")
        blocks[f"block_{int(fx['block_ids'][b])}"] = f"material_{b + 1}"
    D.write_deck(str(tmp_path / "deck.in"),
                 {"genesis input file": "mesh.g", "exodus output file": "out.e",
                  "final time": repr(float(fx["final_time"])), "number of load steps": str(int(fx["num_steps"])),
                  "output frequency": str(int(fx["output_frequency"])), "output fields": str(fx["output_fields"])},
                 mats, blocks, [str(b) for b in fx["bc_lines"]])
    return str(tmp_path / "deck.in")


@pytest.mark.gpu
@pytest.mark.parametrize("name", GOLD_DECKS)
def test_run_deck_against_gold(name, tmp_path):
    from nimblesm_gb300 import build as B
    B.build()
    fx = load("gold_" + name)
    out = D.read_genesis(D.run_deck(_deck_from_fixture(fx, tmp_path)))
    T = len(fx["times"])
    assert np.allclose(out["times"], fx["times"], rtol=1e-12, atol=0)
    for field in ("displacement", "velocity", "acceleration", "internal_force"):
        if "gold:" + field in fx:
            ours = np.stack([out[f"nod:{field}_{c}"] for c in D.VECTOR], axis=2)
            for t in range(T):
                assert exodiff_ok(ours[t], fx["gold:" + field][t], fx["tol:" + field]), (field, t)
    if "gold:lumped_mass" in fx:
        for t in range(T):
            assert exodiff_ok(out["nod:lumped_mass"][t], fx["gold:lumped_mass"][t], fx["tol:lumped_mass"])
    per_point = (("F", "deformation_gradient", D.FULL_TENSOR), ("sigma", "stress", D.SYMMETRIC_TENSOR))
    for tag, key, comps in per_point:
        if "gold:" + tag in fx:
            ours = np.stack([np.stack([out[f"elem:ipt{p + 1:02d}_{key}_{c}"] for c in comps], axis=2)
                             for p in range(8)], axis=2)  # [T,E,8,k]
            for t in range(T):
                assert exodiff_ok(ours[t], fx["gold:" + tag][t], fx["tol:" + tag]), (tag, t)
        if "gold:" + tag + "_avg" in fx:
            ours = np.stack([out[f"elem:{key}_{c}"] for c in comps], axis=2)  # [T,E,k]
            for t in range(T):
                assert exodiff_ok(ours[t], fx["gold:" + tag + "_avg"][t], fx["tol:" + tag + "_avg"]), (tag, t)
    if "gold:volume" in fx:
        for t in range(T):
            assert exodiff_ok(out["elem:volume"][t], fx["gold:volume"][t], fx["tol:volume"]), t


def test_traction_lines_parse_and_drop_out():
    from nimblesm_gb300.mesh import BC_PRESCRIBED_TRACTION, BoundaryCondition
    b = BoundaryCondition.parse("prescribed_traction sideset_1 x 2.5e6")
    assert b.kind == BC_PRESCRIBED_TRACTION and b.line() == "prescribed_traction sideset_1 x 2500000.0"
    p = cube_problem(2)
    p.bcs = p.bcs + [BoundaryCondition.parse("prescribed_traction nodelist_1 x 1.0")]
    kinds = p.bc_arrays()[0]
    assert BC_PRESCRIBED_TRACTION not in kinds and len(kinds) == 3

