"""Loading helpers for the committed golden fixtures (tests/golden/*.npz)."""
import os

import numpy as np

from nimblesm_gb300.mesh import BoundaryCondition, Material, Problem

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def gold_problem(fx) -> Problem:
    """The problem of a gold deck: mesh, node sets, the material of each
    element block, boundary conditions."""
    names = [str(s) for s in fx["ns_names"]]
    models = [str(m) for m in fx["block_models"]] if "block_models" in fx else ["neohookean"]
    params = fx["block_params"] if "block_params" in fx else [[float(fx["density"]), float(fx["bulk_modulus"]),
                                                                float(fx["shear_modulus"])]]
    mats = [Material(mo, *map(float, pr)) for mo, pr in zip(models, params)]
    p = Problem(coords=fx["coords"], conn=fx["conn"], node_sets={n: fx["ns:" + n] for n in names},
                density=mats[0].density, bulk_modulus=mats[0].bulk_modulus, shear_modulus=mats[0].shear_modulus,
                material_model=mats[0].model, bcs=[BoundaryCondition.parse(str(b)) for b in fx["bc_lines"]])
    if len(mats) > 1:
        p.blocks, p.elem_block = mats, np.asarray(fx["elem_block"], np.int32)
    return p


# The reference's regression decks with committed fixtures (test/dynamics/*).
GOLD_DECKS = ["single_elem_native_neohookean", "wave_in_bar", "rigid_body_motion", "simple_deformation_modes",
              "notched_plate_native_neohookean", "notched_plate_native_hypoelastic", "brick_with_fibers"]


def gold_checks(fx, t, st, vol, sig_avg, F_avg):
    """Every field the deck writes, at output time t + 1 of the gold file, at
    the deck's exodiff tolerances."""
    for field, key in (("displacement", "u"), ("velocity", "v"), ("acceleration", "a"),
                       ("internal_force", "f_int")):
        if "gold:" + field in fx:
            assert exodiff_ok(st[key], fx["gold:" + field][t + 1], fx["tol:" + field]), field
    if "gold:lumped_mass" in fx:
        assert exodiff_ok(st["mass"], fx["gold:lumped_mass"][t + 1], fx["tol:lumped_mass"])
    if "gold:F" in fx:
        assert exodiff_ok(st["F"], fx["gold:F"][t + 1], fx["tol:F"])
    if "gold:sigma" in fx:
        assert exodiff_ok(st["sigma"], fx["gold:sigma"][t + 1], fx["tol:sigma"])
    if "gold:volume" in fx:
        assert exodiff_ok(vol, fx["gold:volume"][t + 1], fx["tol:volume"])
    if "gold:F_avg" in fx:
        assert exodiff_ok(F_avg, fx["gold:F_avg"][t + 1], fx["tol:F_avg"])
    if "gold:sigma_avg" in fx:
        assert exodiff_ok(sig_avg, fx["gold:sigma_avg"][t + 1], fx["tol:sigma_avg"])


def uq_problem(fx):
    """Problem and UqSpec of the UQ fixture (one block, material_1)."""
    from nimblesm_gb300.uq import UqSpec
    w = str(fx["material_line"]).split()
    prm = {w[i]: float(w[i + 1]) for i in range(1, len(w) - 1, 2)}
    names = [str(s) for s in fx["ns_names"]]
    p = Problem(coords=fx["coords"], conn=fx["conn"], node_sets={n: fx["ns:" + n] for n in names},
                density=prm["density"], bulk_modulus=prm["bulk_modulus"], shear_modulus=prm["shear_modulus"],
                material_model=w[0], bcs=[BoundaryCondition.parse(str(b)) for b in fx["bc_lines"]])
    spec = UqSpec.parse([str(x) for x in fx["uq_parameters"]], str(fx["uq_samples"]), {"material_1": 0})
    return p, spec


def output_steps(num_steps, output_frequency):
    """1-based step counts after which the reference writes output
    (src/integrators/explicit_time_integrator.cc:192-194)."""
    return [s + 1 for s in range(num_steps)
            if output_frequency != 0 and (s % output_frequency == 0 or s == num_steps - 1)]


def exodiff_ok(ours, gold, abs_tol, rel=1e-6):
    """exodiff semantics of the reference's .exodiff files: a variable listed
    with "absolute X" passes when |a-b| <= X; any other variable falls back to
    the file default "relative 1.e-6 floor 0.0", |a-b| <= 1e-6 max(|a|,|b|).
    abs_tol broadcasts over the trailing axes (0 = not listed)."""
    abs_tol = np.broadcast_to(abs_tol, np.shape(ours))
    d = np.abs(ours - gold)
    rel_ok = d <= rel * np.maximum(np.abs(ours), np.abs(gold))
    return bool(np.all(np.where(abs_tol > 0, d <= abs_tol, rel_ok)))


def rel_err(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))
