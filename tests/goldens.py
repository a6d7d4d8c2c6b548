"""Loading helpers for the committed golden fixtures (tests/golden/*.npz)."""
import os

import numpy as np

from nimblesm_gb300.mesh import BoundaryCondition, Problem

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def gold_problem(fx) -> Problem:
    names = [str(s) for s in fx["ns_names"]]
    return Problem(coords=fx["coords"], conn=fx["conn"], node_sets={n: fx["ns:" + n] for n in names},
                   density=float(fx["density"]), bulk_modulus=float(fx["bulk_modulus"]),
                   shear_modulus=float(fx["shear_modulus"]),
                   bcs=[BoundaryCondition.parse(str(b)) for b in fx["bc_lines"]])


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
