"""The reference's UQ configuration (src/uq/nimble_uq.cc): uncertain material
parameters with their ranges ("uq parameters: material_<b> <name> <range>
..."), exact samples and approximate samples with the coefficients of the
linear force closure (the samples file read by UqModel::ReadSamples,
src/uq/nimble_uq.cc:145-218).

Sample s of parameter i is xi[s][i]; its value is p0 + range * xi
(UqModel::ScaleParameters, src/uq/nimble_uq.cc:220-244), p0 the nominal
value of the block's material.  Exact samples evaluate the element forces
with their own bulk and shear moduli; an approximate sample's force is
c0 f_nominal + sum_k c_k f_exact_k (UqModel::ApplyClosure, :327-345).
"""
from __future__ import annotations

import numpy as np


class UqSpec:
    """params: [(block index, parameter name, range)] in the reference's
    parameter order (materials in name order, each line's parameters in
    order); exact_xi [n_exact, P]; approx_xi [n_approx, P]; coefficients
    [n_approx, n_exact + 1], the nominal's first."""

    def __init__(self, params, exact_xi, approx_xi, coefficients):
        self.params = [(int(b), str(n), float(r)) for b, n, r in params]
        P = len(self.params)
        self.exact_xi = np.asarray(exact_xi, np.float64).reshape(-1, P)
        self.approx_xi = np.asarray(approx_xi, np.float64).reshape(-1, P)
        self.coefficients = np.asarray(coefficients, np.float64).reshape(len(self.approx_xi), len(self.exact_xi) + 1)
        for _, n, _ in self.params:
            if n not in ("bulk_modulus", "shear_modulus", "density"):
                raise ValueError(f"unknown uncertain parameter {n!r}")

    @property
    def num_exact(self):
        return len(self.exact_xi)

    @property
    def num_approx(self):
        return len(self.approx_xi)

    def sample_parameters(self, problem):
        """{name: [n_exact + n_approx, blocks]} of every sample (exact first),
        scaled as the reference scales them."""
        mats = problem.materials()
        xi = np.concatenate([self.exact_xi, self.approx_xi], axis=0)
        out = {}
        for name in ("bulk_modulus", "shear_modulus", "density"):
            out[name] = np.array([[getattr(m, name) for m in mats] for _ in range(len(xi))], np.float64)
        for i, (b, name, rng) in enumerate(self.params):
            for s in range(len(xi)):
                p0 = out[name][s, b]
                out[name][s, b] = p0 + rng * xi[s, i]
        return out

    def parameter_lines(self):
        """The "uq parameters" lines, one per material, material_<b+1>."""
        lines = {}
        for b, name, rng in self.params:
            lines.setdefault(b, []).append(f"{name} {rng!r}")
        return [f"material_{b + 1} " + " ".join(v) for b, v in sorted(lines.items())]

    def samples_text(self):
        """The samples file: "<n_exact> <n_approx>", the exact samples' xi, then
        "<xi ...> : <coefficients ...>" per approximate sample."""
        rows = [f"{self.num_exact} {self.num_approx}"]
        rows += [" ".join(repr(float(x)) for x in r) for r in self.exact_xi]
        rows += [" ".join(repr(float(x)) for x in r) + " : " + " ".join(repr(float(c)) for c in cf)
                 for r, cf in zip(self.approx_xi, self.coefficients)]
        return "\n".join(rows) + "\n"

    @classmethod
    def parse(cls, parameter_lines, samples_text, material_blocks):
        """From "uq parameters" lines (material name first) and the samples
        file text; material_blocks maps material names to block indices."""
        params = []
        for line in sorted(parameter_lines, key=lambda l: l.split()[0]):
            w = line.split()
            b = material_blocks[w[0]]
            for i in range(1, len(w) - 1, 2):
                params.append((b, w[i], float(w[i + 1])))
        rows = [r for r in samples_text.splitlines() if r.strip()]
        ne, na = (int(x) for x in rows[0].split()[:2])
        exact = [[float(x) for x in rows[1 + k].split()] for k in range(ne)]
        approx, coef = [], []
        for k in range(na):
            lhs, rhs = rows[1 + ne + k].split(":")
            approx.append([float(x) for x in lhs.split()])
            coef.append([float(x) for x in rhs.split()])
        return cls(params, exact, approx, coef)
