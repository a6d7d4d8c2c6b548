"""Synthetic hex8 meshes and explicit-dynamics problem definitions.

A problem is what NimbleSM reads from a Genesis mesh plus an input deck
(src/nimble_genesis_mesh.cc:318-427, src/nimble_parser.cc:239-326): nodal
reference coordinates, 8-node connectivity in the reference corner order
(src/nimble_element.cc:113-120), named node sets, one neo-Hookean material
("neohookean density .. bulk_modulus .. shear_modulus ..",
src/nimble_material_factory_base.cc:62-98) and boundary-condition lines
("<kind> <nodeset> <x|y|z> <value>", src/nimble_boundary_condition.cc:65-144).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

BC_INITIAL_VELOCITY = 0
BC_PRESCRIBED_VELOCITY = 1
BC_PRESCRIBED_DISPLACEMENT = 2
# A traction line names a side set; the reference parses it and applies
# nothing (BoundaryConditionManager::ApplyTractionBC is an empty loop,
# src/nimble_boundary_condition_manager.h:230-247), and so does the engine:
# no node set carries its name, so the line drops out like any line whose
# node set is absent.
BC_PRESCRIBED_TRACTION = 3

_BC_KINDS = {
    "initial_velocity": BC_INITIAL_VELOCITY,
    "prescribed_velocity": BC_PRESCRIBED_VELOCITY,
    "prescribed_displacement": BC_PRESCRIBED_DISPLACEMENT,
    "prescribed_traction": BC_PRESCRIBED_TRACTION,
}
_COMPONENTS = {"x": 0, "y": 1, "z": 2}

# Corner signs of the reference's hex (src/nimble_element.cc:113-120).
CORNER_SIGNS = np.array(
    [[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
     [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], dtype=np.int64)


@dataclass
class BoundaryCondition:
    """One boundary-condition line of the input deck: a constant magnitude, or
    an expression f(x, y, z, t) of the node's reference coordinates and the
    time (the quoted form)."""
    kind: int
    node_set: str
    component: int
    value: float
    expression: str | None = None

    @staticmethod
    def parse(line: str) -> "BoundaryCondition":
        """Parses "<kind> <nodeset> <x|y|z> <value>" or "<kind> <nodeset>
        <x|y|z> "<expression>"" as BoundaryCondition::Initialize does
        (src/nimble_boundary_condition.cc:65-144): two quotes make the text
        between the first and the last an expression."""
        quotes = line.count('"')
        if quotes not in (0, 2):
            raise ValueError("illegal number of quotes in boundary condition: " + line)
        expression = None
        if quotes == 2:
            expression = line[line.index('"') + 1: line.rindex('"')]
            parts = line[: line.index('"')].split()
            if len(parts) != 3:
                raise ValueError("malformed boundary condition: " + line)
            kind, ns, comp = parts
            val = 0.0
        else:
            parts = line.split()
            if len(parts) != 4:
                raise ValueError("malformed boundary condition: " + line)
            kind, ns, comp, val = parts
        if kind not in _BC_KINDS:
            raise ValueError("unknown boundary condition type: " + kind)
        if comp.lower() not in _COMPONENTS:
            raise ValueError("unknown coordinate: " + comp)
        return BoundaryCondition(_BC_KINDS[kind], ns, _COMPONENTS[comp.lower()], float(val), expression)

    def line(self) -> str:
        kind = {v: k for k, v in _BC_KINDS.items()}[self.kind]
        if self.expression is not None:
            return f'{kind} {self.node_set} {"xyz"[self.component]} "{self.expression}"'
        return f"{kind} {self.node_set} {'xyz'[self.component]} {self.value!r}"


class Material:
    """One material line of an input deck: "<model> density .. bulk_modulus ..
    shear_modulus ..", model "neohookean" or "elastic"."""

    MODELS = {"neohookean": 0, "elastic": 1}

    def __init__(self, model: str, density: float, bulk_modulus: float, shear_modulus: float):
        if model not in self.MODELS:
            raise ValueError(f"unknown material model {model!r}")
        self.model, self.density = model, float(density)
        self.bulk_modulus, self.shear_modulus = float(bulk_modulus), float(shear_modulus)

    def line(self) -> str:
        return (f"{self.model} density {self.density!r} bulk_modulus {self.bulk_modulus!r} "
                f"shear_modulus {self.shear_modulus!r}")


@dataclass
class Problem:
    """An explicit-dynamics problem on hex8 elements: one block with the
    material (material_model, density, bulk_modulus, shear_modulus), or, with
    `blocks` and `elem_block`, several element blocks each with its own
    Material (elements ordered by block)."""
    coords: np.ndarray               # [N,3] float64
    conn: np.ndarray                 # [E,8] int32, 0-based
    node_sets: dict = field(default_factory=dict)   # name -> int32 array of node ids
    density: float = 7800.0
    bulk_modulus: float = 160e9
    shear_modulus: float = 79.3e9
    bcs: list = field(default_factory=list)         # [BoundaryCondition]
    v_init: np.ndarray | None = None  # [N,3] velocity written after the initial conditions
    material_model: str = "neohookean"  # "neohookean" | "elastic" (MaterialFactory names)
    blocks: list | None = None          # [Material] per element block
    elem_block: np.ndarray | None = None  # [E] block index, non-decreasing

    @property
    def num_nodes(self) -> int:
        return int(self.coords.shape[0])

    @property
    def num_elem(self) -> int:
        return int(self.conn.shape[0])

    def materials(self) -> list:
        """The materials of the blocks (one for a single-block problem)."""
        if self.blocks:
            return list(self.blocks)
        return [Material(self.material_model, self.density, self.bulk_modulus, self.shear_modulus)]

    def material_line(self) -> str:
        return self.materials()[0].line()

    def bc_arrays(self):
        """BCs flattened to (kind[], component[], value[], ptr[], nodes[]) in deck
        order; a BC whose node set is absent is dropped, as the reference does
        (src/nimble_boundary_condition_manager.cc:67-71)."""
        kinds, comps, vals, ptr, nodes = [], [], [], [0], []
        for bc in self.bcs:
            if bc.node_set not in self.node_sets or bc.kind == BC_PRESCRIBED_TRACTION:
                continue
            if bc.expression is not None:
                raise ValueError("constant boundary magnitudes only: " + bc.line())
            ids = np.asarray(self.node_sets[bc.node_set], dtype=np.int32)
            kinds.append(bc.kind)
            comps.append(bc.component)
            vals.append(bc.value)
            nodes.append(ids)
            ptr.append(ptr[-1] + len(ids))
        nodes = np.concatenate(nodes).astype(np.int32) if nodes else np.zeros(0, np.int32)
        return (np.asarray(kinds, np.int32), np.asarray(comps, np.int32),
                np.asarray(vals, np.float64), np.asarray(ptr, np.int32), nodes)


def cube_mesh(n: int, length: float = 1.0, jitter: float = 0.0, seed: int = 0):
    """n^3 hex8 cube [0,L]^3 with lexicographic node and element ids.

    Node (i,j,k) has id i + (n+1)(j + (n+1)k); element (i,j,k) has id
    i + n(j + nk) and corners in the reference order.  Interior nodes (on no
    face) are moved by i.i.d. U(-jitter*h, +jitter*h) per coordinate from a
    seeded generator; nodes on the faces stay put, so faces stay planar."""
    h = length / n
    g = np.arange(n + 1, dtype=np.float64) * h
    z, y, x = np.meshgrid(g, g, g, indexing="ij")
    coords = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        idx = np.arange(n + 1)
        interior = (idx > 0) & (idx < n)
        mask = (interior[None, None, :] & interior[None, :, None] & interior[:, None, None]).ravel()
        d = rng.uniform(-jitter * h, jitter * h, size=(int(mask.sum()), 3))
        coords[mask] += d
    ar = np.arange(n)
    k, j, i = (a.ravel() for a in np.meshgrid(ar, ar, ar, indexing="ij"))  # i fastest
    n1 = n + 1
    conn = np.empty((n ** 3, 8), dtype=np.int32)
    for c, (sx, sy, sz) in enumerate(CORNER_SIGNS):
        conn[:, c] = (i + (sx > 0)) + n1 * ((j + (sy > 0)) + n1 * (k + (sz > 0)))
    return coords, conn


def cube_problem(n: int, jitter: float = 0.0, seed: int = 0, density: float = 7800.0,
                 bulk_modulus: float = 160e9, shear_modulus: float = 79.3e9,
                 v_gradient: float = 10.0, v_noise: float = 0.1, length: float = 1.0) -> Problem:
    """The synthetic unit-cube workload: nodes on z=0 held by prescribed zero
    velocity in x, y, z; initial velocity v_z = v_gradient * z / L plus a
    seeded U(-v_noise, v_noise) per node and component."""
    coords, conn = cube_mesh(n, length, jitter, seed)
    n1 = n + 1
    bottom = np.arange(n1 * n1, dtype=np.int32)          # k = 0 plane
    top = np.arange(n * n1 * n1, n1 ** 3, dtype=np.int32)  # k = n plane
    rng = np.random.default_rng(seed + 1_000_003)
    v0 = rng.uniform(-v_noise, v_noise, size=coords.shape)
    v0[:, 2] += v_gradient * coords[:, 2] / length
    bcs = [BoundaryCondition(BC_PRESCRIBED_VELOCITY, "nodelist_1", c, 0.0) for c in range(3)]
    return Problem(coords=coords, conn=conn, node_sets={"nodelist_1": bottom, "nodelist_2": top},
                   density=density, bulk_modulus=bulk_modulus, shear_modulus=shear_modulus,
                   bcs=bcs, v_init=v0)


def characteristic_lengths(coords: np.ndarray, conn: np.ndarray) -> np.ndarray:
    """Per-element HexElement::ComputeCharacteristicLength
    (src/nimble_element.cc:221-260), vectorised: the smaller of the least
    node-pair distance and the least bounding-box extent (box maxima start at
    0 as in the reference)."""
    x = coords[conn]                                   # [E,8,3]
    d2 = np.full(conn.shape[0], np.inf)
    for a in range(8):
        for b in range(a + 1, 8):
            diff = x[:, a] - x[:, b]
            d2 = np.minimum(d2, (diff[:, 0] * diff[:, 0] + diff[:, 1] * diff[:, 1]) + diff[:, 2] * diff[:, 2])
    lo = x.min(axis=1)
    hi = np.maximum(x.max(axis=1), 0.0)
    box = (hi - lo).min(axis=1)
    return np.minimum(np.sqrt(d2), box)


def critical_time_step(problem: Problem) -> float:
    """BlockBase::ComputeCriticalTimeStep (src/nimble_block_base.cc:51-84):
    min over elements of L_e / sqrt(K / rho)."""
    c = np.sqrt(problem.bulk_modulus / problem.density)
    return float((characteristic_lengths(problem.coords, problem.conn) / c).min())


def uq_ensemble(num_samples: int = 512, n_min: int = 8, n_max: int = 48, seed: int = 0, jitter: float = 0.2,
                cov: float = 0.10, bulk_mean: float = 160e9, shear_mean: float = 79.3e9,
                density: float = 7800.0) -> list:
    """Uncertainty-quantification ensemble: sample g is a jittered cube with
    n_g^3 hexes, n_g ~ U{n_min..n_max}, and log-normal bulk and shear moduli
    (given means, coefficient of variation cov), the unit-cube boundary
    conditions and initial velocity of cube_problem.  All draws are seeded."""
    rng = np.random.default_rng(seed)
    sig = np.sqrt(np.log1p(cov * cov))
    ns = rng.integers(n_min, n_max + 1, size=num_samples)
    K = np.exp(np.log(bulk_mean) - 0.5 * sig * sig + sig * rng.standard_normal(num_samples))
    G = np.exp(np.log(shear_mean) - 0.5 * sig * sig + sig * rng.standard_normal(num_samples))
    return [cube_problem(int(ns[g]), jitter=jitter, seed=seed * 100003 + g, density=density,
                         bulk_modulus=float(K[g]), shear_modulus=float(G[g])) for g in range(num_samples)]

