"""Input decks, Genesis meshes and Exodus II output: run the reference's own
input files on the GPU engine and write output its exodiff files can check.

* read_deck: the reference's "key: value" input format
  (src/nimble_parser.cc:239-326): genesis input file, exodus output file,
  final time, number of load steps, output frequency, output fields,
  material parameters, element block, boundary condition.
* read_genesis: a Genesis / Exodus II mesh (NetCDF-3 classic): coordinates,
  hex8 element blocks in file order, node sets (named nodelist_<id> when the
  file gives no name, as src/nimble_genesis_mesh.cc:160-172 does).
* ExodusWriter: Exodus II results in the layout the reference writes
  (src/nimble_exodus_output.cc): nodal variables <field>_<component>,
  element variables per block, time_whole.
* run_deck: the whole run (python -m nimblesm_gb300.deck input.in).

NetCDF-3 is read and written with scipy.io (I/O only); all arithmetic runs
in the engine.
"""
from __future__ import annotations

import argparse
import os
import re
import sys

import numpy as np
import scipy.io

from .mesh import BoundaryCondition, Material, Problem

# Component labels of the reference's field lengths (src/nimble_data_utils.cc:158-207).
VECTOR = ("x", "y", "z")
FULL_TENSOR = ("xx", "yy", "zz", "xy", "yz", "zx", "yx", "zy", "xz")
SYMMETRIC_TENSOR = ("xx", "yy", "zz", "xy", "yz", "zx")
NODE_VECTOR_FIELDS = ("reference_coordinate", "displacement", "velocity", "acceleration", "internal_force",
                      "external_force")
LEN_NAME = 33


# ---------------------------------------------------------------------------
# input deck

class Deck:
    """The keys of an input deck that the explicit hex8 path uses."""

    def __init__(self, keys, materials, blocks, bcs, path=None):
        self.keys, self.materials, self.blocks, self.bcs, self.path = keys, materials, blocks, bcs, path

    @property
    def genesis_file(self):
        return self.keys["genesis input file"]

    @property
    def exodus_file(self):
        return self.keys.get("exodus output file")

    @property
    def final_time(self):
        return float(self.keys["final time"])

    @property
    def num_steps(self):
        return int(self.keys["number of load steps"])

    @property
    def output_frequency(self):
        return int(self.keys.get("output frequency", "1"))

    @property
    def initial_time(self):
        return float(self.keys.get("initial time", "0.0"))

    @property
    def output_fields(self):
        return self.keys.get("output fields", "").split()

    def problem(self, mesh) -> Problem:
        """The Problem of this deck on `mesh` (read_genesis): each mesh block's
        material from its "element block" line, the boundary conditions."""
        mats = []
        for bid in mesh["block_ids"]:
            name = f"block_{int(bid)}"
            if name not in self.blocks:
                raise ValueError(f"no element block line for {name}")
            prm = self.materials[self.blocks[name]]
            mats.append(Material(prm["model"], prm["density"], prm["bulk_modulus"], prm["shear_modulus"]))
        bcs = [BoundaryCondition.parse(b) for b in self.bcs]
        p = Problem(coords=mesh["coords"], conn=mesh["conn"], node_sets=dict(mesh["node_sets"]),
                    density=mats[0].density, bulk_modulus=mats[0].bulk_modulus,
                    shear_modulus=mats[0].shear_modulus, material_model=mats[0].model, bcs=bcs)
        if len(mats) > 1:
            p.blocks, p.elem_block = mats, np.asarray(mesh["elem_block"], np.int32)
        return p


def read_deck(path) -> Deck:
    """Parses an input deck: one "key: value" per line, '#' comments."""
    keys, materials, blocks, bcs = {}, {}, {}, []
    for raw in open(path):
        line = raw.split("#")[0].strip()
        if ":" not in line:
            continue
        k, val = (s.strip() for s in line.split(":", 1))
        if k == "material parameters":
            w = val.split()
            prm = {w[i]: float(w[i + 1]) for i in range(2, len(w) - 1, 2)}
            prm["model"] = w[1]
            materials[w[0]] = prm
        elif k == "element block":
            w = val.split()
            blocks[w[0]] = w[1]
        elif k == "boundary condition":
            bcs.append(val)
        else:
            keys[k] = val
    return Deck(keys, materials, blocks, bcs, path)


def write_deck(path, deck_keys, materials, blocks, bcs):
    """Writes an input deck in the reference's format (keys dict, materials
    {name: "model density .. .."}, blocks {block: material}, bc lines)."""
    with open(path, "w") as f:
        for k, v in deck_keys.items():
            f.write(f"{k}: {v}\n")
        for name, line in materials.items():
            f.write(f"material parameters: {name} {line}\n")
        for b, mname in blocks.items():
            f.write(f"element block: {b} {mname}\n")
        for bc in bcs:
            f.write(f"boundary condition: {bc}\n")


# ---------------------------------------------------------------------------
# Genesis / Exodus II (NetCDF-3)

def _names(var):
    return [b"".join(r).strip(b"\x00").decode() for r in var[:]]


def read_genesis(path):
    """Mesh (and any results) of a Genesis / Exodus II file: coords [N,3],
    0-based hex8 connectivity of all element blocks in file order (conn
    [E,8], elem_block [E], block_ids), node sets {name: ids}; with results,
    times and "nod:<name>" [T,N] / "elem:<name>" [T,E] arrays (element
    variables concatenated over the blocks)."""
    d = scipy.io.netcdf_file(path, "r", mmap=False)
    v = d.variables
    if "coordx" in v:
        coords = np.stack([v["coordx"][:], v["coordy"][:], v["coordz"][:]], axis=1).astype(np.float64)
    else:
        coords = np.asarray(v["coord"][:], np.float64).T.copy()
    nblk = len([k for k in v if re.fullmatch(r"connect\d+", k)])
    conns = []
    for b in range(nblk):
        c = v[f"connect{b + 1}"]
        et = getattr(c, "elem_type", b"HEX8")
        et = et.decode() if isinstance(et, bytes) else str(et)
        if not et.upper().startswith("HEX") or c.shape[1] != 8:
            raise ValueError(f"element block {b + 1}: only 8-node hexahedra are supported ({et})")
        conns.append(c[:].astype(np.int32) - 1)
    conn = np.concatenate(conns, axis=0) if conns else np.zeros((0, 8), np.int32)
    elem_block = np.concatenate([np.full(len(c), b, np.int32) for b, c in enumerate(conns)]) if conns else \
        np.zeros(0, np.int32)
    block_ids = v["eb_prop1"][:].astype(np.int32) if "eb_prop1" in v else np.arange(1, nblk + 1, dtype=np.int32)
    ns = {}
    if "ns_prop1" in v:
        names = _names(v["ns_names"]) if "ns_names" in v else [""] * len(v["ns_prop1"][:])
        for k, sid in enumerate(v["ns_prop1"][:]):
            nm = names[k] or f"nodelist_{int(sid)}"
            ns[nm] = v[f"node_ns{k + 1}"][:].astype(np.int32) - 1
    out = {"coords": coords, "conn": conn, "node_sets": ns, "elem_block": elem_block, "block_ids": block_ids}
    if "time_whole" in v:
        out["times"] = v["time_whole"][:].astype(np.float64)
        if "name_nod_var" in v:
            for k, nm in enumerate(_names(v["name_nod_var"])):
                out["nod:" + nm] = v[f"vals_nod_var{k + 1}"][:].astype(np.float64)
        if "name_elem_var" in v:
            for k, nm in enumerate(_names(v["name_elem_var"])):
                keys = [f"vals_elem_var{k + 1}eb{b + 1}" for b in range(nblk)]
                if all(key in v for key in keys):
                    out["elem:" + nm] = np.concatenate([v[key][:].astype(np.float64) for key in keys], axis=1)
    d.close()
    return out


def _chars(strings, n):
    a = np.zeros((len(strings), n), "S1")
    for i, s in enumerate(strings):
        b = s.encode()[: n - 1]
        a[i, : len(b)] = np.frombuffer(b, dtype="S1")
    return a


class ExodusWriter:
    """Exodus II (NetCDF-3, 64-bit offsets) results file: the mesh, then one
    time plane per write() with the named nodal ([N]) and element ([E],
    split over the blocks) variables."""

    def __init__(self, path, mesh, node_vars, elem_vars, title="NimbleSM GB300"):
        self.f = f = scipy.io.netcdf_file(path, "w", version=2)
        N, E = mesh["coords"].shape[0], mesh["conn"].shape[0]
        eb = np.asarray(mesh["elem_block"], np.int32)
        nblk = len(mesh["block_ids"])
        self.block_slices = [np.flatnonzero(eb == b) for b in range(nblk)]
        f.title = title
        f.api_version = np.float32(5.22)
        f.version = np.float32(5.22)
        f.floating_point_word_size = np.int32(8)
        f.file_size = np.int32(1)
        f.createDimension("time_step", None)  # the record dimension comes first in this writer
        f.createDimension("len_string", LEN_NAME)
        f.createDimension("len_line", 81)
        f.createDimension("four", 4)
        f.createDimension("len_name", LEN_NAME)
        f.createDimension("num_dim", 3)
        f.createDimension("num_nodes", N)
        f.createDimension("num_elem", E)
        f.createDimension("num_el_blk", nblk)
        f.createVariable("time_whole", "d", ("time_step",))
        for k, c in enumerate(("coordx", "coordy", "coordz")):
            f.createVariable(c, "d", ("num_nodes",))[:] = mesh["coords"][:, k]
        f.createVariable("coor_names", "c", ("num_dim", "len_name"))[:] = _chars(["x", "y", "z"], LEN_NAME)
        f.createVariable("eb_status", "i", ("num_el_blk",))[:] = np.ones(nblk, np.int32)
        prop = f.createVariable("eb_prop1", "i", ("num_el_blk",))
        prop.name = "ID"
        prop[:] = np.asarray(mesh["block_ids"], np.int32)
        f.createVariable("eb_names", "c", ("num_el_blk", "len_name"))[:] = _chars(
            [f"block_{int(b)}" for b in mesh["block_ids"]], LEN_NAME)
        for b, idx in enumerate(self.block_slices):
            f.createDimension(f"num_el_in_blk{b + 1}", len(idx))
            f.createDimension(f"num_nod_per_el{b + 1}", 8)
            c = f.createVariable(f"connect{b + 1}", "i", (f"num_el_in_blk{b + 1}", f"num_nod_per_el{b + 1}"))
            c.elem_type = "HEX8"
            c[:] = np.asarray(mesh["conn"], np.int32)[idx] + 1
        ns = list(mesh["node_sets"].items())
        if ns:
            f.createDimension("num_node_sets", len(ns))
            f.createVariable("ns_status", "i", ("num_node_sets",))[:] = np.ones(len(ns), np.int32)
            p = f.createVariable("ns_prop1", "i", ("num_node_sets",))
            p.name = "ID"
            p[:] = np.arange(1, len(ns) + 1, dtype=np.int32)
            f.createVariable("ns_names", "c", ("num_node_sets", "len_name"))[:] = _chars([n for n, _ in ns], LEN_NAME)
            for k, (_, ids) in enumerate(ns):
                f.createDimension(f"num_nod_ns{k + 1}", len(ids))
                f.createVariable(f"node_ns{k + 1}", "i", (f"num_nod_ns{k + 1}",))[:] = np.asarray(ids, np.int32) + 1
        self.node_vars, self.elem_vars = list(node_vars), list(elem_vars)
        if self.node_vars:
            f.createDimension("num_nod_var", len(self.node_vars))
            f.createVariable("name_nod_var", "c", ("num_nod_var", "len_name"))[:] = _chars(self.node_vars, LEN_NAME)
            for k in range(len(self.node_vars)):
                f.createVariable(f"vals_nod_var{k + 1}", "d", ("time_step", "num_nodes"))
        if self.elem_vars:
            f.createDimension("num_elem_var", len(self.elem_vars))
            f.createVariable("name_elem_var", "c", ("num_elem_var", "len_name"))[:] = _chars(self.elem_vars,
                                                                                              LEN_NAME)
            f.createVariable("elem_var_tab", "i", ("num_el_blk", "num_elem_var"))[:] = np.ones(
                (nblk, len(self.elem_vars)), np.int32)
            for k in range(len(self.elem_vars)):
                for b in range(nblk):
                    f.createVariable(f"vals_elem_var{k + 1}eb{b + 1}", "d", ("time_step", f"num_el_in_blk{b + 1}"))
        self.t = 0

    def write(self, time, node_values: dict, elem_values: dict):
        f, t = self.f, self.t
        f.variables["time_whole"][t] = time
        for k, nm in enumerate(self.node_vars):
            f.variables[f"vals_nod_var{k + 1}"][t, :] = node_values[nm]
        for k, nm in enumerate(self.elem_vars):
            vals = np.asarray(elem_values[nm])
            for b, idx in enumerate(self.block_slices):
                f.variables[f"vals_elem_var{k + 1}eb{b + 1}"][t, :] = vals[idx]
        self.t += 1

    def close(self):
        self.f.close()


def write_genesis(path, mesh):
    """A Genesis mesh file (Exodus II without results)."""
    ExodusWriter(path, mesh, [], []).close()


# ---------------------------------------------------------------------------
# the run

def _output_vars(fields):
    """Exodus variable names of the deck's output fields, nodal and element."""
    node, elem = [], []
    for fld in fields:
        m = re.fullmatch(r"ipt(\d\d)_(deformation_gradient|stress)", fld)
        if fld in NODE_VECTOR_FIELDS:
            node += [f"{fld}_{c}" for c in VECTOR]
        elif fld == "lumped_mass":
            node.append(fld)
        elif fld == "volume":
            elem.append(fld)
        elif fld in ("deformation_gradient", "stress"):
            comps = FULL_TENSOR if fld == "deformation_gradient" else SYMMETRIC_TENSOR
            elem += [f"{fld}_{c}" for c in comps]
        elif m:
            comps = FULL_TENSOR if m.group(2) == "deformation_gradient" else SYMMETRIC_TENSOR
            elem += [f"{fld}_{c}" for c in comps]
        else:
            raise ValueError(f"output field {fld!r} is not produced by this path")
    return node, elem


def _state_values(model, problem, fields):
    """The output values of the model's current state, by Exodus name."""
    nv, ev = {}, {}
    need_ip = any(f.startswith("ipt") for f in fields)
    need_derived = any(f in ("volume", "deformation_gradient", "stress") for f in fields)
    for fld in fields:
        if fld in NODE_VECTOR_FIELDS:
            arr = model.GetVectorNodeData(fld)
            for k, c in enumerate(VECTOR):
                nv[f"{fld}_{c}"] = arr[:, k]
        elif fld == "lumped_mass":
            nv[fld] = model.ComputeLumpedMass()
    if need_ip:
        F, S = model.GetIntegrationPointData()
    if need_derived:
        vol, s_avg, F_avg = model.ComputeDerivedElementData()
    for fld in fields:
        m = re.fullmatch(r"ipt(\d\d)_(deformation_gradient|stress)", fld)
        if fld == "volume":
            ev[fld] = vol
        elif fld == "deformation_gradient":
            for k, c in enumerate(FULL_TENSOR):
                ev[f"{fld}_{c}"] = F_avg[:, k]
        elif fld == "stress":
            for k, c in enumerate(SYMMETRIC_TENSOR):
                ev[f"{fld}_{c}"] = s_avg[:, k]
        elif m:
            ip = int(m.group(1)) - 1
            src, comps = (F, FULL_TENSOR) if m.group(2) == "deformation_gradient" else (S, SYMMETRIC_TENSOR)
            for k, c in enumerate(comps):
                ev[f"{fld}_{c}"] = src[:, ip, k]
    return nv, ev


def output_steps(num_steps, output_frequency):
    """1-based step counts after which the reference writes output
    (src/integrators/explicit_time_integrator.cc:192-194)."""
    return [s + 1 for s in range(num_steps)
            if output_frequency != 0 and (s % output_frequency == 0 or s == num_steps - 1)]


def run_deck(deck_path, output_path=None, precision="fp64", device=0):
    """Runs an input deck on the GPU engine and writes its Exodus output (the
    initial state and every output step, as the reference does); returns the
    output path."""
    from . import engine as E
    deck = read_deck(deck_path)
    base = os.path.dirname(os.path.abspath(deck_path))
    mesh = read_genesis(os.path.join(base, deck.genesis_file))
    problem = deck.problem(mesh)
    out = output_path or os.path.join(base, deck.exodus_file or os.path.splitext(deck_path)[0] + ".e")
    node_vars, elem_vars = _output_vars(deck.output_fields)
    model = E.Model(problem, precision=precision, device=device)
    try:
        model.begin(deck.final_time, deck.num_steps, deck.output_frequency, initial_time=deck.initial_time)
        writer = ExodusWriter(out, mesh, node_vars, elem_vars)
        try:
            nv, ev = _state_values(model, problem, deck.output_fields)
            writer.write(deck.initial_time, nv, ev)
            done = 0
            for s_end in output_steps(deck.num_steps, deck.output_frequency):
                model.advance(s_end - done)
                done = s_end
                nv, ev = _state_values(model, problem, deck.output_fields)
                writer.write(model.progress()[1], nv, ev)
        finally:
            writer.close()
    finally:
        model.close()
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description="Run a NimbleSM input deck (explicit, hex8) on the GPU engine.")
    ap.add_argument("deck")
    ap.add_argument("--output", default=None)
    ap.add_argument("--precision", choices=("fp64", "fp32"), default="fp64")
    ap.add_argument("--device", type=int, default=0)
    args = ap.parse_args(argv)
    print(run_deck(args.deck, args.output, args.precision, args.device))
    return 0


if __name__ == "__main__":
    sys.exit(main())
