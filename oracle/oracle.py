"""ctypes bindings for the CPU oracles.  TEST INFRASTRUCTURE ONLY.

Two libraries, both built by oracle/Makefile:
  * _build/libnsm_oracle.so -- the plain-C restatement (nsm_oracle.c), built on
    every machine (it is the CPU baseline "port" where the reference is absent);
  * _ref/libnimble_ref.so   -- NimbleSM's own host sources plus ref_harness.cc,
    buildable only where the reference sources are present.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs import
this module, as the checker or as the timed CPU baseline.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libnsm_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libnimble_ref.so")
# The reference checkout whose sources oracle/Makefile compiles: the
# NIMBLESM_REFERENCE environment variable, else where this container mounts it.
# Where it is absent, only the C restatement is built.
REF_ROOT = os.environ.get("NIMBLESM_REFERENCE", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "src")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def _d(a):
    return None if a is None else a.ctypes.data_as(_dp)


def _i(a):
    return None if a is None else a.ctypes.data_as(_ip)


def build(ref: bool | None = None) -> None:
    """Builds the C restatement, and the reference library when its sources
    are present (or when ref=True)."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    if ref is None:
        ref = os.path.isdir(REF_SRC)
    if ref:
        subprocess.run(["make", "-s", "-j8", "-C", HERE, "ref", "REF=" + REF_SRC], check=True)


class _Model(C.Structure):
    _fields_ = [
        ("num_nodes", C.c_int), ("num_elem", C.c_int), ("coords", _dp), ("conn", _ip),
        ("density", C.c_double), ("bulk_modulus", C.c_double), ("shear_modulus", C.c_double),
        ("num_bcs", C.c_int), ("bc_kind", _ip), ("bc_component", _ip), ("bc_value", _dp),
        ("bc_ptr", _ip), ("bc_nodes", _ip),
        ("material_model", C.c_int), ("num_blocks", C.c_int), ("elem_block", _ip), ("block_model", _ip),
        ("block_density", _dp), ("block_bulk", _dp), ("block_shear", _dp),
    ]


class _Result(C.Structure):
    _fields_ = [
        ("u", _dp), ("v", _dp), ("a", _dp), ("f_int", _dp), ("F", _dp), ("sigma", _dp), ("mass", _dp),
        ("dt_crit", C.c_double), ("kinetic_energy", C.c_double), ("internal_energy", C.c_double),
        ("loop_seconds", C.c_double),
    ]


_port = None
_ref = None


def port():
    global _port
    if _port is None:
        if not os.path.exists(PORT_SO):
            build(ref=False)
        lib = C.CDLL(PORT_SO)
        lib.nsm_oracle_run.argtypes = [C.POINTER(_Model), C.c_double, C.c_int, C.c_int, _dp, C.c_int,
                                       C.POINTER(_Result)]
        lib.nsm_oracle_continue.argtypes = [C.POINTER(_Model), C.c_double, C.c_double, C.c_int, C.c_int,
                                            _dp, _dp, _dp, _dp]
        lib.nsm_oracle_element.argtypes = [_dp, _dp, C.c_double, C.c_double, _dp, _dp, _dp]
        lib.nsm_oracle_stress.argtypes = [C.c_int, _dp, C.c_double, C.c_double, _dp]
        lib.nsm_oracle_lumped_mass.argtypes = [C.POINTER(_Model), _dp]
        lib.nsm_oracle_critical_time_step.argtypes = [C.POINTER(_Model)]
        lib.nsm_oracle_critical_time_step.restype = C.c_double
        lib.nsm_oracle_energy_density.argtypes = [_dp, C.c_double, C.c_double]
        lib.nsm_oracle_energy_density.restype = C.c_double
        lib.nsm_oracle_shape_tables.argtypes = [_dp, _dp]
        lib.nsm_oracle_create.argtypes = [C.POINTER(_Model), C.c_int]
        lib.nsm_oracle_create.restype = C.c_void_p
        lib.nsm_oracle_destroy.argtypes = [C.c_void_p]
        lib.nsm_oracle_dt_crit.argtypes = [C.c_void_p]
        lib.nsm_oracle_dt_crit.restype = C.c_double
        lib.nsm_oracle_begin.argtypes = [C.c_void_p, C.c_double, C.c_int, C.c_int, _dp]
        lib.nsm_oracle_advance.argtypes = [C.c_void_p, C.c_int, _dp]
        lib.nsm_oracle_time.argtypes = [C.c_void_p]
        lib.nsm_oracle_time.restype = C.c_double
        lib.nsm_oracle_get_state.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        lib.nsm_oracle_set_state.argtypes = [C.c_void_p, _dp, _dp, _dp]
        lib.nsm_oracle_energies.argtypes = [C.c_void_p, _dp, _dp]
        lib.nsm_oracle_stress_exact.argtypes = [C.POINTER(_Model), _dp, C.c_int, _ip, _dp]
        lib.nsm_oracle_volume_average.argtypes = [_dp, C.c_int, _dp, _dp, _dp]
        lib.nsm_oracle_run_uq.argtypes = [C.POINTER(_Model), C.c_int, _dp, _dp, C.c_int, _dp, C.c_double, C.c_int,
                                          C.c_int, _dp, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _ip]
        lib.nsm_oracle_derived_element_data.argtypes = [C.POINTER(_Model), _dp, _dp, _dp, _dp, _dp, _dp]
        _port = lib
    return _port


REF_UQ_SO = os.path.join(HERE, "_ref", "libnimble_ref_uq.so")
_ref_uq = None


def ref_uq():
    """The reference built with its UQ mode (oracle/_ref/libnimble_ref_uq.so)."""
    global _ref_uq
    if _ref_uq is None:
        if not os.path.exists(REF_UQ_SO):
            raise RuntimeError("UQ reference library not built (oracle/_ref); needs the reference sources")
        lib = C.CDLL(REF_UQ_SO)
        lib.nimref_run_uq.argtypes = [C.c_int, _dp, C.c_int, _ip, C.c_int, _ip, C.c_char_p, C.c_int, _ip, _ip,
                                      C.c_char_p, C.c_char_p, C.c_double, C.c_int, C.c_int, _dp, C.c_char_p,
                                      C.c_char_p, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _ip]
        lib.nimref_last_error.restype = C.c_char_p
        _ref_uq = lib
    return _ref_uq


def reference_available() -> bool:
    return os.path.exists(REF_SO)


def ref():
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            raise RuntimeError("reference library not built (oracle/_ref); needs the reference sources")
        lib = C.CDLL(REF_SO)
        lib.nimref_run.argtypes = [C.c_int, _dp, C.c_int, _ip, C.c_int, _ip, _ip, C.c_char_p, C.c_char_p,
                                   C.c_char_p, C.c_double, C.c_int, C.c_int, _dp,
                                   _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        lib.nimref_run_blocks.argtypes = [C.c_int, _dp, C.c_int, _ip, C.c_int, _ip, C.c_char_p, C.c_int, _ip, _ip,
                                          C.c_char_p, C.c_char_p, C.c_double, C.c_int, C.c_int, _dp, C.c_int,
                                          _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _ip]
        lib.nimref_element.argtypes = [_dp, _dp, C.c_double, C.c_double, C.c_double, _dp, _dp, _dp]
        lib.nimref_stress.argtypes = [C.c_int, _dp, C.c_double, C.c_double, _dp]
        lib.nimref_volume_average.argtypes = [_dp, C.c_int, _dp, _dp, _dp]
        lib.nimref_eval_expression.argtypes = [C.c_char_p, C.c_double, C.c_double, C.c_double, C.c_double, _dp]
        lib.nimref_last_error.restype = C.c_char_p
        _ref = lib
    return _ref


def _model(problem, keep):
    kinds, comps, vals, ptr, nodes = problem.bc_arrays()
    coords = np.ascontiguousarray(problem.coords, dtype=np.float64)
    conn = np.ascontiguousarray(problem.conn, dtype=np.int32)
    mats = problem.materials()
    bm = np.array([mt.MODELS[mt.model] for mt in mats], np.int32)
    bd = np.array([mt.density for mt in mats])
    bk = np.array([mt.bulk_modulus for mt in mats])
    bs = np.array([mt.shear_modulus for mt in mats])
    eb = (np.ascontiguousarray(problem.elem_block, dtype=np.int32) if len(mats) > 1
          else np.zeros(problem.num_elem, np.int32))
    keep.extend([kinds, comps, vals, ptr, nodes, coords, conn, bm, bd, bk, bs, eb])
    m0 = mats[0]
    return _Model(problem.num_nodes, problem.num_elem, _d(coords), _i(conn), m0.density,
                  m0.bulk_modulus, m0.shear_modulus, len(kinds), _i(kinds), _i(comps), _d(vals),
                  _i(ptr), _i(nodes), int(bm[0]), len(mats), _i(eb), _i(bm), _d(bd), _d(bk), _d(bs))


def _outputs(problem, with_ip):
    N, E = problem.num_nodes, problem.num_elem
    out = {k: np.zeros((N, 3)) for k in ("u", "v", "a", "f_int")}
    out["mass"] = np.zeros(N)
    if with_ip:
        out["F"] = np.zeros((E, 8, 9))
        out["sigma"] = np.zeros((E, 8, 6))
    return out


def run_port(problem, final_time, num_steps, output_frequency=0, threads=1, with_ip=True):
    """Runs the C restatement; returns a dict of numpy arrays and scalars."""
    keep = []
    m = _model(problem, keep)
    out = _outputs(problem, with_ip)
    res = _Result(_d(out["u"]), _d(out["v"]), _d(out["a"]), _d(out["f_int"]), _d(out.get("F")),
                  _d(out.get("sigma")), _d(out["mass"]), 0.0, 0.0, 0.0, 0.0)
    v0 = None if problem.v_init is None else np.ascontiguousarray(problem.v_init, dtype=np.float64)
    rc = port().nsm_oracle_run(C.byref(m), float(final_time), int(num_steps), int(output_frequency),
                               _d(v0), int(threads), C.byref(res))
    if rc != 0:
        raise RuntimeError(f"oracle run failed ({rc}): non-positive Jacobian")
    out.update(dt_crit=res.dt_crit, kinetic_energy=res.kinetic_energy,
               internal_energy=res.internal_energy, loop_seconds=res.loop_seconds)
    return out


class PortRun:
    """Stateful run of the C restatement: begin(), advance(k), state()."""

    def __init__(self, problem, threads=1):
        self.problem = problem
        self._keep = []
        self._model = _model(problem, self._keep)
        self._h = port().nsm_oracle_create(C.byref(self._model), int(threads))
        if not self._h:
            raise MemoryError("oracle allocation failed")
        self.dt_crit = port().nsm_oracle_dt_crit(self._h)

    def begin(self, final_time, num_steps, output_frequency=0):
        v0 = None if self.problem.v_init is None else np.ascontiguousarray(self.problem.v_init, np.float64)
        self._keep.append(v0)
        port().nsm_oracle_begin(self._h, float(final_time), int(num_steps), int(output_frequency), _d(v0))

    def advance(self, k):
        secs = C.c_double(0.0)
        if port().nsm_oracle_advance(self._h, int(k), C.cast(C.pointer(secs), _dp)) != 0:
            raise RuntimeError("oracle step failed: non-positive Jacobian")
        return secs.value

    def state(self, with_ip=True):
        out = _outputs(self.problem, with_ip)
        port().nsm_oracle_get_state(self._h, _d(out["u"]), _d(out["v"]), _d(out["a"]), _d(out["f_int"]),
                                    _d(out.get("F")), _d(out.get("sigma")), _d(out["mass"]))
        out["time"] = port().nsm_oracle_time(self._h)
        ke, ie = C.c_double(0.0), C.c_double(0.0)
        port().nsm_oracle_energies(self._h, C.cast(C.pointer(ke), _dp), C.cast(C.pointer(ie), _dp))
        out["kinetic_energy"], out["internal_energy"] = ke.value, ie.value
        return out

    def set_state(self, u=None, v=None, a=None):
        arrs = [None if x is None else np.ascontiguousarray(x, np.float64) for x in (u, v, a)]
        port().nsm_oracle_set_state(self._h, *[_d(x) for x in arrs])

    def __del__(self):
        if getattr(self, "_h", None):
            port().nsm_oracle_destroy(self._h)
            self._h = None


def continue_port(problem, u, v, a, t0, dt, num_steps, threads):
    """Advances (u, v, a) in place by num_steps with a fixed step; returns the
    wall seconds of the step loop."""
    keep = []
    m = _model(problem, keep)
    secs = C.c_double(0.0)
    rc = port().nsm_oracle_continue(C.byref(m), float(t0), float(dt), int(num_steps), int(threads),
                                    _d(u), _d(v), _d(a), C.cast(C.pointer(secs), _dp))
    if rc != 0:
        raise RuntimeError(f"oracle continue failed ({rc})")
    return secs.value


def ref_eval_expression(text, x, y, z, t):
    """A boundary-condition expression evaluated by the reference's parser
    (oracle/_ref): its value, or a ValueError with the reference's message."""
    lib = ref()
    v = C.c_double(0.0)
    if lib.nimref_eval_expression(text.encode(), float(x), float(y), float(z), float(t), C.byref(v)) != 0:
        raise ValueError(lib.nimref_last_error().decode())
    return v.value


def run_ref_outputs(problem, final_time, num_steps, output_frequency=0, with_ip=True, lib=None):
    """Runs the reference itself (oracle/_ref) and returns its state after
    every output step of the schedule (after the last step only when
    output_frequency is 0): a list of dicts like run_port's, F and sigma being
    the element data the reference stored in that step.  `lib`: another build
    of the same harness (the adapter test's), default the reference's."""
    lib = lib or ref()
    names = list(problem.node_sets.keys())
    ns_ptr = np.zeros(len(names) + 1, np.int32)
    parts = []
    for s, nm in enumerate(names):
        ids = np.asarray(problem.node_sets[nm], np.int32)
        parts.append(ids)
        ns_ptr[s + 1] = ns_ptr[s] + len(ids)
    ns_nodes = np.concatenate(parts).astype(np.int32) if parts else np.zeros(0, np.int32)
    bcs = "\n".join(bc.line() for bc in problem.bcs)
    N, E = problem.num_nodes, problem.num_elem
    of = int(output_frequency)
    T = 1 if of == 0 else (int(num_steps) + of - 1) // of + 1
    out = {k: np.zeros((T, N, 3)) for k in ("u", "v", "a", "f_int")}
    if with_ip:
        out["F"], out["sigma"] = np.zeros((T, E, 8, 9)), np.zeros((T, E, 8, 6))
    mass = np.zeros(N)
    coords = np.ascontiguousarray(problem.coords, dtype=np.float64)
    conn = np.ascontiguousarray(problem.conn, dtype=np.int32)
    mats = problem.materials()
    eb = np.ascontiguousarray(problem.elem_block, dtype=np.int32) if len(mats) > 1 else None
    v0 = None if problem.v_init is None else np.ascontiguousarray(problem.v_init, dtype=np.float64)
    dt, secs, n = C.c_double(0.0), C.c_double(0.0), C.c_int(0)
    rc = lib.nimref_run_blocks(N, _d(coords), E, _i(conn), len(mats), _i(eb),
                               "\n".join(mt.line() for mt in mats).encode(), len(names), _i(ns_ptr), _i(ns_nodes),
                               "\n".join(names).encode(), bcs.encode(), float(final_time), int(num_steps), of,
                               _d(v0), T, _d(out["u"]), _d(out["v"]), _d(out["a"]), _d(out["f_int"]),
                               _d(out.get("F")), _d(out.get("sigma")), _d(mass), C.cast(C.pointer(dt), _dp),
                               C.cast(C.pointer(secs), _dp), C.byref(n))
    if rc != 0:
        raise RuntimeError("reference run failed: " + lib.nimref_last_error().decode())
    states = []
    for t in range(n.value):
        st = {k: v[t] for k, v in out.items()}
        st.update(mass=mass, dt_crit=dt.value, loop_seconds=secs.value)
        states.append(st)
    return states


def _uq_outputs(problem, spec, num_steps, output_frequency):
    N = problem.num_nodes
    of = int(output_frequency)
    T = 1 if of == 0 else (int(num_steps) + of - 1) // of + 1
    S = spec.num_exact + spec.num_approx
    return T, {"u": np.zeros((T, N, 3)), "v": np.zeros((T, N, 3)), "f": np.zeros((T, N, 3)),
               "su": np.zeros((T, S, N, 3)), "sv": np.zeros((T, S, N, 3)), "sf": np.zeros((T, S, N, 3))}


def run_port_uq(problem, spec, final_time, num_steps, output_frequency=0, threads=1):
    """The C restatement of the reference's UQ mode (nsm_oracle_run_uq): the
    nominal trajectory (u, v, f [T,N,3]) and the samples (su, sv, sf
    [T,S,N,3], exact first) after every output step."""
    keep = []
    m = _model(problem, keep)
    prm = spec.sample_parameters(problem)
    ne = spec.num_exact
    kb = np.ascontiguousarray(prm["bulk_modulus"][:ne])
    ks = np.ascontiguousarray(prm["shear_modulus"][:ne])
    cf = np.ascontiguousarray(spec.coefficients)
    T, out = _uq_outputs(problem, spec, num_steps, output_frequency)
    v0 = None if problem.v_init is None else np.ascontiguousarray(problem.v_init, dtype=np.float64)
    n = C.c_int(0)
    rc = port().nsm_oracle_run_uq(C.byref(m), ne, _d(kb), _d(ks), spec.num_approx, _d(cf), float(final_time),
                                  int(num_steps), int(output_frequency), _d(v0), int(threads), T, _d(out["u"]),
                                  _d(out["v"]), _d(out["f"]), _d(out["su"]), _d(out["sv"]), _d(out["sf"]),
                                  C.byref(n))
    if rc != 0:
        raise RuntimeError(f"oracle UQ run failed ({rc})")
    return {k: v[: n.value] for k, v in out.items()}


def run_ref_uq(problem, spec, final_time, num_steps, output_frequency=0, workdir="."):
    """The reference's own UQ mode (nimble_uq::ModelData through the
    harness): same outputs as run_port_uq.  The samples file is written into
    workdir, which is also the working directory during the run (the
    reference writes parameter_samples.dat there)."""
    lib = ref_uq()
    names = list(problem.node_sets.keys())
    ns_ptr = np.zeros(len(names) + 1, np.int32)
    parts = []
    for s, nm in enumerate(names):
        ids = np.asarray(problem.node_sets[nm], np.int32)
        parts.append(ids)
        ns_ptr[s + 1] = ns_ptr[s] + len(ids)
    ns_nodes = np.concatenate(parts).astype(np.int32) if parts else np.zeros(0, np.int32)
    bcs = "\n".join(bc.line() for bc in problem.bcs)
    coords = np.ascontiguousarray(problem.coords, dtype=np.float64)
    conn = np.ascontiguousarray(problem.conn, dtype=np.int32)
    mats = problem.materials()
    eb = np.ascontiguousarray(problem.elem_block, dtype=np.int32) if len(mats) > 1 else None
    v0 = None if problem.v_init is None else np.ascontiguousarray(problem.v_init, dtype=np.float64)
    T, out = _uq_outputs(problem, spec, num_steps, output_frequency)
    workdir = os.path.abspath(workdir)
    samples = os.path.join(workdir, "uq_samples.txt")
    with open(samples, "w") as f:
        f.write(spec.samples_text())
    mass, dt, n = np.zeros(problem.num_nodes), C.c_double(0.0), C.c_int(0)
    cwd = os.getcwd()
    os.chdir(workdir)
    try:
        rc = lib.nimref_run_uq(problem.num_nodes, _d(coords), problem.num_elem, _i(conn), len(mats), _i(eb),
                               "\n".join(mt.line() for mt in mats).encode(), len(names), _i(ns_ptr), _i(ns_nodes),
                               "\n".join(names).encode(), bcs.encode(), float(final_time), int(num_steps),
                               int(output_frequency), _d(v0), "\n".join(spec.parameter_lines()).encode(),
                               samples.encode(), spec.num_exact + spec.num_approx, T, _d(out["u"]), _d(out["v"]),
                               _d(out["f"]), _d(out["su"]), _d(out["sv"]), _d(out["sf"]), _d(mass),
                               C.cast(C.pointer(dt), _dp), C.byref(n))
    finally:
        os.chdir(cwd)
    if rc != 0:
        raise RuntimeError("reference UQ run failed: " + lib.nimref_last_error().decode())
    return {k: v[: n.value] for k, v in out.items()}


def run_ref(problem, final_time, num_steps, output_frequency=0, with_ip=True):
    """Runs the reference itself (oracle/_ref); same outputs as run_port (the
    state after the last step)."""
    return run_ref_outputs(problem, final_time, num_steps, output_frequency, with_ip)[-1]


def element(X, u, K, G, which="port"):
    """One element (X, u: [8,3]) -> (F [8,9], sigma [8,6], f [8,3])."""
    X = np.ascontiguousarray(X, dtype=np.float64)
    u = np.ascontiguousarray(u, dtype=np.float64)
    F, s, f = np.zeros((8, 9)), np.zeros((8, 6)), np.zeros((8, 3))
    if which == "port":
        port().nsm_oracle_element(_d(X), _d(u), K, G, _d(F), _d(s), _d(f))
    else:
        if ref().nimref_element(_d(X), _d(u), 1.0, K, G, _d(F), _d(s), _d(f)) != 0:
            raise RuntimeError(ref().nimref_last_error().decode())
    return F, s, f


def stress(F, K, G, which="port"):
    F = np.ascontiguousarray(F, dtype=np.float64).reshape(-1, 9)
    s = np.zeros((F.shape[0], 6))
    if which == "port":
        port().nsm_oracle_stress(F.shape[0], _d(F), K, G, _d(s))
    else:
        if ref().nimref_stress(F.shape[0], _d(F), K, G, _d(s)) != 0:
            raise RuntimeError(ref().nimref_last_error().decode())
    return s


def stress_exact(problem, u, elems):
    """Extended-precision stress of displacement u at the points of `elems`
    ([len(elems), 8, 6]): the yardstick for the FP64 stresses' accuracy."""
    keep = []
    m = _model(problem, keep)
    u = np.ascontiguousarray(u, dtype=np.float64)
    elems = np.ascontiguousarray(elems, dtype=np.int32)
    out = np.zeros((len(elems), 8, 6))
    port().nsm_oracle_stress_exact(C.byref(m), _d(u), len(elems), _i(elems), _d(out))
    return out


def volume_average(x_cur, q, which="port"):
    """One element's volume and volume average of point quantities q
    ([8, nq]) at current coordinates x_cur ([8, 3]) -> (volume, avg [nq]),
    HexElement::ComputeVolumeAverage."""
    x = np.ascontiguousarray(x_cur, dtype=np.float64)
    q = np.ascontiguousarray(q, dtype=np.float64).reshape(8, -1)
    nq = q.shape[1]
    vol, avg = C.c_double(0.0), np.zeros(nq)
    if which == "port":
        port().nsm_oracle_volume_average(_d(x), nq, _d(q), C.cast(C.pointer(vol), _dp), _d(avg))
    else:
        if ref().nimref_volume_average(_d(x), nq, _d(q), C.cast(C.pointer(vol), _dp), _d(avg)) != 0:
            raise RuntimeError(ref().nimref_last_error().decode())
    return vol.value, avg


def derived_element_data(problem, u, sigma, F):
    """Element volume [E] and volume-averaged stress [E,6] and deformation
    gradient [E,9] of displacement u ([N,3]) and point data sigma ([E,8,6]),
    F ([E,8,9]), Block::ComputeDerivedElementData."""
    keep = []
    m = _model(problem, keep)
    u = np.ascontiguousarray(u, dtype=np.float64)
    q = np.ascontiguousarray(sigma, dtype=np.float64)
    f = np.ascontiguousarray(F, dtype=np.float64)
    E = problem.num_elem
    vol, avg, avg_F = np.zeros(E), np.zeros((E, 6)), np.zeros((E, 9))
    port().nsm_oracle_derived_element_data(C.byref(m), _d(u), _d(q), _d(f), _d(vol), _d(avg), _d(avg_F))
    return vol, avg, avg_F


def shape_tables():
    N, dN = np.zeros((8, 8)), np.zeros((8, 8, 3))
    port().nsm_oracle_shape_tables(_d(N), _d(dN))
    return N, dN


def energy_density(F, K, G):
    F = np.ascontiguousarray(F, dtype=np.float64)
    return port().nsm_oracle_energy_density(_d(F), K, G)
