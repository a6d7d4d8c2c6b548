"""Python binding of the engine's C ABI (include/nimble_gb300.h).

`Model` mirrors the reference's ModelDataBase interface for one block
(src/nimble_model_data_base.h:87-345: ComputeLumpedMass, GetCriticalTimeStep,
ApplyInitialConditions, ApplyKinematicConditions, ComputeInternalForce,
GetVectorNodeData, ...) and adds the device-resident explicit loop of
ExplicitTimeIntegrator::Integrate (src/integrators/explicit_time_integrator.cc:61-325)
as `begin` / `advance`.  Every call goes through libnimble_gb300.so; there is
no other implementation behind it, and a missing library is an ImportError.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .mesh import BC_PRESCRIBED_DISPLACEMENT, BC_PRESCRIBED_TRACTION, Problem

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libnimble_gb300.so")

NSM_OK = 0
ERRORS = {1: "invalid argument", 2: "CUDA error", 3: "non-positive Jacobian", 4: "non-finite force",
          5: "call out of order", 6: "out of memory"}
PRECISION = {"fp64": 0, "fp32": 1, "fp32_mixed": 1}
FIELDS = {"reference_coordinate": 0, "displacement": 1, "velocity": 2, "acceleration": 3,
          "internal_force": 4, "external_force": 5}


class EngineError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class _Mesh(C.Structure):
    _fields_ = [("num_nodes", C.c_int), ("num_elem", C.c_int), ("coords", C.POINTER(C.c_double)),
                ("conn", C.POINTER(C.c_int))]


class _Material(C.Structure):
    _fields_ = [("density", C.c_double), ("bulk_modulus", C.c_double), ("shear_modulus", C.c_double)]


class _AnyMaterial(C.Structure):
    _fields_ = [("model", C.c_int), ("reserved", C.c_int), ("density", C.c_double), ("bulk_modulus", C.c_double),
                ("shear_modulus", C.c_double)]


class _Options(C.Structure):
    _fields_ = [("precision", C.c_int), ("store_ip_data", C.c_int), ("device", C.c_int),
                ("graph_steps", C.c_int)]


_dp = C.POINTER(C.c_double)
_dp_f = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int)
_vp = C.c_void_p


class _HostBcs(C.Structure):
    _fields_ = [("num_bcs", C.c_int), ("kind", _ip), ("component", _ip), ("value", _dp), ("ptr", _ip),
                ("nodes", _ip)]

# name -> (restype, argtypes); kept in step with include/nimble_gb300.h
SIGNATURES = {
    "nsm_last_error": (C.c_char_p, []),
    "nsm_abi_version": (C.c_int, []),
    "nsm_create": (C.c_int, [C.POINTER(_Mesh), C.POINTER(_Material), C.POINTER(_Options), C.POINTER(_vp)]),
    "nsm_create_blocks": (C.c_int, [C.POINTER(_Mesh), C.c_int, _ip, C.POINTER(_AnyMaterial), C.POINTER(_Options),
                                    C.POINTER(_vp)]),
    "nsm_create_uq": (C.c_int, [C.POINTER(_Mesh), C.c_int, _ip, C.POINTER(_AnyMaterial), C.c_int, _dp, _dp, C.c_int,
                                _dp, C.POINTER(_Options), C.POINTER(_vp)]),
    "nsm_destroy": (C.c_int, [_vp]),
    "nsm_add_boundary_condition": (C.c_int, [_vp, C.c_int, C.c_int, C.c_double, _ip, C.c_int]),
    "nsm_add_boundary_condition_expression": (C.c_int, [_vp, C.c_int, C.c_int, C.c_char_p, _ip, C.c_int]),
    "nsm_bc_expression_eval": (C.c_int, [C.c_char_p, C.c_double, C.c_double, C.c_double, C.c_double, _dp]),
    "nsm_compute_lumped_mass": (C.c_int, [_vp, _dp]),
    "nsm_critical_time_step": (C.c_int, [_vp, _dp]),
    "nsm_apply_initial_conditions": (C.c_int, [_vp]),
    "nsm_apply_kinematic_conditions": (C.c_int, [_vp, C.c_double, C.c_double]),
    "nsm_set_node_field": (C.c_int, [_vp, C.c_int, _dp]),
    "nsm_get_node_field": (C.c_int, [_vp, C.c_int, _dp]),
    "nsm_compute_internal_force": (C.c_int, [_vp, C.c_double, C.c_double, C.c_int]),
    "nsm_compute_internal_force_host": (C.c_int, [_vp, _dp, _dp]),
    "nsm_set_host_chunks": (C.c_int, [_vp, C.c_int]),
    "nsm_set_block_material_callback": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _vp]),
    "nsm_get_state_data": (C.c_int, [_vp, _dp]),
    "nsm_example_neohookean_callback": (C.c_int, [_vp, _vp]),
    "nsm_example_history_callback": (C.c_int, [_vp, _vp]),
    "nsm_host_chunks": (C.c_int, [_vp, _ip]),
    "nsm_get_ip_data": (C.c_int, [_vp, _dp, _dp]),
    "nsm_compute_derived_element_data": (C.c_int, [_vp, _dp, _dp, _dp]),
    "nsm_get_energies": (C.c_int, [_vp, _dp, _dp]),
    "nsm_begin": (C.c_int, [_vp, C.c_double, C.c_double, C.c_int, C.c_int, _dp]),
    "nsm_advance": (C.c_int, [_vp, C.c_int]),
    "nsm_advance_timed": (C.c_int, [_vp, C.c_int, _dp]),
    "nsm_progress": (C.c_int, [_vp, _ip, _dp]),
    "nsm_synchronize": (C.c_int, [_vp]),
    "nsm_check_status": (C.c_int, [_vp]),
    "nsm_time_kernels": (C.c_int, [_vp, C.c_int, _dp, _dp]),
    "nsm_launches_per_advance": (C.c_int, [_vp, C.c_int]),
    "nsm_set_profiling": (C.c_int, [_vp, C.c_int]),
    "nsm_get_profile": (C.c_int, [_vp, _dp, _ip, _dp, _ip]),
    "nsm_create_ensemble": (C.c_int, [C.c_int, C.POINTER(_Mesh), C.POINTER(_Material), C.POINTER(_Options),
                                      C.POINTER(_vp)]),
    "nsm_ensemble_offsets": (C.c_int, [_vp, _ip, _ip]),
    "nsm_ensemble_time_steps": (C.c_int, [_vp, _dp]),
    "nsm_ensemble_max_abs": (C.c_int, [_vp, C.c_int, C.c_int, _ip, C.c_int, _dp]),
    "nsm_begin_ensemble": (C.c_int, [_vp, C.c_double, _dp, C.c_int, C.c_int, _dp]),
    "nsm_autotune": (C.c_int, [_vp, C.c_int, _ip, _dp]),
    "nsm_launch_candidate_times": (C.c_int, [_vp, C.c_int, _dp, C.c_int, _ip]),
    "nsm_set_launch_candidate": (C.c_int, [_vp, C.c_int]),
    "nsm_critical_time_step_noalloc": (C.c_int, [C.c_int, C.c_int, _vp, _vp, _vp, C.c_double, C.c_double, _vp,
                                                _vp]),
    "nsm_mlp_last_error": (C.c_char_p, []),
    "nsm_mlp_create": (C.c_int, [C.c_double, C.c_double, C.c_ulonglong, C.c_int, C.POINTER(_vp)]),
    "nsm_mlp_destroy": (C.c_int, [_vp]),
    "nsm_mlp_generate": (C.c_int, [_vp, C.c_long, C.c_ulonglong, C.c_double, C.c_double]),
    "nsm_mlp_train": (C.c_int, [_vp, C.c_int, C.c_int, C.c_double, _dp]),
    "nsm_mlp_get_params": (C.c_int, [_vp, _dp_f, _dp_f]),
    "nsm_mlp_set_params": (C.c_int, [_vp, _dp_f, _dp_f]),
    "nsm_mlp_training_sample": (C.c_int, [_vp, C.c_long, C.c_long, _dp_f, _dp_f]),
    "nsm_mlp_gradient": (C.c_int, [_vp, C.c_long, _dp_f, _dp_f, _dp_f, _dp]),
    "nsm_mlp_predict": (C.c_int, [_vp, C.c_long, _dp, _dp, _ip]),
    "nsm_set_mlp_closure": (C.c_int, [_vp, _vp]),
    "nsm_closure_fallbacks": (C.c_int, [_vp, C.POINTER(C.c_ulonglong)]),
    "nsm_tc_selftest": (C.c_int, [C.c_int, C.c_int, _dp_f, _dp_f, _dp_f]),
    "nsm_tc_wait_timeout_selftest": (C.c_int, [C.c_long, C.POINTER(C.c_int)]),
    "nsm_device_sm_count": (C.c_int, [C.c_int, C.POINTER(C.c_int)]),
    "nsm_host_loop_steps": (C.c_int, [_vp, C.c_int, _dp, C.c_double, C.c_int, C.c_int, C.c_int, _dp,
                                      C.POINTER(_HostBcs), _dp, _dp, _dp, _dp, _dp]),
    "nsm_host_alloc": (_vp, [C.c_size_t]),
    "nsm_host_free": (None, [_vp]),
}

_lib = None


def library():
    """Loads libnimble_gb300.so (built by nimblesm_gb300.build)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with nimblesm_gb300.build.build()")
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _check(rc):
    if rc != NSM_OK:
        raise EngineError(rc, library().nsm_last_error().decode())


def _add_bc(lib, h, bc, nodes):
    """One boundary-condition line over its (global) node ids (a traction line
    applies nothing, as in the reference)."""
    if bc.kind == BC_PRESCRIBED_TRACTION:
        return
    if bc.expression is not None:
        _check(lib.nsm_add_boundary_condition_expression(h, bc.kind, bc.component, bc.expression.encode(),
                                                         nodes.ctypes.data_as(_ip), len(nodes)))
    else:
        _check(lib.nsm_add_boundary_condition(h, bc.kind, bc.component, bc.value, nodes.ctypes.data_as(_ip),
                                              len(nodes)))


# The block-material callback type (nsm_stress_callback): int fn(void* user,
# const nsm_stress_request* request).
STRESS_CALLBACK = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p)


def example_callback(name):
    """The address of one of the library's example block-material callbacks:
    "neohookean" (stateless) or "history" (one state variable per point)."""
    return C.cast(getattr(library(), f"nsm_example_{name}_callback"), C.c_void_p).value


def bc_expression_eval(expression, x=0.0, y=0.0, z=0.0, t=0.0):
    """One host evaluation of a boundary-condition expression as the engine
    parses it (nsm_bc_expression_eval)."""
    v = C.c_double()
    _check(library().nsm_bc_expression_eval(expression.encode(), float(x), float(y), float(z), float(t),
                                           C.byref(v)))
    return v.value


def _d(a):
    return a.ctypes.data_as(_dp)


class PinnedArray:
    """A page-locked host array (nsm_host_alloc) viewed as numpy."""

    def __init__(self, shape, dtype=np.float64):
        self.shape = tuple(shape)
        nbytes = int(np.prod(self.shape)) * np.dtype(dtype).itemsize
        self._ptr = library().nsm_host_alloc(max(nbytes, 8))
        if not self._ptr:
            raise MemoryError("pinned allocation failed")
        buf = (C.c_char * max(nbytes, 8)).from_address(self._ptr)
        self.array = np.frombuffer(buf, dtype=dtype, count=int(np.prod(self.shape))).reshape(self.shape)

    def __del__(self):
        if getattr(self, "_ptr", None):
            library().nsm_host_free(self._ptr)
            self._ptr = None


class Model:
    """Device-resident ModelData for one block of hex8 elements (or, built
    from several problems, an ensemble of independent samples in one handle)."""

    def __init__(self, problem, precision: str = "fp64", store_ip_data: bool = True, device: int = 0,
                 graph_steps: int = 50):
        lib = library()
        problems = list(problem) if isinstance(problem, (list, tuple)) else [problem]
        self.problems = problems
        self.problem = problems[0] if len(problems) == 1 else _concatenate(problems)
        self.precision = precision
        keep = []
        meshes = (_Mesh * len(problems))()
        mats = (_Material * len(problems))()
        for g, p in enumerate(problems):
            coords = np.ascontiguousarray(p.coords, dtype=np.float64)
            conn = np.ascontiguousarray(p.conn, dtype=np.int32)
            keep += [coords, conn]
            meshes[g] = _Mesh(p.num_nodes, p.num_elem, _d(coords), conn.ctypes.data_as(_ip))
            mats[g] = _Material(p.density, p.bulk_modulus, p.shear_modulus)
        opt = _Options(PRECISION[precision], 1 if store_ip_data else 0, device, graph_steps)
        h = _vp()
        single = problems[0]
        if len(problems) == 1 and (single.blocks or single.material_model != "neohookean"):
            blocks = single.materials()
            bm = (_AnyMaterial * len(blocks))()
            for b, mt in enumerate(blocks):
                bm[b] = _AnyMaterial(mt.MODELS[mt.model], 0, mt.density, mt.bulk_modulus, mt.shear_modulus)
            eb = None
            if len(blocks) > 1:
                eb = np.ascontiguousarray(single.elem_block, dtype=np.int32)
                keep.append(eb)
            _check(lib.nsm_create_blocks(meshes, len(blocks), eb.ctypes.data_as(_ip) if eb is not None else None,
                                         bm, C.byref(opt), C.byref(h)))
        elif len(problems) == 1:
            _check(lib.nsm_create(meshes, mats, C.byref(opt), C.byref(h)))
        else:
            _check(lib.nsm_create_ensemble(len(problems), meshes, mats, C.byref(opt), C.byref(h)))
        self._h = h
        S = len(problems)
        no, eo = np.zeros(S + 1, np.int32), np.zeros(S + 1, np.int32)
        _check(lib.nsm_ensemble_offsets(h, no.ctypes.data_as(_ip), eo.ctypes.data_as(_ip)))
        self.node_offsets, self.elem_offsets = no, eo
        for g, p in enumerate(problems):
            for bc in p.bcs:
                if bc.node_set not in p.node_sets:
                    continue  # the reference drops lines naming an absent node set
                nodes = np.ascontiguousarray(np.asarray(p.node_sets[bc.node_set]) + no[g], dtype=np.int32)
                _add_bc(lib, h, bc, nodes)

    def close(self):
        if getattr(self, "_h", None):
            library().nsm_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    # ---- ModelDataBase mirror ----
    def ComputeLumpedMass(self) -> np.ndarray:
        m = np.zeros(self.problem.num_nodes)
        _check(library().nsm_compute_lumped_mass(self._h, _d(m)))
        return m

    def GetCriticalTimeStep(self) -> float:
        dt = C.c_double()
        _check(library().nsm_critical_time_step(self._h, C.byref(dt)))
        return dt.value

    def ApplyInitialConditions(self):
        _check(library().nsm_apply_initial_conditions(self._h))

    def ApplyKinematicConditions(self, time_current, time_previous):
        _check(library().nsm_apply_kinematic_conditions(self._h, time_current, time_previous))

    def GetVectorNodeData(self, label) -> np.ndarray:
        out = np.zeros((self.problem.num_nodes, 3))
        _check(library().nsm_get_node_field(self._h, FIELDS[label], _d(out)))
        return out

    def SetVectorNodeData(self, label, values):
        v = np.ascontiguousarray(values, dtype=np.float64)
        assert v.shape == (self.problem.num_nodes, 3)
        _check(library().nsm_set_node_field(self._h, FIELDS[label], _d(v)))

    def ComputeInternalForce(self, time_previous=0.0, time_current=0.0, is_output_step=False):
        _check(library().nsm_compute_internal_force(self._h, time_previous, time_current, int(is_output_step)))

    def set_block_material_callback(self, block, fn, num_state=0, user=None):
        """Block `block`'s stress computed by the callback `fn` (a C function
        address, or a STRESS_CALLBACK instance kept alive by the caller) with
        num_state variables per point; fn None restores the block's material."""
        addr = None if fn is None else (C.cast(fn, C.c_void_p).value if isinstance(fn, STRESS_CALLBACK) else fn)
        _check(library().nsm_set_block_material_callback(self._h, int(block), int(num_state), addr, user))
        self._num_state = max(getattr(self, "_num_state", 0), int(num_state)) if fn is not None else \
            getattr(self, "_num_state", 0)

    def get_state_data(self):
        """The per-point state after the last step, [E, 8, num_state]."""
        ns = getattr(self, "_num_state", 0)
        out = np.zeros((self.problem.num_elem, 8, ns))
        if ns:
            _check(library().nsm_get_state_data(self._h, _d(out)))
        return out

    def set_host_chunks(self, chunks):
        """Element ranges of the host-buffer pipeline (0: default)."""
        _check(library().nsm_set_host_chunks(self._h, int(chunks)))

    def host_chunks(self):
        c = C.c_int()
        _check(library().nsm_host_chunks(self._h, C.byref(c)))
        return c.value

    def ComputeInternalForceHost(self, displacement, out=None) -> np.ndarray:
        u = np.ascontiguousarray(displacement, dtype=np.float64)
        f = out if out is not None else np.zeros((self.problem.num_nodes, 3))
        _check(library().nsm_compute_internal_force_host(self._h, _d(u), _d(f)))
        return f

    def HostLoopSteps(self, num_steps, time_current, dt_user, mass, u, v, a, f_int, output_frequency=0,
                      first_step=0, num_load_steps=0):
        """The reference integrator's loop on host arrays (u, v, a, f_int
        [N][3], updated in place; mass [N]) around the host-buffer force call:
        num_steps steps from time_current.  Returns (time, host seconds)."""
        kinds, comps, vals, ptr, nodes = self.problem.bc_arrays()
        bcs = _HostBcs(len(kinds), kinds.ctypes.data_as(_ip), comps.ctypes.data_as(_ip), _d(vals),
                       ptr.ctypes.data_as(_ip), nodes.ctypes.data_as(_ip))
        t, secs = C.c_double(time_current), C.c_double(0.0)
        for x in (u, v, a, f_int):
            assert x.dtype == np.float64 and x.flags.c_contiguous and x.shape == (self.problem.num_nodes, 3)
        m = np.ascontiguousarray(mass, dtype=np.float64)
        _check(library().nsm_host_loop_steps(self._h, int(num_steps), C.byref(t), float(dt_user),
                                             int(output_frequency), int(first_step), int(num_load_steps), _d(m),
                                             C.byref(bcs), _d(u), _d(v), _d(a), _d(f_int), C.byref(secs)))
        return t.value, secs.value

    def GetIntegrationPointData(self):
        E = self.problem.num_elem
        F, s = np.zeros((E, 8, 9)), np.zeros((E, 8, 6))
        _check(library().nsm_get_ip_data(self._h, _d(F), _d(s)))
        return F, s

    def ComputeDerivedElementData(self):
        """Element volume [E], volume-averaged stress [E][6] and deformation
        gradient [E][9] of the current configuration
        (Block::ComputeDerivedElementData)."""
        E = self.problem.num_elem
        vol, s, F = np.zeros(E), np.zeros((E, 6)), np.zeros((E, 9))
        _check(library().nsm_compute_derived_element_data(self._h, _d(vol), _d(s), _d(F)))
        return vol, s, F

    def GetEnergies(self):
        ke, ie = C.c_double(), C.c_double()
        _check(library().nsm_get_energies(self._h, C.byref(ke), C.byref(ie)))
        return ke.value, ie.value

    # ---- explicit loop ----
    def begin(self, final_time, num_steps, output_frequency=0, initial_time=0.0, v_init="problem"):
        """final_time: a number, or one per sample for an ensemble."""
        if isinstance(v_init, str):
            v_init = self.problem.v_init
        v = None if v_init is None else np.ascontiguousarray(v_init, dtype=np.float64)
        ft = np.ascontiguousarray(np.broadcast_to(np.asarray(final_time, np.float64), (len(self.problems),)))
        _check(library().nsm_begin_ensemble(self._h, initial_time, _d(ft), num_steps, output_frequency,
                                            None if v is None else _d(v)))

    # ---- ensemble ----
    def sample_time_steps(self):
        dt = np.zeros(len(self.problems))
        _check(library().nsm_ensemble_time_steps(self._h, _d(dt)))
        return dt

    def sample_max_abs(self, label, component, node_sets):
        """Per-sample max |field component| over node_sets[g] (local ids of
        sample g)."""
        ids = np.ascontiguousarray(np.concatenate([np.asarray(ns, np.int64) + self.node_offsets[g]
                                                   for g, ns in enumerate(node_sets)]), dtype=np.int32)
        out = np.zeros(len(self.problems))
        _check(library().nsm_ensemble_max_abs(self._h, FIELDS[label], component, ids.ctypes.data_as(_ip),
                                              len(ids), _d(out)))
        return out

    def sample_slice(self, g):
        return slice(int(self.node_offsets[g]), int(self.node_offsets[g + 1]))

    def set_closure(self, closure):
        """Use a trained MLPClosure as the material (FP32-mixed form)."""
        self._closure = closure
        _check(library().nsm_set_mlp_closure(self._h, None if closure is None else closure._h))

    def closure_fallbacks(self):
        c = C.c_ulonglong()
        _check(library().nsm_closure_fallbacks(self._h, C.byref(c)))
        return c.value

    def autotune(self, repeats=5):
        c, ms = C.c_int(), C.c_double()
        _check(library().nsm_autotune(self._h, repeats, C.byref(c), C.byref(ms)))
        return c.value, ms.value

    def set_launch_candidate(self, candidate):
        _check(library().nsm_set_launch_candidate(self._h, int(candidate)))

    def launch_candidate_times(self, repeats=5):
        """Mean element-kernel milliseconds of every candidate launch shape."""
        n = C.c_int()
        _check(library().nsm_launch_candidate_times(self._h, repeats, None, 0, C.byref(n)))
        ms = (C.c_double * n.value)()
        _check(library().nsm_launch_candidate_times(self._h, repeats, ms, n.value, None))
        return list(ms)

    def advance(self, num_steps):
        _check(library().nsm_advance(self._h, int(num_steps)))

    def advance_timed(self, num_steps) -> float:
        """Advances and returns the device milliseconds (CUDA events on the
        engine's stream)."""
        ms = C.c_double()
        _check(library().nsm_advance_timed(self._h, int(num_steps), C.byref(ms)))
        return ms.value

    def synchronize(self):
        _check(library().nsm_synchronize(self._h))
        _check(library().nsm_check_status(self._h))

    def progress(self):
        s, t = C.c_int(), C.c_double()
        _check(library().nsm_progress(self._h, C.byref(s), C.byref(t)))
        return s.value, t.value

    def state(self, with_ip=True):
        """Post-step state in the reference layouts."""
        self.synchronize()
        out = {k: self.GetVectorNodeData(lbl) for k, lbl in
               (("u", "displacement"), ("v", "velocity"), ("a", "acceleration"), ("f_int", "internal_force"))}
        if with_ip:
            out["F"], out["sigma"] = self.GetIntegrationPointData()
        out["mass"] = self.ComputeLumpedMass()
        out["steps"], out["time"] = self.progress()
        return out

    # ---- measurement helpers ----
    def time_kernels(self, repeats=10):
        e, n = C.c_double(), C.c_double()
        _check(library().nsm_time_kernels(self._h, repeats, C.byref(e), C.byref(n)))
        return e.value, n.value

    def launches_per_advance(self, num_steps):
        return library().nsm_launches_per_advance(self._h, int(num_steps))

    def set_profiling(self, enable):
        _check(library().nsm_set_profiling(self._h, int(bool(enable))))

    def get_profile(self):
        te, tn = C.c_double(), C.c_double()
        ne, nn = C.c_int(), C.c_int()
        _check(library().nsm_get_profile(self._h, C.byref(te), C.byref(ne), C.byref(tn), C.byref(nn)))
        return {"element_ms": te.value, "element_launches": ne.value, "node_ms": tn.value,
                "node_launches": nn.value}


def _check_mlp(rc):
    if rc != NSM_OK:
        raise EngineError(rc, library().nsm_mlp_last_error().decode())


class MLPClosure:
    """The learned constitutive closure (nsm_mlp_*): a BF16 tensor-core MLP
    standing in for the neo-Hookean stress update."""

    PARAMS = 5190

    def __init__(self, bulk_modulus, shear_modulus, seed=1, device=0):
        h = _vp()
        _check_mlp(library().nsm_mlp_create(bulk_modulus, shear_modulus, seed, device, C.byref(h)))
        self._h = h
        self.bulk_modulus, self.shear_modulus = bulk_modulus, shear_modulus

    def close(self):
        if getattr(self, "_h", None):
            library().nsm_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def generate(self, n, seed=7, perturbation=0.05, min_det=0.5):
        _check_mlp(library().nsm_mlp_generate(self._h, int(n), seed, perturbation, min_det))

    def train(self, epochs, batch_tiles=128, lr=2e-3):
        loss = C.c_double()
        _check_mlp(library().nsm_mlp_train(self._h, int(epochs), int(batch_tiles), lr, C.byref(loss)))
        return loss.value

    def params(self):
        p = np.zeros(self.PARAMS, np.float32)
        s = np.zeros(5, np.float32)
        _check_mlp(library().nsm_mlp_get_params(self._h, p.ctypes.data_as(_dp_f), s.ctypes.data_as(_dp_f)))
        return p, s

    def set_params(self, params=None, scales=None):
        p = None if params is None else np.ascontiguousarray(params, np.float32)
        s = None if scales is None else np.ascontiguousarray(scales, np.float32)
        _check_mlp(library().nsm_mlp_set_params(self._h, None if p is None else p.ctypes.data_as(_dp_f),
                                                None if s is None else s.ctypes.data_as(_dp_f)))

    def training_sample(self, first, count):
        H = np.zeros((count, 9), np.float32)
        Y = np.zeros((count, 6), np.float32)
        _check_mlp(library().nsm_mlp_training_sample(self._h, first, count, H.ctypes.data_as(_dp_f),
                                                     Y.ctypes.data_as(_dp_f)))
        return H, Y

    def gradient(self, H, Y):
        H = np.ascontiguousarray(H, np.float32)
        Y = np.ascontiguousarray(Y, np.float32)
        g = np.zeros(self.PARAMS, np.float32)
        loss = C.c_double()
        _check_mlp(library().nsm_mlp_gradient(self._h, H.shape[0], H.ctypes.data_as(_dp_f), Y.ctypes.data_as(_dp_f),
                                              g.ctypes.data_as(_dp_f), C.byref(loss)))
        return g, loss.value

    def predict(self, F):
        F = np.ascontiguousarray(F, np.float64).reshape(-1, 9)
        s = np.zeros((F.shape[0], 6))
        fb = C.c_int()
        _check_mlp(library().nsm_mlp_predict(self._h, F.shape[0], _d(F), _d(s), C.byref(fb)))
        return s, fb.value


class UqModel(Model):
    """The reference's UQ mode on one mesh (nsm_create_uq) for a UqSpec:
    trajectory 0 is the nominal, then the exact samples (element forces with
    their own moduli), then the approximate samples (force from the linear
    closure).  Every trajectory gets the velocity-type conditions, the nominal
    alone the prescribed displacements, all of them the nominal's schedule and
    the problem's initial velocity."""

    def __init__(self, problem, spec, precision: str = "fp64", store_ip_data: bool = True, device: int = 0,
                 graph_steps: int = 50):
        lib = library()
        ne, na = spec.num_exact, spec.num_approx
        S = 1 + ne + na
        N, E = problem.num_nodes, problem.num_elem
        self.spec, self.num_trajectories, self.mesh_problem = spec, S, problem
        self.problems = [problem] * S
        self.problem = Problem(coords=np.concatenate([problem.coords] * S),
                               conn=np.concatenate([problem.conn + k * N for k in range(1 + ne)]).astype(np.int32),
                               node_sets={}, density=problem.density, bulk_modulus=problem.bulk_modulus,
                               shear_modulus=problem.shear_modulus, bcs=[],
                               v_init=None if problem.v_init is None else np.concatenate([problem.v_init] * S))
        self.precision = precision
        mats = problem.materials()
        bm = (_AnyMaterial * len(mats))()
        for b, mt in enumerate(mats):
            bm[b] = _AnyMaterial(mt.MODELS[mt.model], 0, mt.density, mt.bulk_modulus, mt.shear_modulus)
        prm = spec.sample_parameters(problem)
        kb = np.ascontiguousarray(prm["bulk_modulus"][:ne])
        ks = np.ascontiguousarray(prm["shear_modulus"][:ne])
        cf = np.ascontiguousarray(spec.coefficients, dtype=np.float64)
        coords = np.ascontiguousarray(problem.coords, dtype=np.float64)
        conn = np.ascontiguousarray(problem.conn, dtype=np.int32)
        eb = np.ascontiguousarray(problem.elem_block, dtype=np.int32) if len(mats) > 1 else None
        self._keep = [coords, conn, kb, ks, cf, eb]
        mesh = _Mesh(N, E, _d(coords), conn.ctypes.data_as(_ip))
        opt = _Options(PRECISION[precision], 1 if store_ip_data else 0, device, graph_steps)
        h = _vp()
        _check(lib.nsm_create_uq(C.byref(mesh), len(mats), None if eb is None else eb.ctypes.data_as(_ip), bm, ne,
                                 _d(kb), _d(ks), na, _d(cf), C.byref(opt), C.byref(h)))
        self._h = h
        no, eo = np.zeros(S + 1, np.int32), np.zeros(S + 1, np.int32)
        _check(lib.nsm_ensemble_offsets(h, no.ctypes.data_as(_ip), eo.ctypes.data_as(_ip)))
        self.node_offsets, self.elem_offsets = no, eo
        for t in range(S):
            for bc in problem.bcs:
                if bc.node_set not in problem.node_sets:
                    continue
                if bc.kind == BC_PRESCRIBED_DISPLACEMENT and t > 0:
                    continue
                nodes = np.ascontiguousarray(np.asarray(problem.node_sets[bc.node_set]) + no[t], dtype=np.int32)
                _add_bc(lib, h, bc, nodes)

    def trajectories(self, label):
        """A nodal vector field of every trajectory: [trajectories, N, 3]
        (nominal, exact samples, approximate samples)."""
        return self.GetVectorNodeData(label).reshape(self.num_trajectories, self.mesh_problem.num_nodes, 3)


def _concatenate(problems):
    """The ensemble's problems as one mesh with offset ids (host view)."""
    no = np.cumsum([0] + [p.num_nodes for p in problems])
    coords = np.concatenate([p.coords for p in problems])
    conn = np.concatenate([p.conn + no[g] for g, p in enumerate(problems)]).astype(np.int32)
    # the initial velocity fields, for all samples or none (a sample without
    # nodes has none to give)
    given = [p.v_init is not None for p in problems if p.num_nodes > 0]
    if any(given) and not all(given):
        raise ValueError("v_init must be given for every sample of an ensemble or for none")
    v0 = None
    if given and all(given):
        v0 = np.concatenate([p.v_init if p.num_nodes > 0 else np.zeros((0, 3)) for p in problems])
    return Problem(coords=coords, conn=conn, node_sets={}, density=problems[0].density,
                   bulk_modulus=problems[0].bulk_modulus, shear_modulus=problems[0].shear_modulus, bcs=[],
                   v_init=v0)


def device_sm_count(device=0):
    n = C.c_int(0)
    _check(library().nsm_device_sm_count(device, C.byref(n)))
    return n.value


def run(problem: Problem, final_time: float, num_steps: int, output_frequency: int = 0,
        precision: str = "fp64", with_ip=True) -> dict:
    """Whole explicit run on the device; returns the final state."""
    m = Model(problem, precision=precision)
    m.begin(final_time, num_steps, output_frequency)
    m.advance(num_steps)
    out = m.state(with_ip=with_ip)
    out["kinetic_energy"], out["internal_energy"] = m.GetEnergies()
    out["dt_crit"] = m.GetCriticalTimeStep()
    m.close()
    return out
