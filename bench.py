#!/usr/bin/env python3
"""Benchmark: hex8 integration-point stress updates per second of the
explicit neo-Hookean step on a jittered 128^3 cube (2,097,152 elements,
2,146,689 nodes, 8 Gauss points per element), FP64 plain form.

A step is one central-difference step of the whole mesh: element kernel
(gather, F, stress, B^T sigma) plus node kernel (assembly gather, a = f/m,
velocity/displacement update, boundary conditions).  value = 8 E K / device
time of K steps, with the state resident in HBM.  The FP32-mixed form is
measured on the same mesh and reported under "variants" with its error
against the FP64 form.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU implementation of the same step on this
machine's host cores (the oracle's C restatement of the reference; see
oracle/), the only place besides the cpu_baseline leg where bench.py runs it.
"""
from __future__ import annotations

import argparse
import json
import os
import signal
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from nimblesm_gb300.mesh import cube_problem, critical_time_step, uq_ensemble  # noqa: E402

PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0
METRIC = "hex8 IP stress updates/sec, plain FP64 vs mixed/MLP at <=1e-3 rel. disp error"
UNIT = "IP-updates/s"
SCHEDULE_STEPS = 2000  # the workload's schedule: dt = 0.5 dt_crit, 2000 steps
UQ_SCHEDULE_STEPS = 1000  # the ensemble's schedule: 1000 steps per sample
# FP64 work per integration point of the FP64 element kernel's formulation:
# 87.9 DFMA (2 flops each) + 44.5 DADD + 37.9 DMUL executed per point (counted
# by ncu on the 64^3 case).  The FP64 pipe issues 2 of these instructions per
# SM per cycle, whatever their kind.
FP64_FLOPS_PER_IP = 258.1
FP64_INSTR_PER_IP = 170.2
# DRAM bytes (read + write) of one element launch on the 128^3 cube, from one
# ncu capture per form.
ELEMENT_TRAFFIC_128 = {"fp64": 2.696480768e9 + 2.657063168e9, "fp32": 0.119112960e9 + 1.213583360e9}


def algorithmic_bytes(N, E, precision):
    """Bytes each step moves once in the reference's field layout (the
    ModelData contract after every step): nodes read X, u, v, a, m and write
    u, v, a, f_int (200 B/node; this engine keeps a and f_int in registers
    between the steps of one advance and writes them at its end);
    elements read connectivity and write F and sigma per integration point
    (992 B/element in FP64, 512 B in FP32).  The element kernel's share is
    connectivity, F, sigma and the gathered X and u (48 B/node)."""
    ip = 8 * (9 + 6) * (8 if precision == "fp64" else 4)
    step = 200 * N + (32 + ip) * E
    element = (32 + ip) * E + 48 * N
    return step, element


# Algorithmic work of one training pair in one epoch: the forward pass
# (9*64 + 64*64 + 64*6 = 5,056 multiply-adds), the weight gradients (the same
# 5,056) and the input gradients of layers 3 and 2 (64*6 + 64*64 = 4,480; layer
# 1's input gradient is not needed): 14,592 multiply-adds, 2 flops each.
TRAIN_FLOPS_PER_PAIR = 2 * (5056 + 5056 + 4480)
# Optimizer batch: 152 tiles of 128 pairs, one tile per SM of the GPU, with a
# learning rate of 2e-2 (cosine-decayed): measured against 16 tiles at 5e-3,
# the same 20 epochs reach a stress error of 1.6e-3 against 1.4e-3 on the
# training distribution in 0.72 s instead of 5.7 s.
TRAIN_BATCH_TILES = 152
TRAIN_LR = 2e-2


def bf16_peak():
    """Dense BF16 tensor peak (TFLOP/s), the measured burst figure."""
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["bf16_tflops"]), "measured"
    except Exception:
        return 1900.0, "fallback"


def hbm_peak():
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        self.proc = None
        self.device = device

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.send_signal(signal.SIGTERM)
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            # a region shorter than the sampler's start-up: one sample at its end
            try:
                if not open(self.path).read().strip():
                    with open(self.path, "w") as f:
                        subprocess.run(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                        "--format=csv,noheader,nounits"], stdout=f, stderr=subprocess.DEVNULL,
                                       timeout=10)
            except Exception:
                pass

    def summary(self):
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
            os.unlink(self.path)
        except Exception:
            return None
        if not rows:
            return None
        sm = [float(r[1]) for r in rows]
        mx = float(rows[0][2])
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.strip() == "Active"})
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": reasons, "samples": len(rows)}


def workload_config(n, problem, ws):
    """The workload's description, the same dict in both arms."""
    return {"workload": f"hex8 neo-Hookean explicit step, jittered {n}^3 cube (±20% interior jitter), "
                        f"dt = 0.5 dt_crit, {SCHEDULE_STEPS}-step schedule",
            "elements": problem.num_elem, "nodes": problem.num_nodes, "parallelism": f"replicas{ws}",
            "l2": "inputs larger than L2 (per-step traffic >> 129 MB)"}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def replica_value(units_per_rank, ms_per_rank, reps):
    """Whole-job throughput of weak-scaled replicas: the units all ranks
    processed over the slowest rank's time (ms)."""
    return reps.sum(units_per_rank) / (reps.max(ms_per_rank) * 1e-3)


def cpu_baseline(problem, dt, seconds_budget=15.0, threads=None, max_steps=40):
    """The oracle (C restatement of the reference's host path, whose gather
    assembly is the reference's serial order at any thread count) on all host
    cores, or on the given number of threads, from the workload's initial
    state, on a bounded number of steps."""
    from oracle import oracle

    oracle.build(ref=False)
    threads = threads or os.cpu_count()
    u = np.zeros_like(problem.coords)
    v = problem.v_init.copy()
    v[problem.node_sets["nodelist_1"]] = 0.0
    a = np.zeros_like(u)
    t1 = oracle.continue_port(problem, u, v, a, 0.0, dt, 1, threads)  # includes first-touch
    k = int(max(1, min(max_steps, seconds_budget / max(t1, 1e-3))))
    secs = oracle.continue_port(problem, u, v, a, dt, dt, k, threads)
    return {"value": 8.0 * problem.num_elem * k / secs, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{k} steps of the same {round(problem.num_elem ** (1 / 3))}^3 mesh from its initial state "
                      f"({secs:.1f} s)"}


def run_reference(args):
    """--impl reference: the CPU implementation of the step, all host cores."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import oracle

    oracle.build(ref=False)
    n = args.n
    problem = cube_problem(n, jitter=0.2, seed=0)
    dt = 0.5 * critical_time_step(problem)
    threads = os.cpu_count()
    u = np.zeros_like(problem.coords)
    v = problem.v_init.copy()
    v[problem.node_sets["nodelist_1"]] = 0.0
    a = np.zeros_like(u)
    t = 0.0
    for _ in range(max(args.warmup, 1) if args.warmup < 3 else 3):
        oracle.continue_port(problem, u, v, a, t, dt, 1, threads)
        t += dt
    est = oracle.continue_port(problem, u, v, a, t, dt, 1, threads)
    t += dt
    # each step is one full explicit step of the mesh; the count is capped so
    # that the run ends within a few minutes
    steps = int(min(args.steps, max(1, 120.0 / max(est, 1e-3))))
    secs = oracle.continue_port(problem, u, v, a, t, dt, steps, threads)
    value = 8.0 * problem.num_elem * steps / secs
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * secs / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(n, problem, ws), "steps_requested": args.steps,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{steps} full steps of the {n}^3 mesh"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def uq_variants(E, args, device):
    """Ensemble workload: 512 jittered cubes with n ~ U{8..48} and log-normal moduli in
    one handle (one launch per phase for all samples), each sample with its
    own time step, CUDA graphs of 100 steps; launch shape by the autotuner.
    Throughput over `uq_steps` timed steps; then the rest of the 1000-step
    schedule runs untimed and the QoI per sample (max |u_z| on its z = L face)
    is taken after the last step, in both precisions, with the FP32-mixed
    form's QoI error against the FP64 form's."""
    probs = uq_ensemble(num_samples=args.uq_samples, seed=0)
    E_tot = sum(p.num_elem for p in probs)
    out, qois = {}, {}
    schedule = max(UQ_SCHEDULE_STEPS, args.uq_steps + 200)
    for precision in ("fp64", "fp32"):
        m = E.Model(probs, precision=precision, graph_steps=100, device=device)
        dts = m.sample_time_steps()
        m.begin([schedule * 0.5 * d for d in dts], schedule, schedule)
        choice, tune_ms = m.autotune(repeats=3)
        m.advance(100)  # warm-up chunk (graph capture)
        m.synchronize()
        with ClockSampler(device) as clk:
            ms = m.advance_timed(args.uq_steps)
        t0 = time.perf_counter()
        m.advance(schedule - 100 - args.uq_steps)
        m.synchronize()
        rest_s = time.perf_counter() - t0
        top = [p.node_sets["nodelist_2"] for p in probs]
        q = m.sample_max_abs("displacement", 2, top)
        qois[precision] = q
        out[f"uq_ensemble_{precision}"] = {
            "value": 8.0 * E_tot * args.uq_steps / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms / args.uq_steps,
            "samples": len(probs), "elements": E_tot, "nodes": int(sum(p.num_nodes for p in probs)),
            "steps_timed": args.uq_steps, "after_steps": schedule, "graph_steps": 100,
            "autotune_choice": choice, "element_launch_ms_tuned": tune_ms, "untimed_wall_s": rest_s,
            "qoi_max_abs_uz": {"min": float(q.min()), "mean": float(q.mean()), "max": float(q.max())},
            "clocks": clk.summary()}
        m.close()
    d = np.abs(qois["fp32"] - qois["fp64"]) / np.abs(qois["fp64"])
    out["uq_ensemble_fp32"]["qoi_rel_err_vs_fp64"] = {"max": float(d.max()), "mean": float(d.mean())}
    return out


def uq_closure_variant(E, args, problem, device):
    """The reference's UQ mode on the 128^3 mesh in one handle: the nominal
    trajectory, 2 exact samples (element forces with their own bulk and
    shear moduli, +-5% of the nominal's) and 8 approximate samples whose force
    is the linear closure c0 f_nominal + sum_k c_k f_exact_k.  One element
    launch covers the nominal's and the exact samples' elements; the closure
    is formed inside the node launch.  Sample values and closure coefficients
    are synthetic (seeded).  value counts the element work (integration-point
    updates of the nominal and exact trajectories)."""
    from nimblesm_gb300.uq import UqSpec
    rng = np.random.default_rng(5)
    n_exact, n_approx = 2, 8
    params = [(0, "bulk_modulus", 0.1 * problem.bulk_modulus), (0, "shear_modulus", 0.1 * problem.shear_modulus)]
    exact = np.array([[-0.5, 0.5], [0.5, -0.5]])
    approx = rng.uniform(-0.5, 0.5, (n_approx, 2))
    w = rng.uniform(0.0, 0.5, (n_approx, n_exact))
    coef = np.concatenate([1.0 - w.sum(axis=1, keepdims=True), w], axis=1)
    spec = UqSpec(params, exact, approx, coef)
    dt = 0.5 * critical_time_step(problem)
    steps = args.uq_closure_steps
    m = E.UqModel(problem, spec, device=device)
    m.begin(SCHEDULE_STEPS * dt, SCHEDULE_STEPS, SCHEDULE_STEPS)
    m.advance(3)
    m.synchronize()
    with ClockSampler(device) as clk:
        ms = m.advance_timed(steps)
    S = 1 + n_exact + n_approx
    res = {"uq_closure": {
        "value": 8.0 * problem.num_elem * (1 + n_exact) * steps / (ms * 1e-3), "unit": UNIT,
        "ms_per_step": ms / steps, "trajectories": S, "exact_samples": n_exact, "approximate_samples": n_approx,
        "trajectory_steps_per_s": S * steps / (ms * 1e-3), "elements_per_trajectory": problem.num_elem,
        "steps_timed": steps, "after_steps": 3 + steps, "clocks": clk.summary()}}
    m.close()
    return res


def big_fp32_variant(E, args, device):
    """The FP32-mixed form on a 256^3 jittered cube (16.8M elements): its
    throughput over `big_steps` timed steps, and its displacement, velocity and
    energy-drift error against the FP64 form on the same mesh after the whole
    2000-step schedule (the steps past the timed ones run untimed)."""
    n = args.big_n
    prob = cube_problem(n, jitter=0.2, seed=0)
    dt = 0.5 * critical_time_step(prob)
    steps = args.big_steps
    total = max(SCHEDULE_STEPS if args.big_full else 3 + steps, 3 + steps)
    out, st = {}, {}
    for precision in ("fp32", "fp64"):
        m = E.Model(prob, precision=precision, device=device, graph_steps=100)
        m.begin(SCHEDULE_STEPS * dt, SCHEDULE_STEPS, SCHEDULE_STEPS)
        m.advance(1)
        e0 = sum(m.GetEnergies())
        m.advance(2)
        m.synchronize()
        ms = m.advance_timed(steps)
        out[precision] = 8.0 * prob.num_elem * steps / (ms * 1e-3)
        t0 = time.perf_counter()
        m.advance(total - 3 - steps)
        m.synchronize()
        ke, ie = m.GetEnergies()
        st[precision] = dict(u=m.GetVectorNodeData("displacement"), v=m.GetVectorNodeData("velocity"),
                             drift=(ke + ie - e0) / e0, rest_s=time.perf_counter() - t0)
        m.close()
    a, b = st["fp32"], st["fp64"]
    rel = lambda x, y: float(np.linalg.norm(x - y) / np.linalg.norm(y))
    return {f"fp32_{n}cube": {"value": out["fp32"], "unit": UNIT, "elements": prob.num_elem, "steps_timed": steps,
                              "fp64_value": out["fp64"], "speedup_vs_fp64": out["fp32"] / out["fp64"],
                              "rel_disp_err_vs_fp64": rel(a["u"], b["u"]), "rel_vel_err_vs_fp64": rel(a["v"], b["v"]),
                              "energy_drift": a["drift"], "energy_drift_fp64": b["drift"], "after_steps": total,
                              "untimed_wall_s": {"fp32": a["rest_s"], "fp64": b["rest_s"]}}}


def mlp_variant(E, args, problem, device, fp64_value, fp32_value):
    """The learned closure: generated and trained on the GPU (tensor-core
    forward/backward), then fused into the element kernel of the 128^3 run.
    Errors against the FP64 plain form at the same step; speedups against the
    FP64 and FP32 plain forms."""
    t0 = time.perf_counter()
    mlp = E.MLPClosure(problem.bulk_modulus, problem.shear_modulus, seed=1, device=device)
    mlp.generate(args.mlp_pairs, seed=7, perturbation=0.05, min_det=0.5)
    t1 = time.perf_counter()
    loss = mlp.train(epochs=args.mlp_epochs, batch_tiles=TRAIN_BATCH_TILES, lr=TRAIN_LR)
    t2 = time.perf_counter()
    dt = 0.5 * critical_time_step(problem)
    steps = args.mlp_steps
    res = {}
    for form in ("mlp", "fp64"):
        m = E.Model(problem, precision="fp32" if form == "mlp" else "fp64", device=device)
        if form == "mlp":
            m.set_closure(mlp)
        m.begin(SCHEDULE_STEPS * dt, SCHEDULE_STEPS, SCHEDULE_STEPS)
        m.advance(1)
        e0 = sum(m.GetEnergies())
        m.synchronize()
        if form == "mlp":
            m.set_profiling(True)
            m.advance(2)
            prof = m.get_profile()
            m.set_profiling(False)
            ms = m.advance_timed(steps - 3)
        else:
            m.advance(steps - 1)
            ms = None
        ke, ie = m.GetEnergies()
        F, sig = m.GetIntegrationPointData()
        res[form] = dict(u=m.GetVectorNodeData("displacement"), sig=sig, drift=(ke + ie - e0) / e0, ms=ms,
                         fallbacks=m.closure_fallbacks(), prof=prof if form == "mlp" else None)
        m.close()
    a, b = res["mlp"], res["fp64"]
    value = 8.0 * problem.num_elem * (steps - 3) / (a["ms"] * 1e-3)
    return {"mlp_closure": {
        "value": value, "unit": UNIT, "ms_per_step": a["ms"] / (steps - 3),
        "element_launch_ms": a["prof"]["element_ms"] / max(a["prof"]["element_launches"], 1),
        "speedup_vs_fp64": value / fp64_value, "speedup_vs_fp32": value / fp32_value,
        "rel_disp_err_vs_fp64": float(np.linalg.norm(a["u"] - b["u"]) / np.linalg.norm(b["u"])),
        "rel_stress_err_vs_fp64": float(np.linalg.norm(a["sig"] - b["sig"]) / np.linalg.norm(b["sig"])),
        "energy_drift": a["drift"], "energy_drift_fp64": b["drift"], "after_steps": steps,
        "envelope_fallbacks": a["fallbacks"], "training_pairs": args.mlp_pairs, "epochs": args.mlp_epochs,
        "final_loss": loss, "generate_s": t1 - t0, "train_s": t2 - t1,
        "train_batch_pairs": 128 * TRAIN_BATCH_TILES, "train_lr": TRAIN_LR,
        "train_tflops": args.mlp_pairs * args.mlp_epochs * TRAIN_FLOPS_PER_PAIR / (t2 - t1) / 1e12,
        "train_tensor_frac": args.mlp_pairs * args.mlp_epochs * TRAIN_FLOPS_PER_PAIR / (t2 - t1) / 1e12
        / bf16_peak()[0], "train_flops_per_pair_epoch": TRAIN_FLOPS_PER_PAIR,
        "train_peak_source": bf16_peak()[1],
        "network": "9-64-64-6 GELU, BF16 weights/activations, FP32 accumulate, tcgen05; second-order neo-Hookean base, cubic gate"}}, mlp


def accuracy_variant(E, args, problem, device, mlp):
    """The workload's full schedule (2000 steps at dt = 0.5 dt_crit) in the
    FP64, FP32-mixed and learned-closure forms from the same initial state:
    each form's displacement and velocity error against the FP64 form after
    the last step (CUDA graphs of 100 steps; not part of the timed value)."""
    dt = 0.5 * critical_time_step(problem)
    steps = args.acc_steps
    out, ref = {}, None
    forms = ("fp64", "fp32") + (("mlp",) if mlp is not None else ())
    for form in forms:
        m = E.Model(problem, precision="fp64" if form == "fp64" else "fp32", device=device, graph_steps=100)
        if form == "mlp":
            m.set_closure(mlp)
        m.begin(steps * dt, steps, steps)
        t0 = time.perf_counter()
        m.advance(1)
        e0 = sum(m.GetEnergies())
        m.advance(steps - 1)
        m.synchronize()
        wall = time.perf_counter() - t0
        ke, ie = m.GetEnergies()
        st = dict(u=m.GetVectorNodeData("displacement"), v=m.GetVectorNodeData("velocity"),
                  drift=(ke + ie - e0) / e0, wall=wall,
                  fallbacks=m.closure_fallbacks() if form == "mlp" else 0)
        m.close()
        if form == "fp64":
            ref = st
            out["fp64"] = {"energy_drift": st["drift"], "wall_s": wall}
            continue
        out[form] = {"rel_disp_err_vs_fp64": float(np.linalg.norm(st["u"] - ref["u"]) / np.linalg.norm(ref["u"])),
                     "rel_vel_err_vs_fp64": float(np.linalg.norm(st["v"] - ref["v"]) / np.linalg.norm(ref["v"])),
                     "energy_drift": st["drift"], "wall_s": wall}
        if form == "mlp":
            out[form]["envelope_fallbacks"] = st["fallbacks"]
    return {f"accuracy_{steps}_steps": {"steps": steps, "mesh": f"{round(problem.num_elem ** (1 / 3))}^3",
                                          "forms": out, "bound": 1e-3}}


def run_ours(args):
    from nimblesm_gb300 import engine as E

    from nimblesm_gb300.replicas import Replicas

    reps = Replicas()
    ws, rank, local = reps.world, reps.rank, reps.device
    if ws > 1:
        # a scaling run measures the workload on every GPU; the variants are
        # single-GPU measurements and would only hold the GPUs longer
        args.variants = False

    n = args.n
    problem = cube_problem(n, jitter=0.2, seed=0)
    N, E_ = problem.num_nodes, problem.num_elem
    dt_crit = critical_time_step(problem)
    dt = 0.5 * dt_crit
    final_time = SCHEDULE_STEPS * dt
    sched = max(SCHEDULE_STEPS, args.warmup + 2 * args.steps + 1)
    final_time = sched * dt

    barrier, max_over_ranks = reps.barrier, reps.max

    results = {}
    for precision in ([args.precision] + ([p for p in ("fp64", "fp32") if p != args.precision]
                                          if args.variants else [])):
        m = E.Model(problem, precision=precision, device=local)
        m.begin(final_time, sched, sched)
        m.advance(args.warmup)
        m.synchronize()
        barrier()
        with ClockSampler(local) as clk:
            ms_rank = m.advance_timed(args.steps)
        barrier()
        value_p = replica_value(8.0 * E_ * args.steps, ms_rank, reps)
        ms = max_over_ranks(ms_rank)
        # per-kernel device times over the same number of steps (events on the
        # engine's stream around every element and node launch)
        m.set_profiling(True)
        m.advance(args.steps)
        prof = m.get_profile()
        m.set_profiling(False)
        state_u = m.GetVectorNodeData("displacement")
        results[precision] = dict(ms=ms, value=value_p, prof=prof, clocks=clk.summary(),
                                  launches=m.launches_per_advance(args.steps), u=state_u, model=m)
        if precision != args.precision:
            m.close()

    head = results[args.precision]
    m = head["model"]
    ms = head["ms"]
    value = head["value"]

    # end to end through the drop-in host-buffer entry point: each step copies
    # the displacement in from pinned host memory and the internal force out
    e2e_steps = max(3, min(args.steps, 30))
    u_host = E.PinnedArray((N, 3))
    f_host = E.PinnedArray((N, 3))
    u_host.array[:] = head["u"]
    m.ComputeInternalForceHost(u_host.array, f_host.array)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        m.ComputeInternalForceHost(u_host.array, f_host.array)
    t1 = time.perf_counter()
    barrier()
    e2e_value = replica_value(8.0 * E_ * e2e_steps, 1e3 * (t1 - t0), reps)

    # the whole drop-in step: the reference integrator's loop on host arrays
    # (its O(N) velocity / displacement / acceleration updates and kinematic
    # conditions on one host thread, as ExplicitTimeIntegrator runs them
    # through a GpuModelData) around the same host-buffer force call
    hl = {k: E.PinnedArray((N, 3)) for k in ("v", "a")}
    hl["v"].array[:] = m.GetVectorNodeData("velocity")
    hl["a"].array[:] = m.GetVectorNodeData("acceleration")
    mass = m.ComputeLumpedMass()
    t_now = m.progress()[1]
    t_now, _ = m.HostLoopSteps(1, t_now, dt, mass, u_host.array, hl["v"].array, hl["a"].array, f_host.array)
    barrier()
    t0 = time.perf_counter()
    t_now, host_s = m.HostLoopSteps(e2e_steps, t_now, dt, mass, u_host.array, hl["v"].array, hl["a"].array,
                                    f_host.array)
    t1 = time.perf_counter()
    barrier()
    e2e_step_value = replica_value(8.0 * E_ * e2e_steps, 1e3 * (t1 - t0), reps)
    e2e_step = {"value": e2e_step_value, "unit": UNIT, "h2d_bytes_per_step": 24 * N, "d2h_bytes_per_step": 24 * N,
                "ms_per_step": 1e3 * (t1 - t0) / e2e_steps, "host_loop_ms_per_step": 1e3 * host_s / e2e_steps,
                "host_loop_share": host_s / (t1 - t0), "steps": e2e_steps,
                "path": "nsm_host_loop_steps: the reference loop's host-side updates (one thread, pinned [N][3] "
                        "u, v, a, f_int) + nsm_compute_internal_force_host per step"}

    step_bytes, elem_bytes = algorithmic_bytes(N, E_, args.precision)
    peak, peak_kind = hbm_peak()
    elem_ms = head["prof"]["element_ms"] / max(head["prof"]["element_launches"], 1)
    node_ms = head["prof"]["node_ms"] / max(head["prof"]["node_launches"], 1)
    achieved = elem_bytes / (elem_ms * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64",
        "data": "synthetic",
        "config": workload_config(n, problem, ws),
        "form": args.precision, "ips_per_step": 8 * E_, "dt": dt, "schedule_steps": sched,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 24 * N, "d2h_bytes_per_step": 24 * N,
                "path": "nsm_compute_internal_force_host only (pinned u in, f_int out); the nodal updates of the "
                        "step are not in it (see e2e_step)", "steps": e2e_steps,
                "host_chunks": m.host_chunks()},
        "e2e_step": e2e_step,
        "gpu_launches": head["launches"],
        "clocks": head["clocks"],
    }
    hbm_roof = {"bound": "hbm", "kernel": "k_element<double>" if args.precision == "fp64" else "k_element_staged",
                "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": peak_kind,
                "traffic": ELEMENT_TRAFFIC_128.get(args.precision) if n == 128 else None,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, one 128^3 launch"
                if n == 128 else None,
                "algorithmic_bytes_per_launch": elem_bytes, "launch_ms": elem_ms, "node_launch_ms": node_ms,
                "step_algorithmic_bytes": step_bytes}
    if args.precision == "fp64":
        # The FP64 element kernel is bound by the FP64 pipe, not by HBM: its
        # roofline is the pipe's rate, 2 FP64 instructions (a DFMA counting 2
        # flops) per SM per cycle at the maximum SM clock.  MEASURED_PEAKS.json
        # holds no FP64 figure, so the peak is that nominal rate.  The HBM
        # fraction of the same launch is reported beside it (roofline_hbm).
        sms = E.device_sm_count(local)
        max_mhz = (head["clocks"] or {}).get("sm_max_mhz") or 2070.0
        nominal = 2 * 2 * sms * max_mhz * 1e6 / 1e12
        ach64 = FP64_FLOPS_PER_IP * 8 * E_ / (elem_ms * 1e-3) / 1e12
        instr_rate = FP64_INSTR_PER_IP * 8 * E_ / (elem_ms * 1e-3)
        pipe_rate = 2 * sms * max_mhz * 1e6
        line["roofline"] = {"bound": "fp64", "kernel": "k_element<double>", "achieved": ach64, "peak": nominal,
                            "unit": "TFLOP/s", "frac": ach64 / nominal,
                            "peak_source": f"nominal FP64 pipe: 2 DFMA per SM per cycle x {sms} SMs x {max_mhz:.0f} MHz",
                            "traffic": hbm_roof["traffic"], "traffic_source": hbm_roof["traffic_source"],
                            "launch_ms": elem_ms, "flops_per_ip": FP64_FLOPS_PER_IP,
                            "fp64_instructions_per_ip": FP64_INSTR_PER_IP,
                            "pipe_instruction_frac": instr_rate / pipe_rate,
                            "flops_source": "executed DFMA/DADD/DMUL per point, ncu (FMA = 2 flops)",
                            "hbm_frac": hbm_roof["frac"]}
        line["roofline_hbm"] = hbm_roof
    else:
        line["roofline"] = hbm_roof
    variants = {}
    for prec, r in results.items():
        if prec == args.precision:
            continue
        v = r["value"]
        err = float(np.linalg.norm(r["u"] - head["u"]) / max(np.linalg.norm(head["u"]), 1e-300))
        variants[prec] = {"value": v, "ms_per_step": r["ms"] / args.steps, "speedup_vs_fp64": v / value,
                          "rel_disp_err_vs_fp64": err, "after_steps": args.warmup + args.steps,
                          "element_launch_ms": r["prof"]["element_ms"] / max(r["prof"]["element_launches"], 1),
                          "clocks": r["clocks"]}
    if args.variants and args.uq_steps > 0:
        variants.update(uq_variants(E, args, local))
    if args.variants and args.big_steps > 0:
        variants.update(big_fp32_variant(E, args, local))
    if args.variants and args.uq_closure_steps > 0:
        variants.update(uq_closure_variant(E, args, problem, local))
    mlp = None
    if args.variants and args.mlp_steps > 0:
        fp32_value = variants.get("fp32", {}).get("value", float("nan"))
        res, mlp = mlp_variant(E, args, problem, local, value / ws, fp32_value / ws)
        variants.update(res)
    if args.variants and args.acc_steps > 0:
        variants.update(accuracy_variant(E, args, problem, local, mlp))
    if mlp is not None:
        mlp.close()
    if variants:
        line["variants"] = variants
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(problem, dt)
        line["cpu_baseline"]["single_core"] = cpu_baseline(problem, dt, seconds_budget=8.0, threads=1, max_steps=4)
    m.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    reps.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--n", type=int, default=128, help="cube divisions (default 128: 2,097,152 elements)")
    ap.add_argument("--precision", choices=("fp64", "fp32"), default="fp64")
    ap.add_argument("--no-variants", dest="variants", action="store_false",
                    help="only the headline form (no FP32, ensemble, 256^3, closure or accuracy runs)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--uq-steps", type=int, default=100, help="timed steps of the 512-sample ensemble (0: skip)")
    ap.add_argument("--uq-samples", type=int, default=512)
    ap.add_argument("--uq-closure-steps", type=int, default=20,
                    help="timed steps of the reference-style UQ mode on the main mesh (0: skip)")
    ap.add_argument("--big-n", type=int, default=256, help="cube divisions of the large FP32-mixed variant")
    ap.add_argument("--big-steps", type=int, default=20, help="timed steps of the large variant (0: skip)")
    ap.add_argument("--no-big-full", dest="big_full", action="store_false",
                    help="compare the large variant's forms after the timed steps, not after the whole schedule")
    ap.add_argument("--mlp-steps", type=int, default=103, help="steps of the learned-closure run (0: skip)")
    ap.add_argument("--mlp-pairs", type=int, default=20_000_000,
                    help="training pairs of the learned closure (the workload's 20M)")
    ap.add_argument("--acc-steps", type=int, default=SCHEDULE_STEPS,
                    help="steps of the FP64 / FP32 / closure accuracy run (0: skip)")
    ap.add_argument("--mlp-epochs", type=int, default=20)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
