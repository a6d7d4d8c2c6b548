"""Replicas across processes (nimblesm_gb300/replicas.py and bench.py's
aggregation) on the CPU: two gloo ranks, each running and timing its own
replica of a small problem on the CPU oracle, a barrier around the timed
region, the slowest rank's time, and the whole-job throughput of weakly
scaled replicas."""
import json
import os
import socket
import sys

import numpy as np
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_dir):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import time

    import bench
    from nimblesm_gb300.mesh import cube_problem, critical_time_step
    from nimblesm_gb300.replicas import Replicas
    from oracle import oracle as O

    reps = Replicas(backend="gloo")
    # this rank's own replica: a different jitter seed per rank, nothing shared
    p = cube_problem(4, jitter=0.2, seed=10 + rank)
    dt = 0.5 * critical_time_step(p)
    reps.barrier()
    t0 = time.perf_counter()
    r = O.run_port(p, 20 * dt, 20, 0, threads=1)
    ms = 1e3 * (time.perf_counter() - t0) + 5.0 * rank  # ranks finish at different times
    reps.barrier()
    units = 8.0 * p.num_elem * 20
    out = {"rank": rank, "world": reps.world, "ms": ms, "max_ms": reps.max(ms), "sum_units": reps.sum(units),
           "value": bench.replica_value(units, ms, reps), "u_norm": float(np.linalg.norm(r["u"]))}
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump(out, f)
    reps.close()


def test_two_gloo_replicas(tmp_path):
    from oracle import oracle as O
    O.build(ref=False)
    mp.spawn(_rank, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(2)]
    units = 8.0 * 64 * 20
    for r in res:
        assert r["world"] == 2
        assert r["max_ms"] == max(x["ms"] for x in res)  # the slowest rank's time on every rank
        assert r["sum_units"] == 2 * units
        assert np.isclose(r["value"], 2 * units / (r["max_ms"] * 1e-3))
    assert res[0]["u_norm"] != res[1]["u_norm"]  # independent replicas


def test_single_process_needs_no_collective():
    sys.path.insert(0, ROOT)
    import bench
    from nimblesm_gb300.replicas import Replicas
    env = {k: os.environ.pop(k) for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK") if k in os.environ}
    try:
        reps = Replicas()
        assert reps.world == 1 and reps.backend is None and reps.device == 0
        assert reps.max(3.0) == 3.0 and reps.sum(3.0) == 3.0
        assert bench.replica_value(1000.0, 2.0, reps) == 1000.0 / 2e-3
        reps.barrier()
        reps.close()
    finally:
        os.environ.update(env)
