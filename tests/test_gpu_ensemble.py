"""Batched uncertainty-quantification ensembles: many meshes of uneven size
and per-sample moduli in one handle, each sample with its own time step.

Each sample must equal, bit for bit, the same sample run alone through the
single-mesh entry points (same kernels, same arithmetic), and hence the
oracle within the FP64 parity tolerance."""
import numpy as np
import pytest

from nimblesm_gb300 import engine as E
from nimblesm_gb300.mesh import uq_ensemble
from oracle import oracle as O
from tests.gpu_util import rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from nimblesm_gb300 import build as B
    B.build()
    O.build(ref=False)


def small_ensemble():
    return uq_ensemble(num_samples=7, n_min=2, n_max=7, seed=11)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_each_sample_equals_its_single_run(precision):
    probs = small_ensemble()
    steps, of = 60, 25
    ens = E.Model(probs, precision=precision, graph_steps=9)
    dts = ens.sample_time_steps()
    final = [steps * 0.5 * d for d in dts]
    ens.begin(final, steps, of)
    ens.advance(steps)
    st = ens.state()
    F, S = st["F"], st["sigma"]
    for g, p in enumerate(probs):
        single = E.Model(p, precision=precision)
        assert single.GetCriticalTimeStep() == dts[g]
        single.begin(final[g], steps, of)
        single.advance(steps)
        ss = single.state()
        sl = ens.sample_slice(g)
        es = slice(int(ens.elem_offsets[g]), int(ens.elem_offsets[g + 1]))
        for k in ("u", "v", "a", "f_int", "mass"):
            assert np.array_equal(st[k][sl], ss[k]), (g, k)
        assert np.array_equal(F[es], ss["F"]) and np.array_equal(S[es], ss["sigma"])
        single.close()


def test_samples_match_the_oracle():
    probs = small_ensemble()
    steps = 80
    ens = E.Model(probs)
    dts = ens.sample_time_steps()
    final = [steps * 0.5 * d for d in dts]
    ens.begin(final, steps, 0)
    ens.advance(steps)
    st = ens.state()
    for g, p in enumerate(probs):
        r = O.run_port(p, final[g], steps, 0)
        assert r["dt_crit"] == dts[g]
        sl = ens.sample_slice(g)
        assert rel(st["u"][sl], r["u"]) < 1e-10
        assert rel(st["v"][sl], r["v"]) < 1e-10
        es = slice(int(ens.elem_offsets[g]), int(ens.elem_offsets[g + 1]))
        assert rel(st["sigma"][es], r["sigma"]) < 1e-9


def test_qoi_and_autotune():
    probs = small_ensemble()
    steps = 40
    ens = E.Model(probs)
    dts = ens.sample_time_steps()
    final = [steps * 0.5 * d for d in dts]
    ens.begin(final, steps, 0)
    ens.advance(steps // 2)
    choice, ms = ens.autotune(repeats=2)
    assert 0 <= choice < len(ens.launch_candidate_times(1)) and ms > 0
    ens.advance(steps - steps // 2)
    st = ens.state()
    top = [p.node_sets["nodelist_2"] for p in probs]
    q = ens.sample_max_abs("displacement", 2, top)
    for g in range(len(probs)):
        assert q[g] == np.abs(st["u"][ens.sample_slice(g)][top[g], 2]).max()
    # the launch shape does not change the arithmetic
    ref = E.Model(probs)
    ref.begin(final, steps, 0)
    ref.advance(steps)
    assert np.array_equal(ref.state()["u"], st["u"])
