"""Boundary-condition expressions f(x, y, z, t) (nimblesm_gb300/csrc/
bc_expression.cu, nsm_add_boundary_condition_expression): the engine's parser
against the reference's own ExpressionParsing (values it computed, committed
in tests/golden/ref_bc_expressions.npz by tests/golden/make_golden.py), and a
run driven only by expression conditions against the reference's run of the
same deck (tests/golden/ref_bc_expression_cube6.npz)."""
import numpy as np
import pytest

from nimblesm_gb300 import engine as E
from nimblesm_gb300.mesh import BoundaryCondition, cube_problem, critical_time_step
from tests.goldens import load, output_steps
from tests.gpu_util import rel

FUNCTIONS = ("sin", "cos", "tan", "erf", "exp", "log", "abs", "asin", "acos", "atan", "sqrt", "cbrt", "ceil",
             "round", "floor", "^", "%")


@pytest.fixture(scope="module", autouse=True)
def _built():
    from nimblesm_gb300 import build as B
    B.build()


def test_parser_matches_the_reference_parser():
    """The host evaluation of each compiled expression (the device's operation
    order, the host's math library) equals the reference parser's value:
    bit for bit where only + - * / and comparisons are involved, within 4 ulp
    where a math-library function is (the reference values were made on
    x86-64; another host's libm may round those differently)."""
    fx = load("ref_bc_expressions")
    for e, row in zip(fx["expressions"], fx["values"]):
        e = str(e)
        for pt, ref in zip(fx["points"], row):
            ours = E.bc_expression_eval(e, *pt)
            if any(f in e.lower() for f in FUNCTIONS):
                assert abs(ours - ref) <= 4 * np.spacing(abs(ref)), (e, pt, ours, ref)
            else:
                assert ours == ref, (e, pt, ours, ref)


def test_parser_refuses_what_the_reference_refuses():
    fx = load("ref_bc_expressions")
    for e in fx["bad"]:
        with pytest.raises(E.EngineError):
            E.bc_expression_eval(str(e), 0.3, 0.7, 0.25, 1.0e-6)


def test_deck_lines_with_expressions_round_trip():
    fx = load("ref_bc_expression_cube6")
    for line in fx["bc_lines"]:
        b = BoundaryCondition.parse(str(line))
        assert b.expression is not None and b.line() == str(line)
        assert BoundaryCondition.parse(b.line()) == b
    with pytest.raises(ValueError):
        BoundaryCondition.parse('prescribed_velocity nodelist_1 x "t')
    with pytest.raises(ValueError):  # the port oracle takes constant magnitudes only
        p = cube_problem(2)
        p.bcs = [BoundaryCondition.parse(str(fx["bc_lines"][0]))]
        p.bc_arrays()


@pytest.mark.gpu
def test_expression_run_against_the_reference():
    """u and v at every output step, F and sigma at the last, within 1e-10 of
    the reference's run (the device evaluates sin etc. with CUDA's
    double-precision functions, which may differ from the host's by an ulp)."""
    fx = load("ref_bc_expression_cube6")
    p = cube_problem(6, jitter=0.2, seed=3)
    p.v_init = None
    p.bcs = [BoundaryCondition.parse(str(line)) for line in fx["bc_lines"]]
    steps, of = int(fx["steps"]), int(fx["output_frequency"])
    assert np.isclose(float(fx["final_time"]), steps * 0.5 * critical_time_step(p), rtol=1e-15)
    outs = output_steps(steps, of)  # after steps 1, 51, ..., 300
    assert len(outs) == fx["u"].shape[0]
    m = E.Model(p)
    m.begin(float(fx["final_time"]), steps, of)
    done = 0
    for t, s in enumerate(outs):
        m.advance(s - done)
        done = s
        st = m.state(with_ip=(t == len(outs) - 1))
        assert rel(st["u"], fx["u"][t]) <= 1e-10, (t, rel(st["u"], fx["u"][t]))
        assert rel(st["v"], fx["v"][t]) <= 1e-10, (t, rel(st["v"], fx["v"][t]))
    assert rel(st["F"], fx["F"]) <= 1e-10 and rel(st["sigma"], fx["sigma"]) <= 1e-10
    m.close()


def _random_expression(rng, depth=0):
    """A random expression of the reference's grammar: numbers (plain,
    decimal, exponent forms), x y z t, e pi tau, + - * / % ^, unary minus,
    parentheses, the math functions, and conditions under "? :"."""
    leaves = ["x", "y", "z", "t", "e", "pi", "tau", "2", "0.5", "3.25", "1e-3", "2.5e2", "7"]
    if depth > 3 or rng.random() < 0.25:
        return str(rng.choice(leaves))
    k = rng.integers(0, 10)
    a = _random_expression(rng, depth + 1)
    if k <= 4:
        op = str(rng.choice(["+", "-", "*", "/", "%"]))
        return f"{a} {op} {_random_expression(rng, depth + 1)}"
    if k == 5:
        return f"({a})"
    if k == 6:
        return f"-({a})"
    if k == 7:
        f = str(rng.choice(["sin", "cos", "exp", "abs", "atan", "sqrt", "floor", "ceil", "round", "cbrt", "erf"]))
        return f"{f}({a})"
    if k == 8:
        return f"({a})^{rng.choice(['2', '3', '0.5', '-1'])}"
    cmp = str(rng.choice([">", "<", ">=", "<="]))
    return f"{a} {cmp} {_random_expression(rng, depth + 1)} ? {_random_expression(rng, depth + 1)} : {a}"


def test_random_expressions_against_the_reference_parser():
    """400 seeded random expressions at 3 points: the engine's host
    evaluation equals the reference parser's value bit for bit (NaN for NaN),
    or both refuse the text.  Needs the reference built from its sources
    (oracle/_ref), so it runs where those sources are."""
    from oracle import oracle as O
    if not O.reference_available():
        pytest.skip("the reference library is not built here")
    rng = np.random.default_rng(2024)
    pts = [(0.3, 0.7, 0.25, 1.0e-6), (0.75, 0.2, 0.5, 5.0e-6), (1.0, 0.0, 0.125, 0.0)]
    checked = 0
    for _ in range(400):
        text = _random_expression(rng)
        for pt in pts:
            try:
                ref = O.ref_eval_expression(text, *pt)
            except ValueError:
                ref = None
            try:
                ours = E.bc_expression_eval(text, *pt)
            except E.EngineError:
                ours = None
            assert (ref is None) == (ours is None), (text, ref, ours)
            if ref is not None:
                assert ours == ref or (np.isnan(ours) and np.isnan(ref)), (text, pt, ours, ref)
                checked += 1
    assert checked > 900  # most of them parse
