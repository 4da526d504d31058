"""Step-direction and step parity of the GPU path (rs_flow_direction / rs_flow_step through the
C ABI) against the FP64 oracle and the reference's golden vectors.

* ``saddle`` fixtures (lean/oracle/fixtures/rs, replayed by RS/tests/gmres.rs:651-763 and
  RS/tests/oracle.rs:377-420): with the exact energy (theta = 0) and the exact metric (chi = 0)
  the GPU's direction x and differential g equal the fixture's within 1e-5 normwise. Cases with
  pinned vertices are left out: the GPU path holds barycenters, area and volume only.
* The same direction against the oracle's hierarchical solve on the same face tree, block
  cluster tree and Barnes-Hut lists (chi = 0.5, theta = 0.25 and 0): c1, a 48 x 24 torus and
  the fixture meshes; energy within 1e-6, g and x within 1e-5 normwise.
* ``step`` fixtures (RS/tests/oracle.rs:557-668): one step with the fixture's start rule, Armijo
  constant, halving cap and Newton rule; F, <g, x>, tau0, every trial's step size and outcome
  (Armijo margins below 1e-5 excepted: the GPU energies carry FP32 pair rounding; rejected
  trials' energies within 1e-5, accepted ones within 1e-6), the result,
  the Newton rounds, Phi and the final positions.
"""
import numpy as np
import pytest

import golden_io as G
import rs_oracle as O
import rs_gb300 as R
from rs_gb300 import generators as gen

pytestmark = pytest.mark.gpu

ENERGY_TOL = 1e-6
DIR_TOL = 1e-5
GPU_SADDLE = ["rs-icosa-saddle", "rs-mobius-saddle", "rs-octa-saddle-none", "rs-torus-saddle", "rs-two-saddle"]
GPU_STEP = ["rs-icosa-step", "rs-icosa-step-stuck", "rs-torus-step-ref", "rs-mobius-step", "rs-two-step"]


@pytest.fixture(scope="module")
def ctx():
    return R.Context(0)


def _holds(c: G.LeanCase):
    kinds = [k for k, comp, _, _ in c.constraint_items()]
    return int("area" in kinds), int("volume" in kinds)


def _targets(c: G.LeanCase):
    out = {}
    for kind, comp, targets, _ in c.constraint_items():
        if kind in ("area", "volume") and targets:
            out[kind + "_target"] = targets[0]
    return out


def _weights(c: G.LeanCase):
    w = c.line("weights")
    return (G.hexf(w[0]), G.hexf(w[1])) if w else (1.0, 1.0)


def lean_flow(c: G.LeanCase, ctx, **kw):
    ha, hv = _holds(c)
    wtp, clo = _weights(c)
    o = R.flow_options(alpha=c.alpha, beta=c.beta, theta=0.0, hold_area=ha, hold_volume=hv,
                       solver_chi=0.0, solver_tolerance=1e-9, solver_restart=60, solver_max_iterations=600,
                       solver_tp_weight=wtp, solver_low_order=int(clo != 0.0), solver_barycenter_per_component=1,
                       **_targets(c), **kw)
    return R.Flow(c.faces, c.positions, o, ctx)


@pytest.mark.parametrize("name", GPU_SADDLE)
def test_direction_reproduces_saddle_fixture(ctx, name):
    c = G.LeanCase(name)
    flow = lean_flow(c, ctx)
    rep = flow.direction()
    x, g = flow.last_direction()
    print(name, rep["relative_residual"], G.normwise(g, c.vectors("g")), G.normwise(x, c.vectors("x")))
    assert G.normwise(g, c.vectors("g")) <= DIR_TOL
    assert G.normwise(x, c.vectors("x")) <= DIR_TOL
    assert abs(rep["slope"] - c.scalar("gx")) <= DIR_TOL * np.linalg.norm(g) * np.linalg.norm(x)


def _oracle_direction(P, F, theta, chi, hold_area=True, hold_volume=True):
    cons = O.Constraints().barycenter()
    if hold_area:
        cons.area()
    if hold_volume:
        cons.volume()
    o = O.step_options(backend=1, energy_theta=theta, max_halvings=0,
                       solver={"chi": chi, "tolerance": 1e-10, "restart": 60, "max_iterations": 800})
    return O.step(P, F, cons, o)


MESHES = {
    "c1": lambda: gen.config_c1(),
    "torus48x24": lambda: gen.noisy_torus(48, 24, 1.0, 0.3, 0.003, 7),
    "icosa": lambda: (G.LeanCase("rs-icosa-saddle").positions, G.LeanCase("rs-icosa-saddle").faces),
    "torus5x3": lambda: (G.LeanCase("rs-torus-saddle").positions, G.LeanCase("rs-torus-saddle").faces),
}


@pytest.mark.parametrize("mesh", list(MESHES))
@pytest.mark.parametrize("theta,chi", [(0.0, 0.0), (0.25, 0.5)])
def test_direction_matches_oracle_on_the_same_trees(ctx, mesh, theta, chi):
    P, F = MESHES[mesh]()
    ref = _oracle_direction(P, F, theta, chi)
    o = R.flow_options(theta=theta, hold_area=1, hold_volume=1, solver_chi=chi, solver_tolerance=1e-9,
                       solver_restart=60, solver_max_iterations=600)
    flow = R.Flow(F, P, o, ctx)
    rep = flow.direction()
    x, g = flow.last_direction()
    e_err = abs(rep["energy_before"] - ref["energy_before"]) / abs(ref["energy_before"])
    g_err, x_err = G.normwise(g, ref["gradient"]), G.normwise(x, ref["direction"])
    print(f"{mesh} theta {theta} chi {chi}: energy {e_err:.2e} g {g_err:.2e} x {x_err:.2e} "
          f"gpu residual {rep['relative_residual']:.1e} oracle {ref['worst_residual']:.1e}")
    assert e_err <= ENERGY_TOL
    assert g_err <= DIR_TOL
    assert x_err <= DIR_TOL


def _step_kw(c: G.LeanCase):
    wtp, _ = _weights(c)
    st = c.line("start")
    if st is None:
        rule, val = R.START_MAX_DISPLACEMENT, 0.1
    elif st[0] == "abs":
        rule, val = R.START_ABSOLUTE, G.hexf(st[1]) / wtp
    elif st[0] == "maxdisp":
        rule, val = R.START_MAX_DISPLACEMENT, G.hexf(st[1])
    else:
        rule, val = R.START_REFERENCE, 1.0
    nw = c.line("newton") or ["tol", "5"]
    return dict(start_rule=rule, start_value=val,
                armijo_c=G.hexf(c.line("armijo")[0]) if c.line("armijo") else 1e-2,
                max_halvings=int(c.line("maxhalv")[0]) if c.line("maxhalv") else 60,
                newton_fixed=int(nw[0] == "fixed"), newton_max=int(nw[1]), guard_projection=0)


@pytest.mark.parametrize("name", GPU_STEP)
def test_step_reproduces_step_fixture(ctx, name):
    c = G.LeanCase(name)
    flow = lean_flow(c, ctx, **_step_kw(c))
    rep = flow.step()
    trials = flow.last_trials()
    rel = lambda got, want, tol: abs(got - want) <= tol * abs(want)  # noqa: E731
    assert rel(rep["energy_before"], c.scalar("energy0"), ENERGY_TOL)
    assert rel(rep["slope"], c.scalar("slope"), DIR_TOL)
    want = sorted(c.out.get("trial", []), key=lambda t: int(t[0]))
    if want:
        assert rel(rep["tau0"], c.scalar("tau0"), DIR_TOL)
    n = min(len(want), len(trials))
    for (tau, energy, outcome), t in zip(trials[:n], want[:n]):
        if outcome != t[2]:
            margin = G.hexf(t[4])
            assert abs(margin) < 1e-5, (outcome, t)
            pytest.skip(f"borderline Armijo margin {margin:.1e}")
        assert rel(tau, G.hexf(t[1]), DIR_TOL)
        if outcome != "non-finite":
            # a rejected trial can be far off the surface (the stuck case moves vertices by 1e6):
            # its energy carries the FP32 rounding of such a geometry, so 1e-5 here
            assert rel(energy, G.hexf(t[3]), ENERGY_TOL if outcome == "accepted" else DIR_TOL)
    assert len(trials) == len(want)
    res = c.out["result"][0]
    assert bool(rep["accepted"]) == (res[0] == "accepted")
    assert int(rep["halvings"]) == int(res[2])
    assert rel(rep["energy_trial"], c.scalar("energy1"), ENERGY_TOL)
    assert int(rep["newton_steps"]) == int(c.out["newton"][0][0])
    assert rel(rep["energy_after"], c.scalar("energy-final"), ENERGY_TOL)
    P = flow.positions()
    assert G.normwise(P, c.vectors("x")) <= DIR_TOL


def test_coarse_correction_on_linked_tori(ctx):
    """Two linked tori under one global barycenter: no component's translation is fixed by rows
    of its own, so the preconditioner carries the coarse (deflation) correction of
    RS/src/solve/coarse.rs. With it the direction solves take fewer iterations, and the direction
    still equals the oracle's (which builds the same coarse space) within 1e-5."""
    P, F = gen.config_c5(n=24, sigma=0.0005)
    ref = _oracle_direction(P, F, 0.25, 0.5)
    its = {}
    for coarse in (1, 0):
        o = R.flow_options(theta=0.25, hold_area=1, hold_volume=1, solver_chi=0.5, solver_tolerance=1e-9,
                           solver_restart=60, solver_max_iterations=800, solver_coarse=coarse)
        flow = R.Flow(F, P, o, ctx)
        rep = flow.direction()
        x, g = flow.last_direction()
        its[coarse] = rep["gmres_area"] + rep["gmres_volume"] + rep["gmres_direction"]
        err = G.normwise(x, ref["direction"])
        print(f"coarse {coarse}: iterations {its[coarse]:.0f} direction error {err:.2e} "
              f"(oracle {ref['gmres_iterations']:.0f})")
        assert err <= DIR_TOL
    assert its[1] < its[0]
