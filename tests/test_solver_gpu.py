"""GPU saddle solver (operator, preconditioner, GMRES) against the FP64 oracle operator.

* A' x on the device equals the oracle's metric product plus the barycenter rows
  (normwise <= 1e-7; measured 4.7e-8).
* GMRES reaches the requested true relative residual (1e-6, the target of the flow), and the
  solution also solves the FP64 oracle system: ||A'_oracle y - rhs|| / ||rhs|| <= 1e-6
  (measured about 1.2e-7), for one and several right-hand sides.
* The preconditioner keeps the iteration count low (<= 60 at restart 30).
"""
import numpy as np
import pytest

import golden_io as G
import rs_oracle as O
import rs_gb300 as R
from rs_gb300 import generators as gen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return R.Context(0)


def oracle_operator(P, F, chi=0.5):
    """A' of the oracle: metric (w = 1, c_lo = 1) plus the global barycenter rows."""
    o = O.FaceMetricTree(P, F, chi=chi)
    a, _, _ = O.face_geometry(P, F)
    mass = np.zeros(len(P))
    np.add.at(mass, F.ravel().astype(np.int64), np.repeat(a / 3.0, 3))
    c = mass / mass.sum()
    nd = 3 * len(P)

    def apply(v):
        v = np.atleast_2d(v)
        out = np.empty_like(v)
        out[:, :nd] = o.apply(v[:, :nd])
        lam = v[:, nd:]
        out[:, :nd] += (c[None, :, None] * lam[:, None, :]).reshape(len(v), nd)
        out[:, nd:] = np.einsum("v,qvk->qk", c, v[:, :nd].reshape(len(v), -1, 3))
        return out

    return apply


def test_operator_matches_oracle(ctx):
    P, F = gen.config_c2(level=4)
    S = R.SaddleSolver(F, P, R.Exponents(), R.solver_options(), ctx)
    A = oracle_operator(P, F)
    x = np.random.default_rng(1).standard_normal((3, S.n))
    print(f"operator error {G.normwise(S.apply(x), A(x)):.2e}")
    assert G.normwise(S.apply(x), A(x)) <= 1e-7


@pytest.mark.parametrize("mesh", ["c1", "c2-level4", "torus48x24"])
def test_gmres_solves_the_saddle(ctx, mesh):
    P, F = {"c1": gen.config_c1, "c2-level4": lambda: gen.config_c2(level=4),
            "torus48x24": lambda: gen.noisy_torus(48, 24, 1.0, 0.3, 0.003, 7)}[mesh]()
    S = R.SaddleSolver(F, P, R.Exponents(), R.solver_options(tolerance=1e-6), ctx)
    A = oracle_operator(P, F)
    rng = np.random.default_rng(3)
    rhs = rng.standard_normal((3, S.n))
    rhs[:, S.n_dofs:] = 0.0
    y, reps = S.solve_many(rhs)
    for i, r in enumerate(reps):
        print(mesh, r)
        assert r["converged"] and r["relative_residual"] <= 1e-6
        assert r["iterations"] <= 60
        res = np.linalg.norm(A(y[i])[0] - rhs[i]) / np.linalg.norm(rhs[i])
        print(f"{mesh}: residual of the oracle operator {res:.2e}")
        assert res <= 1e-6, res
    y1, _ = S.solve_many(rhs[:1])
    assert G.normwise(y1[0], y[0]) <= 1e-5


def test_gmres_without_preconditioner_needs_more_iterations(ctx):
    P, F = gen.config_c1()
    rhs = np.random.default_rng(5).standard_normal((1, 3 * len(P) + 3))
    rhs[:, 3 * len(P):] = 0.0
    with_p = R.SaddleSolver(F, P, R.Exponents(), R.solver_options(), ctx).solve_many(rhs)[1][0]
    no_p = R.SaddleSolver(F, P, R.Exponents(), R.solver_options(preconditioner=0, max_iterations=400,
                                                                 tolerance=1e-3), ctx)
    try:
        r = no_p.solve_many(rhs)[1][0]
        assert r["iterations"] > with_p["iterations"]
    except R.RsError as e:  # diverging without a preconditioner is the expected failure mode
        assert e.kind == "SolverDiverged"


@pytest.mark.parametrize("mesh", ["c1", "torus48x24"])
def test_preconditioner_matches_oracle_with_converged_lprime(ctx, mesh):
    """The fractional preconditioner (a20) and its L' solve (a19) against the oracle's restatement
    of the crate's (the augmented form with an exact sparse LDL^T of L', pinned to the Lean
    precond fixtures): with enough conjugate-gradient steps the multigrid L'^-1 converges, and
    the GPU's X (s L + C) X equals the crate's X + X (s L - K) X (identical for an exact X)."""
    P, F = {"c1": gen.config_c1, "torus48x24": lambda: gen.noisy_torus(48, 24, 1.0, 0.3, 0.003, 7)}[mesh]()
    S = R.SaddleSolver(F, P, R.Exponents(), R.solver_options(chi=0.5, vcycles=100), ctx)
    H = O.HSolver(P, F, O.Constraints().barycenter(), O.solver_options(chi=0.5, coarse=0))
    r = np.random.default_rng(12).standard_normal((2, S.n))
    err = G.normwise(S.precondition(r), H.precondition(r))
    print(f"{mesh}: preconditioner against the oracle's {err:.2e}")
    assert err <= 1e-4


@pytest.mark.parametrize("mesh", ["c1", "torus48x24"])
def test_dense_last_resort_solves_the_exact_saddle(ctx, mesh):
    """The last stage of the recovery chain (DenseSaddle, RS/src/solve/dense.rs:282-470, for at
    most 6000 vertices): A' with the exact metric assembled densely on the device and factored by
    a pivoted FP64 LU with one refinement step. Its solution solves the oracle's FP64 operator
    with the exact metric (chi = 0) to 1e-6 and equals GMRES on the library's chi = 0 operator
    to 1e-6; the equilibrated pivot ratio is above PIVOT_TOLERANCE (1e-13)."""
    P, F = {"c1": gen.config_c1, "torus48x24": lambda: gen.noisy_torus(48, 24, 1.0, 0.3, 0.003, 7)}[mesh]()
    S = R.SaddleSolver(F, P, R.Exponents(), R.solver_options(), ctx)
    rng = np.random.default_rng(21)
    rhs = rng.standard_normal((2, S.n))
    rhs[1, S.n_dofs:] = 0.0
    y, reps = S.dense_solve_many(rhs)
    ratio = S.dense_pivot_ratio()
    print(mesh, reps, f"pivot ratio {ratio:.3e}")
    assert ratio > 1e-13
    A = oracle_operator(P, F, chi=0.0)
    S0 = R.SaddleSolver(F, P, R.Exponents(), R.solver_options(chi=0.0, tolerance=1e-10, restart=60,
                                                             max_iterations=2000), ctx)
    y0, _ = S0.solve_many(rhs)
    for i, r in enumerate(reps):
        assert r["converged"] and r["relative_residual"] <= 1e-10
        res = np.linalg.norm(A(y[i])[0] - rhs[i]) / np.linalg.norm(rhs[i])
        print(f"{mesh}: dense solution, residual of the oracle operator {res:.2e}, "
              f"against GMRES {G.normwise(y[i], y0[i]):.2e}")
        assert res <= 1e-6
        assert G.normwise(y[i], y0[i]) <= 1e-6
    # the factor is kept: a second call solves with it again
    y2, _ = S.dense_solve_many(rhs[:1])
    assert G.normwise(y2[0], y[0]) <= 1e-12


@pytest.mark.parametrize("mesh", ["c1", "torus320"])
def test_inner_operator_keeps_the_solution(ctx, mesh):
    """inner_plain (the default): the Arnoldi steps apply the operator with plain-FP32 near-field
    sums, while every cycle-start residual, the convergence test and the reported residual use
    the full operator. The solves reach the same true relative residual (1e-6, on the full
    operator and on the oracle's FP64 one) and the same solution as with the full operator
    throughout, within 1e-5."""
    P, F = {"c1": gen.config_c1, "torus320": lambda: gen.noisy_torus(320, 320, 1.0, 0.3, 0.001, 3)}[mesh]()
    rng = np.random.default_rng(31)
    S1 = R.SaddleSolver(F, P, R.Exponents(), R.solver_options(tolerance=1e-6, inner_plain=1), ctx)
    rhs = rng.standard_normal((3, S1.n))
    rhs[:, S1.n_dofs:] = 0.0
    y1, r1 = S1.solve_many(rhs)
    del S1
    S0 = R.SaddleSolver(F, P, R.Exponents(), R.solver_options(tolerance=1e-6, inner_plain=0), ctx)
    y0, r0 = S0.solve_many(rhs)
    x1 = S0.apply(y1)
    for i in range(3):
        true_res = np.linalg.norm(x1[i] - rhs[i]) / np.linalg.norm(rhs[i])
        print(f"{mesh}: iterations {r0[i]['iterations']} (full) {r1[i]['iterations']} (inner); residual "
              f"{r1[i]['relative_residual']:.2e}, on the full operator {true_res:.2e}; "
              f"solutions {G.normwise(y1[i], y0[i]):.2e}")
        assert r1[i]["converged"] and r1[i]["relative_residual"] <= 1e-6 and true_res <= 1e-6
        assert G.normwise(y1[i], y0[i]) <= 1e-5
    if mesh == "c1":
        A = oracle_operator(P, F)
        for i in range(3):
            assert np.linalg.norm(A(y1[i])[0] - rhs[i]) / np.linalg.norm(rhs[i]) <= 1e-6
