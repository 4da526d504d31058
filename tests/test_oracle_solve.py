"""Pins the oracle's constraint rows, dense saddle, preconditioner and step to the reference's
golden vectors (CPU only), with the tolerances of RS/tests/oracle.rs:30-50:

* ``constraints``: Phi within 1e-12 of max(1, |targets|), the Jacobian within 1e-12, the vertex
  components exactly (run_constraints, oracle.rs:332-375);
* ``saddle``: g 1e-12; x, <g, x>, Phi_N, S, h 1e-10 (run_saddle, oracle.rs:377-420);
* ``precond``: eps and L_{2-s} 1e-12; L' and P^-1 r 1e-10 (run_precond, oracle.rs:422-478);
* ``step``: one dense step with the exact energy, per-component barycenters, no projection
  guard (run_step, oracle.rs:557-668): F, <g, x>, |x|, tau0, every trial's tau, outcome and
  energy, the result, the Newton rounds, Phi and the final positions 1e-10; the mean edge
  length 1e-12.

It also checks the hierarchical path against the dense one: GMRES on the oracle's A' with the
augmented preconditioner reproduces the dense direct solve at chi = 0, and the sparse
preconditioner is symmetric with C_Q P^-1 [r; b] = b (RS/tests/hierarchical.rs:318,624).
"""
import numpy as np
import pytest

import golden_io as G
import rs_oracle as O

SOLVE = 1e-10
MATRIX = 1e-12


def cons_of(c: G.LeanCase) -> O.Constraints:
    k = O.Constraints(per_component=True)
    for kind, comp, targets, verts in c.constraint_items():
        if kind == "barycenter":
            k.barycenter(comp, targets or None)
        elif kind == "pins":
            k.pins(verts, np.reshape(targets, (-1, 3)) if targets else None)
        elif kind == "area":
            k.area(comp, targets[0] if targets else None)
        else:
            k.volume(comp, targets[0] if targets else None)
    return k


def weights(c: G.LeanCase):
    w = c.line("weights")
    return (G.hexf(w[0]), G.hexf(w[1]), G.hexf(w[2])) if w else (1.0, 1.0, 0.0)


def lowest_vertex_per_component(faces, nv):
    parent = list(range(nv))

    def find(x):
        while parent[x] != x:
            parent[x] = parent[parent[x]]
            x = parent[x]
        return x

    for f in faces:
        for v in f[1:]:
            a, b = find(int(f[0])), find(int(v))
            if a != b:
                parent[max(a, b)] = min(a, b)
    return sorted({find(int(f[0])) for f in faces})


@pytest.mark.parametrize("name", G.lean_names("constraints", "ok"))
def test_constraint_fixtures(name):
    """Cases that leave a translation free get a pin on every component after the oracle's rows,
    as the reference's replay does (the check belongs to the saddle there)."""
    c = G.LeanCase(name)
    cons = cons_of(c)
    try:
        rows = O.constraint_rows(c.positions, c.faces, cons)
    except O.OracleError as e:
        assert "TranslationNotFixed" in e.message
        rows = O.constraint_rows(c.positions, c.faces,
                                 cons.pins(lowest_vertex_per_component(c.faces, len(c.positions))))
    want = c.out["row"]
    nr = len(want)
    assert rows["n_components"] == int(c.out["mesh"][0][2])
    assert rows["vcomp"].tolist() == [int(x) for x in c.out["vcomp"][0]]
    names = ["barycenter", "pins", "area", "volume"]
    for i, w in enumerate(sorted(want, key=lambda r: int(r[0]))):
        assert names[rows["kind"][i]] == w[1]
        assert bool(rows["positional"][i]) == (w[2] == "positional")
    phi_want = np.array([G.hexf(w[3]) for w in sorted(want, key=lambda r: int(r[0]))])
    targets = [abs(x) for _, _, t, _ in c.constraint_items() for x in t]
    scale = max([1.0] + targets)
    assert np.max(np.abs(rows["phi"][:nr] - phi_want)) <= 1e-12 * scale
    assert G.normwise(rows["jac"][:nr], c.matrix("J")) <= MATRIX


@pytest.mark.parametrize("name", [n for n in G.lean_names("constraints", "error")])
def test_constraint_error_fixtures(name):
    c = G.LeanCase(name)
    with pytest.raises(O.OracleError) as e:
        O.constraint_rows(c.positions, c.faces, cons_of(c))
    kind = c.error_kind
    assert {"ConstraintOutOfRange": "ConstraintOutOfRange", "NonOrientable": "NonOrientable"}[kind] in e.value.message


@pytest.mark.parametrize("name", G.lean_names("saddle", "ok"))
def test_saddle_fixtures(name):
    c = G.LeanCase(name)
    wtp, clo, ww = weights(c)
    assert ww == 0.0
    r = O.dense_saddle(c.positions, c.faces, cons_of(c), c.alpha, c.beta, wtp, clo != 0.0)
    kq, kn = (int(x) for x in c.out["rows"][0])
    assert (r["kq"], r["kn"]) == (kq, kn)
    assert G.normwise(r["g"], c.vectors("g")) <= 1e-12
    assert G.normwise(r["x"], c.vectors("x")) <= SOLVE
    gn, xn = np.linalg.norm(r["g"]), np.linalg.norm(r["x"])
    assert abs(r["gx"] - c.scalar("gx")) <= SOLVE * gn * xn
    if kn:
        phin = np.array([G.hexf(x) for x in c.out["phin"][0]])
        assert np.max(np.abs(r["phin"] - phin)) <= SOLVE * max(1.0, np.abs(phin).max())
        assert G.normwise(r["S"], c.matrix("S")) <= SOLVE
        assert G.normwise(r["h"], c.vectors("h")) <= SOLVE


@pytest.mark.parametrize("name", G.lean_names("saddle", "error"))
def test_saddle_error_fixtures(name):
    c = G.LeanCase(name)
    with pytest.raises(O.OracleError) as e:
        O.dense_saddle(c.positions, c.faces, cons_of(c), c.alpha, c.beta)
    assert c.error_kind in e.value.message


@pytest.mark.parametrize("name", G.lean_names("precond", "ok"))
def test_precond_fixtures(name):
    c = G.LeanCase(name)
    eps_rel = G.hexf(c.line("eps-rel")[0]) if c.line("eps-rel") else 1e-10
    rows = sorted(c.inputs["r"], key=lambda t: int(t[0]))
    r = np.array([[G.hexf(x) for x in t[1:4]] for t in rows])
    p = O.dense_precond(c.positions, c.faces, cons_of(c), r, c.alpha, c.beta, eps_rel)
    assert abs(p["eps"] - c.scalar("eps")) <= MATRIX * abs(c.scalar("eps"))
    assert G.normwise(p["Lfr"], c.matrix("Lfr")) <= MATRIX
    assert G.normwise(p["Lp"], c.matrix("Lp")) <= SOLVE
    assert G.normwise(p["z"], c.vectors("z")) <= SOLVE


def step_options_of(c: G.LeanCase) -> O.StepOptions:
    wtp, clo, _ = weights(c)
    st = c.line("start")
    if st is None:
        rule, val = 1, 0.1
    elif st[0] == "abs":
        rule, val = 0, G.hexf(st[1]) / wtp
    elif st[0] == "maxdisp":
        rule, val = 1, G.hexf(st[1])
    else:
        rule, val = 2, 0.0
    nw = c.line("newton") or ["tol", "5"]
    return O.step_options(backend=0, energy_theta=-1.0, start_rule=rule, start_value=val,
                          armijo_c=G.hexf(c.line("armijo")[0]) if c.line("armijo") else 1e-2,
                          max_halvings=int(c.line("maxhalv")[0]) if c.line("maxhalv") else 60,
                          newton_fixed=int(nw[0] == "fixed"), newton_max=int(nw[1]), guard_projection=0,
                          solver={"tp_weight": wtp, "low_order": int(clo != 0.0)})


@pytest.mark.parametrize("name", G.lean_names("step", "ok"))
def test_step_fixtures(name):
    c = G.LeanCase(name)
    r = O.step(c.positions, c.faces, cons_of(c), step_options_of(c), c.alpha, c.beta)
    rel = lambda got, want: abs(got - want) <= SOLVE * abs(want)  # noqa: E731
    assert rel(r["energy_before"], c.scalar("energy0"))
    assert rel(r["slope"], c.scalar("slope"))
    assert rel(r["xnorm"], c.scalar("xnorm"))
    assert abs(r["l0"] - c.scalar("lbar")) <= MATRIX * c.scalar("lbar")
    trials = sorted(c.out.get("trial", []), key=lambda t: int(t[0]))
    if trials:
        assert rel(r["tau0"], c.scalar("tau0"))
    assert len(r["trials"]) == len(trials)
    for (tau, energy, outcome), t in zip(r["trials"], trials):
        assert outcome == t[2]
        assert rel(tau, G.hexf(t[1]))
        if outcome != "non-finite":
            assert rel(energy, G.hexf(t[3]))
    res = c.out["result"][0]
    assert bool(r["accepted"]) == (res[0] == "accepted")
    assert int(r["halvings"]) == int(res[2])
    assert rel(r["energy_trial"], c.scalar("energy1"))
    assert int(r["newton_rounds"]) == int(c.out["newton"][0][0])
    phi_want = np.array([G.hexf(x) for x in c.out["phi"][0]])
    targets = [abs(x) for _, _, t, _ in c.constraint_items() for x in t]
    scale = max([1.0] + targets + list(np.abs(O.constraint_rows(c.positions, c.faces, cons_of(c))["phi"]) * 0))
    assert np.max(np.abs(r["phi_after"] - phi_want)) <= SOLVE * max(scale, 1.0)
    assert rel(r["energy_after"], c.scalar("energy-final"))
    assert np.max(np.abs(r["positions"] - c.vectors("x"))) <= SOLVE * max(1.0, np.abs(c.vectors("x")).max())


def _dense_vertex_fractional(P, mass, tau):
    """L^V_tau over vertex pairs, dense: 2 (diag(a . H a) - diag(a) H diag(a)), H_vw =
    |f_v - f_w|^-(2 tau + 2) (vertex_fractional_operator, RS/src/metric/dense.rs:469-520)."""
    d2 = ((P[:, None, :] - P[None, :, :]) ** 2).sum(-1)
    np.fill_diagonal(d2, 1.0)
    H = d2 ** (-(tau + 1.0))
    np.fill_diagonal(H, 0.0)
    return 2.0 * (np.diag(mass * (H @ mass)) - mass[:, None] * H * mass[None, :])


@pytest.mark.parametrize("name", ["rs-icosa-precond", "rs-two-precond"])
def test_sparse_preconditioner_equals_its_dense_form(name):
    """The oracle's hierarchical preconditioner at chi = 0 (the augmented form with the symbol
    scale, L' by the sparse LDL^T; RS/src/solve/precond.rs:1026-1079) equals the same formula
    evaluated densely from the fixture-pinned L' (the Lean fixture's Lp, reproduced by
    test_precond_fixtures) and a dense vertex-pair L_{2-s}:
    P^-1 = X + X blockdiag((s L - K) x I3, 0) X, X = L'^-1."""
    c = G.LeanCase(name)
    P, F = c.positions, c.faces
    cons = O.Constraints(per_component=True).barycenter()
    d = O.dense_precond(P, F, cons, np.zeros_like(P), c.alpha, c.beta, 1e-10)
    Lp = d["Lp"]
    nd = 3 * len(P)
    X = np.linalg.inv(Lp)
    a, _, _ = O.face_geometry(P, F)
    mass = np.zeros(len(P))
    np.add.at(mass, F.ravel().astype(np.int64), np.repeat(a / 3.0, 3))
    s = (c.beta - 2.0) / c.alpha
    Lv = _dense_vertex_fractional(P, mass, 2.0 - s)
    h = O.HSolver(P, F, cons, O.solver_options(chi=0.0, coarse=0), c.alpha, c.beta)
    scale = h.info()["fractional_scale"]
    K = Lp[:nd, :nd]
    mid = np.zeros_like(Lp)
    mid[:nd, :nd] = scale * np.kron(Lv, np.eye(3)) - K
    Pinv = X + X @ mid @ X
    r = np.random.default_rng(8).standard_normal((3, h.n))
    z = h.precondition(r)
    zd = r @ Pinv.T
    # X K X cancels against X to O(1) from entries of order 1/eps (eps = 1e-10 tr W / tr M): both
    # evaluations keep about nine digits, so 1e-6 (measured 2.6e-7); a wrong term is O(1)
    assert G.normwise(z, zd) <= 1e-6
    # the constraint rows are reproduced: C_Q P^-1 [r; b] = b
    assert np.abs((Lp[nd:, :nd] @ z[:, :nd].T).T - r[:, nd:]).max() <= 1e-6 * np.abs(r).max()
