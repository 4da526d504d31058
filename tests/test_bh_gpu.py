"""GPU parity of the Barnes-Hut energy path against the FP64 oracle, through the C ABI.

Tolerances (the FP32 pair kernel with Kahan accumulation against FP64):
  energy: relative 1e-6; differential: normwise max-relative 1e-5
(``max |got - want| / max |want|``, the comparison of RS/tests/oracle.rs). Integer data (the
interaction lists) must be bit-identical. Cases follow RS/tests/gpu.rs:347-434 (theta in
{0, 0.25, 0.5}, exponents (6,12) and (4,9), before and after a refit, bitwise run to run)
plus the Lean and authors' fixtures, and size-independent identities at full size.
"""
import numpy as np
import pytest

import golden_io as G
import rs_oracle as O
import rs_gb300 as R
from rs_gb300 import generators as gen

pytestmark = pytest.mark.gpu

E_TOL = 1e-6
D_TOL = 1e-5


@pytest.fixture(scope="module")
def ctx():
    return R.Context(0)


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def check(ctx, P, F, theta, alpha=6.0, beta=12.0, leaf=8, lists_equal=True):
    ex = R.Exponents(alpha, beta)
    t = R.BhTree.build(F, P, R.BhOptions(theta, leaf), ctx)
    o = O.BhTree(P, F, theta=theta, leaf_size=leaf)
    if lists_equal:
        tree, lists = t.export()
        ot, ol = o.tree(), o.lists()
        for k in ("start", "end", "right", "order"):
            assert np.array_equal(tree[k], ot[k]), k
        for k in ("lumped_off", "lumped", "exact_off", "exact"):
            assert np.array_equal(lists[k], ol[k]), k
        s, so = t.sizes(), o.sizes()
        assert s["pairs_exact"] == so["pairs_exact"]
    E, dE = t.energy_and_differential(ex)
    Eo, dEo = o.energy_and_differential(alpha, beta)
    print(f"energy {rel(E, Eo):.2e} differential {G.normwise(dE, dEo):.2e}")
    assert rel(E, Eo) <= E_TOL, (E, Eo)
    assert G.normwise(dE, dEo) <= D_TOL
    return t, o, E, dE


MESHES = {
    "c1": lambda: gen.config_c1(),
    "c2-level4": lambda: gen.config_c2(level=4),
    "torus48x24": lambda: gen.noisy_torus(48, 24, 1.0, 0.3, 0.003, 7),
    "torus192": lambda: (G.reference_mesh("torus192")["positions"], G.reference_mesh("torus192")["faces"]),
    "tube_regular": lambda: (G.reference_mesh("tube_regular")["positions"],
                             G.reference_mesh("tube_regular")["faces"]),
}


@pytest.mark.parametrize("mesh", list(MESHES))
@pytest.mark.parametrize("theta", [0.0, 0.25, 0.5])
def test_bh_parity(ctx, mesh, theta):
    P, F = MESHES[mesh]()
    check(ctx, P, F, theta)


@pytest.mark.parametrize("alpha,beta", [(4.0, 9.0), (3.0, 7.5), (4.0, 8.0), (2.0, 5.0)])
def test_bh_parity_other_exponents(ctx, alpha, beta):
    P, F = gen.config_c2(level=3)
    check(ctx, P, F, 0.5, alpha, beta)


@pytest.mark.parametrize("name", G.lean_names("energy", "ok"))
def test_lean_energy_fixtures_on_gpu(ctx, name):
    c = G.LeanCase(name)
    r = R.energy(c.faces, c.positions, R.Exponents(c.alpha, c.beta), "exact", ctx)
    want, dwant = c.scalar("energy"), c.vectors("d")
    if want == 0.0:  # the flat patch: N.(X - Y) = 0 exactly
        assert r.energy == 0.0 and np.abs(r.differential).max() == 0.0
        return
    assert rel(r.energy, want) <= E_TOL
    assert G.normwise(r.differential, dwant) <= D_TOL


@pytest.mark.parametrize("name", ["torus192", "torus504", "tube_regular"])
def test_authors_program_fixtures_on_gpu(ctx, name):
    m = G.reference_mesh(name)
    ex = R.Exponents(m["alpha"], m["beta"])
    r = R.energy(m["faces"], m["positions"], ex, "exact", ctx)
    assert rel(r.energy, m["all_pairs"]) <= E_TOL
    assert G.normwise(r.differential, m["d_all"]) <= D_TOL
    t = R.BhTree.build(m["faces"], m["positions"], R.BhOptions(m["theta"]), ctx)
    E, dE = t.energy_and_differential(ex)
    assert rel(E, m["barnes_hut"]) < 1e-2  # the reference's band: different trees
    assert G.normwise(dE, m["d_bh"]) < 1e-2


def test_bitwise_run_to_run_and_value_path(ctx):
    P, F = gen.config_c2(level=4)
    t = R.BhTree.build(F, P, R.BhOptions(0.25), ctx)
    E1, d1 = t.energy_and_differential()
    E2, d2 = t.energy_and_differential()
    assert E1 == E2 and np.array_equal(d1, d2)
    assert t.try_energy() == E1  # the value path performs the energy's operations


def test_attach_equals_build(ctx):
    P, F = gen.config_c2(level=4)
    o = O.BhTree(P, F, theta=0.25)
    t1 = R.BhTree.build(F, P, R.BhOptions(0.25), ctx)
    t2 = R.BhTree.attach(F, P, o.tree(), o.lists(), ctx)
    a, b = t1.energy_and_differential(), t2.energy_and_differential()
    assert a[0] == b[0] and np.array_equal(a[1], b[1])


def test_refit(ctx):
    P, F = gen.config_c2(level=4)
    rng = np.random.default_rng(5)
    Q = P + 0.002 * rng.standard_normal(P.shape)
    t = R.BhTree.build(F, P, R.BhOptions(0.25), ctx)
    o = O.BhTree(P, F, theta=0.25)
    for X in (Q, P):
        t.refit(X)
        o.refit(X)
        E, dE = t.energy_and_differential()
        Eo, dEo = o.energy_and_differential()
        assert rel(E, Eo) <= E_TOL
        assert G.normwise(dE, dEo) <= D_TOL
        assert rel(t.try_energy(), o.energy()) <= E_TOL


def test_face_partials(ctx):
    P, F = gen.config_c1()
    t = R.BhTree.build(F, P, R.BhOptions(0.5), ctx)
    o = O.BhTree(P, F, theta=0.5)
    E, p = t.try_face_partials()
    Eo, _, po = o.energy_and_differential(partials=True)
    assert rel(E, Eo) <= E_TOL
    for cols in ([0], [1, 2, 3], [4, 5, 6]):
        assert G.normwise(p[:, cols], po[:, cols]) <= D_TOL


def test_non_finite_energy_names_the_pair(ctx):
    c = G.LeanCase("rs-error-same-barycenter")
    with pytest.raises(R.RsError) as ei:
        R.energy(c.faces, c.positions, R.Exponents(c.alpha, c.beta), "exact", ctx)
    assert ei.value.kind == "NonFiniteEnergy"
    assert "(0, 1)" in ei.value.detail


def test_errors(ctx):
    P, F = gen.config_c1()
    with pytest.raises(R.RsError, match="InvalidExponents"):
        R.Exponents(6.0, 8.0)
    t = R.BhTree.build(F, P, R.BhOptions(0.5), ctx)
    with pytest.raises(R.RsError) as ei:
        t.refit(P[:-1])
    assert ei.value.kind == "PositionCountMismatch"
    Q = P.copy()
    Q[3, 0] = np.inf
    with pytest.raises(R.RsError) as ei:
        t.refit(Q)
    assert ei.value.kind == "NonFinitePosition"
    with pytest.raises(R.RsError) as ei:
        R.BhTree.build(F, P, R.BhOptions(0.5, 16), ctx)
    assert ei.value.kind == "InvalidOption"


def test_device_entry_points(ctx):
    torch = pytest.importorskip("torch")
    P, F = gen.config_c2(level=4)
    t = R.BhTree.build(F, P, R.BhOptions(0.25), ctx)
    E, dE = t.energy_and_differential()
    pos = torch.from_numpy(P.copy()).cuda()
    e_dev = torch.zeros(1, dtype=torch.float64, device="cuda")
    d_dev = torch.zeros(P.shape, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    t.refit_device(pos.data_ptr())
    t.energy_and_differential_device(R.Exponents(), e_dev.data_ptr(), d_dev.data_ptr())
    ctx.synchronize()
    assert e_dev.item() == E
    assert np.array_equal(d_dev.cpu().numpy(), dE)


def test_full_size_c2_against_oracle(ctx):
    """Config c2 at its full size (81,920 faces, theta 0.25) against the FP64 oracle."""
    P, F = gen.config_c2()
    check(ctx, P, F, 0.25)


@pytest.mark.parametrize("sigma", [0.01, 0.001])
def test_full_size_c3_against_oracle(ctx, sigma):
    """The 204,800-face torus of the step configuration at its full size (theta 0.25), as
    specified (noise 0.01, crumpled) and as the flow bench runs it (0.001): trees and lists equal
    to the oracle's, energy within 1e-6 and differential within 1e-5 of the FP64 oracle."""
    P, F = gen.config_c3(sigma=sigma)
    _, _, E, dE = check(ctx, P, F, 0.25)
    print(f"c3 sigma {sigma}: E {E:.6e}")


def test_full_size_c3_identities(ctx):
    """Config c3 (204,800 faces): translation and rotation invariance (sum g = 0,
    sum f x g = 0) and the Euler identity sum f.g = (4 + alpha - beta) E, which hold for the
    exact derivative of the frozen-list energy (RS/tests/energy.rs:250)."""
    P, F = gen.config_c3()
    t = R.BhTree.build(F, P, R.BhOptions(0.25), ctx)
    E, g = t.energy_and_differential()
    scale = np.abs(g).sum()
    assert np.isfinite(E) and E > 0
    assert np.abs(g.sum(0)).max() <= 1e-5 * scale
    c = P.mean(0)
    assert np.abs(np.cross(P - c, g).sum(0)).max() <= 1e-5 * np.abs(np.cross(P - c, g)).sum()
    euler = np.sum((P - c) * g)
    assert abs(euler - (4 + 6 - 12) * E) <= 1e-5 * np.abs((P - c) * g).sum()
    assert t.try_energy() == E


def test_build_phase_times(ctx):
    """rs_bh_build_times / rs_metric_build_times: every phase non-negative, and the phases
    together within the build's wall time."""
    import time

    P, F = gen.config_c2(level=4)
    t0 = time.perf_counter()
    t = R.BhTree.build(F, P, R.BhOptions(0.25), ctx)
    wall = time.perf_counter() - t0
    bt = t.build_times()
    assert set(bt) == {"geometry", "tree", "topology", "list_counts", "list_fill", "list_finish", "refit"}
    assert all(v >= 0.0 for v in bt.values()) and sum(bt.values()) <= wall
    t0 = time.perf_counter()
    m = R.FaceMetricTree(F, P, R.Exponents(), R.ClusterTreeOptions(chi=0.5), ctx)
    wall = time.perf_counter() - t0
    mt = m.build_times()
    assert len(mt) == 8 and all(v >= 0.0 for v in mt.values()) and sum(mt.values()) <= wall
