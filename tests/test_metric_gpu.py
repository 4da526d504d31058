"""GPU parity of the hierarchical Hs metric B~ + B~0 and of the vertex-pair fractional
operator L^V against the FP64 oracle, through the C ABI (RS/tests/hierarchical.rs,
RS/tests/gpu.rs:116-254 for the cases).

* The block structure (far and near blocks by row node) must equal the oracle's exactly.
* Products are float-pair sums of FP32 kernel values on the device: normwise max-relative error
  against the FP64 oracle <= 1e-7 on random inputs (5e-7 for B~0 alone, whose norm is small),
  <= 1e-6 on smooth inputs (a small difference of large sums), at c1, c2 and the 204,800-face
  torus; chi = 0 reproduces the Lean dense B (2e-7) and B0 (5e-7).
* L 1 = 0 holds exactly for the average (B0) channels: H~a is formed with the operations of
  H~(a m) (hierarchical.rs:13-16).
* A batch of vectors gives every vector bitwise the result of a single product.
"""
import numpy as np
import pytest

import golden_io as G
import rs_oracle as O
import rs_gb300 as R
from rs_gb300 import generators as gen

pytestmark = pytest.mark.gpu

PRODUCT_TOL = 1e-7      # random inputs, B~ + B~0 and B~ (measured <= 6.5e-8)
PRODUCT_TOL_LO = 5e-7   # random inputs, B~0 alone (measured <= 3.9e-7)
SMOOTH_TOL = 1e-6       # smooth inputs (measured <= 6.5e-7)
VERTEX_TOL = 2e-7       # L^V on random inputs (measured <= 1.1e-7)


@pytest.fixture(scope="module")
def ctx():
    return R.Context(0)


MESHES = {
    "c1": lambda: gen.config_c1(),
    "c2-level4": lambda: gen.config_c2(level=4),
    "torus48x24": lambda: gen.noisy_torus(48, 24, 1.0, 0.3, 0.003, 7),
    "torus192": lambda: (G.reference_mesh("torus192")["positions"], G.reference_mesh("torus192")["faces"]),
}


def dual_areas(P, F):
    a, _, _ = O.face_geometry(P, F)
    m = np.zeros(len(P))
    np.add.at(m, F.ravel().astype(np.int64), np.repeat(a / 3.0, 3))
    return m


@pytest.mark.parametrize("mesh", list(MESHES))
@pytest.mark.parametrize("chi", [0.0, 0.5, 1.0])
def test_metric_blocks_and_product(ctx, mesh, chi):
    P, F = MESHES[mesh]()
    m = R.FaceMetricTree(F, P, R.Exponents(), R.ClusterTreeOptions(chi=chi), ctx)
    o = O.FaceMetricTree(P, F, chi=chi)
    assert m.stats() == o.stats()
    b, ob = m.blocks(), o.blocks()
    for k in ("far_ptr", "far_col", "near_ptr", "near_col"):
        assert np.array_equal(b[k].astype(np.int64), ob[k].astype(np.int64)), k
    rng = np.random.default_rng(11)
    x = rng.standard_normal((3, 3 * len(P)))
    for w_hi, w_lo in ((1.0, 1.0), (1.0, 0.0), (0.0, 1.0), (0.7, 0.3)):
        y = m.apply(x, w_hi, w_lo)
        yo = o.apply(x, w_hi, w_lo)
        print(f"{mesh} chi {chi} w ({w_hi}, {w_lo}): random-input error {G.normwise(y, yo):.2e}")
        assert G.normwise(y, yo) <= (PRODUCT_TOL if w_hi > 0.0 else PRODUCT_TOL_LO), (w_hi, w_lo)


@pytest.mark.parametrize("name", G.lean_names("metric", "ok"))
def test_chi0_reproduces_lean_dense_metric(ctx, name):
    c = G.LeanCase(name)
    nv = len(c.positions)
    m = R.FaceMetricTree(c.faces, c.positions, R.Exponents(c.alpha, c.beta),
                         R.ClusterTreeOptions(chi=0.0), ctx)
    X = np.zeros((nv, 3 * nv))
    X[np.arange(nv), 3 * np.arange(nv)] = 1.0
    Bh = m.apply(X, 1.0, 0.0)[:, 0::3].T
    Bl = m.apply(X, 0.0, 1.0)[:, 0::3].T
    print(f"{name}: B {G.normwise(Bh, c.matrix('B')):.2e} B0 {G.normwise(Bl, c.matrix('B0')):.2e}")
    assert G.normwise(Bh, c.matrix("B")) <= 2 * PRODUCT_TOL
    assert G.normwise(Bl, c.matrix("B0")) <= PRODUCT_TOL_LO


def test_null_space_and_batches(ctx):
    P, F = gen.config_c2(level=4)
    m = R.FaceMetricTree(F, P, R.Exponents(), R.ClusterTreeOptions(), ctx)
    one = np.ones(3 * len(P))
    assert np.all(m.apply(one, 0.0, 1.0) == 0.0)
    rng = np.random.default_rng(2)
    x = rng.standard_normal((5, 3 * len(P)))
    yb = m.apply(x)
    for i in range(5):
        assert np.array_equal(m.apply(x[i]), yb[i])


def test_smooth_input_accuracy(ctx):
    """A smooth field (low-degree polynomial of the positions): the operator's output is a
    small difference of large sums, the hard case for FP32."""
    P, F = gen.config_c2(level=5)
    m = R.FaceMetricTree(F, P, R.Exponents(), R.ClusterTreeOptions(), ctx)
    o = O.FaceMetricTree(P, F)
    x = np.stack([P[:, 0] * P[:, 1], P[:, 2] ** 2, np.sin(P[:, 0])], axis=1).ravel()
    y, yo = m.apply(x), o.apply(x)
    err = G.normwise(y, yo)
    print(f"smooth-input metric product error {err:.3e}")
    assert err <= SMOOTH_TOL


def test_smooth_input_accuracy_full_size(ctx):
    """The smooth-input product on the 204,800-face torus of the flow (noise 0.001) and the
    81,920-face c2 sphere, and a random input on both."""
    for P, F, name in ((*gen.config_c3s(), "c3s"), (*gen.config_c2(), "c2")):
        m = R.FaceMetricTree(F, P, R.Exponents(), R.ClusterTreeOptions(), ctx)
        o = O.FaceMetricTree(P, F)
        x = np.stack([P[:, 0] * P[:, 1], P[:, 2] ** 2, np.sin(P[:, 0])], axis=1).ravel()
        xr = np.random.default_rng(5).standard_normal(3 * len(P))
        es, er = G.normwise(m.apply(x), o.apply(x)), G.normwise(m.apply(xr), o.apply(xr))
        print(f"{name}: smooth-input error {es:.2e} random-input error {er:.2e}")
        assert es <= SMOOTH_TOL and er <= PRODUCT_TOL


@pytest.mark.parametrize("mesh", ["c1", "c2-level4", "torus192"])
def test_vertex_fractional(ctx, mesh):
    P, F = MESHES[mesh]()
    mass = dual_areas(P, F)
    tau = 2.0 - 5.0 / 3.0
    v = R.VertexFractionalTree(P, mass, tau, R.ClusterTreeOptions(), ctx)
    o = O.VertexFractionalTree(P, mass, tau)
    assert v.stats() == o.stats()
    x = np.random.default_rng(4).standard_normal((2, 3 * len(P)))
    print(f"{mesh}: vertex fractional error {G.normwise(v.apply(x), o.apply(x)):.2e}")
    assert G.normwise(v.apply(x), o.apply(x)) <= VERTEX_TOL
    assert np.all(v.apply(np.ones(3 * len(P))) == 0.0)  # L 1 = 0 exactly
