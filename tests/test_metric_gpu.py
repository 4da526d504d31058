"""GPU parity of the hierarchical Hs metric B~ + B~0 and of the vertex-pair fractional
operator L^V against the FP64 oracle, through the C ABI (RS/tests/hierarchical.rs,
RS/tests/gpu.rs:116-254 for the cases).

* The block structure (far and near blocks by row node) must equal the oracle's exactly.
* Products are FP32 on the device: normwise max-relative error <= 2e-5 against the FP64
  oracle on random inputs (PRODUCT_TOL), and chi = 0 reproduces the Lean dense B and B0.
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

PRODUCT_TOL = 2e-5


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
        assert G.normwise(y, yo) <= PRODUCT_TOL, (w_hi, w_lo)


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
    assert G.normwise(Bh, c.matrix("B")) <= PRODUCT_TOL
    assert G.normwise(Bl, c.matrix("B0")) <= PRODUCT_TOL


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
    assert err <= 1e-3


@pytest.mark.parametrize("mesh", ["c1", "c2-level4", "torus192"])
def test_vertex_fractional(ctx, mesh):
    P, F = MESHES[mesh]()
    mass = dual_areas(P, F)
    tau = 2.0 - 5.0 / 3.0
    v = R.VertexFractionalTree(P, mass, tau, R.ClusterTreeOptions(), ctx)
    o = O.VertexFractionalTree(P, mass, tau)
    assert v.stats() == o.stats()
    x = np.random.default_rng(4).standard_normal((2, 3 * len(P)))
    assert G.normwise(v.apply(x), o.apply(x)) <= PRODUCT_TOL
    assert np.all(v.apply(np.ones(3 * len(P))) == 0.0)  # L 1 = 0 exactly
