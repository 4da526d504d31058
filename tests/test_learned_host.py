"""Host side of the learned preconditioner's training: the seeded training meshes span the
configured sizes (20,000-204,800 faces, tori and spheres), and the right-hand sides are unit
vectors of the mesh's size (CPU only)."""
import numpy as np

from rs_gb300 import learned as L


def test_training_meshes_span_the_configured_sizes():
    meshes = L.training_meshes(8)
    faces = [len(F) for _, F in meshes]
    assert min(faces) >= 20_000 and max(faces) == 204_800
    # one icosphere in four (level 6: 81,920 faces; level 5: 20,480)
    assert faces[3] == 81_920 and faces[7] == 20_480
    # the tori take the sizes of TRAIN_TORI from the largest down
    tori = [f for i, f in enumerate(faces) if i % 4 != 3]
    assert tori == [2 * a * b for a, b in L.TRAIN_TORI[::-1][:len(tori)]]
    # seeded: the same meshes every time
    P0, _ = L.training_meshes(1)[0]
    assert np.array_equal(P0, meshes[0][0])


def test_torus_noise_stays_within_a_third_of_the_minor_edge():
    P, F = L.training_meshes(1)[0]
    Fi = F.astype(np.int64)
    e = np.linalg.norm(P[Fi[:, 1]] - P[Fi[:, 0]], axis=1)
    # the noise (0.1-0.3 of the minor edge per coordinate) leaves every edge non-degenerate
    assert e.min() > 0.0 and np.isfinite(P).all()


def test_residuals_are_unit_vectors():
    P, F = L.training_meshes(1)[0]
    rng = np.random.default_rng(0)
    dE = rng.standard_normal(P.shape)
    rs = L.residuals(P, F, dE, 3, rng)
    assert len(rs) == 3
    for r in rs:
        assert r.shape == (3 * len(P),) and abs(np.linalg.norm(r) - 1.0) < 1e-12
