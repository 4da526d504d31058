"""Continuous collision detection on the GPU against the oracle: tau_max bitwise, and the
window, candidate-pair, close-pair and touching-pair counts equal, on the reference's
known-answer scenes, seeded random soups, sphere pairs and a torus sweep over several windows
(first_contact, RS/src/ccd.rs:762-884)."""
import numpy as np
import pytest

import ccd_scenes as S
import rs_gb300 as R
import rs_oracle as O

pytestmark = pytest.mark.gpu

KEYS = ("tau_max", "contact", "windows", "pairs_tested", "close_pairs", "touching_pairs")


def _both(f, p, v, tau_end, ell, **kw):
    o = O.ccd_first_contact(f, p, v, tau_end, reference_length=ell, **kw)
    g = R.CcdSurface(f, len(p)).first_contact(p, v, tau_end, R.ccd_options(reference_length=ell, **kw))
    return o, g


def _same(o, g):
    assert {k: g[k] for k in KEYS} == {k: o[k] for k in KEYS}, (o, g)


@pytest.mark.parametrize("name", list(S.known_answer_scenes()))
def test_known_answer_scenes_bitwise(name):
    f, p, v, tau_end, ell, *_ = S.known_answer_scenes()[name]
    _same(*_both(f, p, v, tau_end, ell))


def test_random_soups_bitwise():
    contacts = 0
    for seed in range(40):
        f, p, v, tau_end, ell = S.random_soup(1000 + seed)
        o, g = _both(f, p, v, tau_end, ell)
        _same(o, g)
        contacts += o["contact"]
    assert contacts >= 3


def test_sphere_pairs_bitwise():
    for seed in range(6):
        _same(*_both(*S.sphere_pair(77 + seed, level=2)))


@pytest.mark.parametrize("reach", [0.5, 3.0, 12.0])
def test_torus_sweep_bitwise(reach):
    f, p, v, tau_end, ell = S.torus_sweep(48, 24, reach=reach)
    o, g = _both(f, p, v, tau_end, ell)
    _same(o, g)
    assert g["pairs_tested"] > 0 and g["evaluations"] >= g["pairs_tested"]


def test_options_change_the_result_as_in_the_oracle():
    f, p, v, tau_end, ell = S.torus_sweep(24, 12, reach=3.0)
    for kw in ({"gap": 0.2}, {"max_iterations": 2}, {"close_factor": 0.0}):
        _same(*_both(f, p, v, tau_end, ell, **kw))


def test_repeated_calls_reuse_the_topology():
    f, p, v, tau_end, ell = S.torus_sweep(24, 12, reach=3.0)
    c = R.CcdSurface(f, len(p))
    a = c.first_contact(p, v, tau_end)
    b = c.first_contact(p, v, tau_end)
    assert a == b
    o = O.ccd_first_contact(f, p, v, tau_end)
    assert a["tau_max"] == o["tau_max"]
    assert c.last_seconds() > 0.0


def test_errors_are_invalid_option():
    f, p, v, *_ = S.known_answer_scenes()["stationary"]
    c = R.CcdSurface(f, len(p))
    for kw in ({"gap": 0.0}, {"max_iterations": 0}, {"close_factor": 1.0}, {"reference_length": -1.0}):
        with pytest.raises(R.RsError) as e:
            c.first_contact(p, v, 1.0, R.ccd_options(**kw))
        assert e.value.kind == "InvalidOption"
    bad = v.copy()
    bad[2, 1] = np.nan
    with pytest.raises(R.RsError):
        c.first_contact(p, bad, 1.0)
    with pytest.raises(R.RsError):
        c.first_contact(p, v, -1.0)


def test_intersecting_pairs_and_band_bitwise():
    f, p, r = S.overlapping_and_apart()
    ell = S._mean_edge_length(f, p)
    c = R.CcdSurface(f, len(p))
    assert c.intersecting_pairs(p).tolist() == O.ccd_intersecting_pairs(p, f).tolist()
    npairs, nverts = c.set_band(p)
    assert npairs == len(O.ccd_intersecting_pairs(p, f)) and nverts > 0
    for k, vz in ((1, 0.4), (2, 1.0)):
        v = np.zeros_like(p)
        v[r[k].start:r[k].stop] = [0.0, 0.0, vz]
        o = O.ccd_first_contact(f, p, v, 3.0, reference_length=ell, band=True)
        g = c.first_contact(p, v, 3.0, R.ccd_options(reference_length=ell))
        _same(o, g)
        assert g["exempt_pairs"] == o["exempt_pairs"] and o["band_vertices"] == nverts
    c.set_band(None)
    v = np.zeros_like(p)
    v[r[1].start:r[1].stop] = [0.0, 0.0, 0.4]
    _same(O.ccd_first_contact(f, p, v, 1.0, reference_length=ell), c.first_contact(p, v, 1.0, R.ccd_options(reference_length=ell)))


def test_band_of_an_embedded_mesh_is_empty():
    f, p, v, tau_end, ell = S.embedded_spheres()
    c = R.CcdSurface(f, len(p))
    assert c.set_band(p) == (0, 0)
    assert len(c.intersecting_pairs(p)) == 0
    _same(O.ccd_first_contact(f, p, v, tau_end, reference_length=ell), c.first_contact(p, v, tau_end,
                                                                                    R.ccd_options(reference_length=ell)))


def test_coplanar_and_random_intersections_bitwise():
    for seed in range(4):
        f, p = S.flat_grid(12, seed)
        assert len(R.CcdSurface(f, len(p)).intersecting_pairs(p)) == 0
    for seed in range(20):
        f, p, v, tau_end, ell = S.random_soup(2000 + seed, k=12)
        c = R.CcdSurface(f, len(p))
        assert c.intersecting_pairs(p).tolist() == O.ccd_intersecting_pairs(p, f).tolist()
        c.set_band(p)
        _same(O.ccd_first_contact(f, p, v, tau_end, reference_length=ell, band=True),
              c.first_contact(p, v, tau_end, R.ccd_options(reference_length=ell)))


def test_full_size_torus_bitwise():
    """The bench's workload: the 204,800-face torus along a smooth motion (tau_max and every
    exact count equal to the oracle's at full size)."""
    import bench

    P, F, _, _ = bench.workload("flow")
    V = bench.ccd_motion(P, F)
    g = R.CcdSurface(F, len(P)).first_contact(P, V, 1.0)
    o = O.ccd_first_contact(F, P, V, 1.0)
    _same(o, g)
    assert g["pairs_tested"] > 1_000_000


def test_edge_cases_bitwise():
    # tau_end = 0, no motion, one triangle, a degenerate (zero-area) triangle, many windows
    f, p, v, tau_end, ell = S.random_soup(3000, k=6)
    _same(*_both(f, p, v, 0.0, ell))
    _same(*_both(f, p, np.zeros_like(v), 2.0, ell))
    one_f = np.array([[0, 1, 2]], np.uint32)
    one_p = np.array([[0.0, 0, 0], [1, 0, 0], [0, 1, 0]])
    o, g = _both(one_f, one_p, np.ones((3, 3)), 1.0, 1.0)
    _same(o, g)
    assert g["pairs_tested"] == 0 and g["tau_max"] == 1.0
    deg_f, deg_p = S.soup([[[0.0, 0, 0], [1, 0, 0], [0, 1, 0]], [[0.3, 0.3, 1.0], [0.3, 0.3, 1.0], [0.6, 0.6, 1.0]]])
    deg_v = np.zeros((6, 3))
    deg_v[3:] = [0.0, 0.0, -1.0]
    _same(*_both(deg_f, deg_p, deg_v, 2.0, 1.0))
    # a long sweep: the window doubles several times before the contact near t = 9.95
    f, p, v = S.two_triangles([[0.2, 0.2, 10.0], [1.0, 1.0, 10.5], [-0.5, 1.2, 10.5]], [0.0, 0.0, -1.0])
    o, g = _both(f, p, v, 20.0, 1.0)
    _same(o, g)
    assert g["windows"] >= 4 and 9.9 < g["tau_max"] <= 9.95 + 1e-9
