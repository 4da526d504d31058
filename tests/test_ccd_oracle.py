"""The CCD oracle pinned by the reference's known-answer scenes (crates/ddg-repulsive-surfaces/
tests/ccd.rs:91-196, 363-389) and by sampling: nothing closer than the gap before tau_max, and
tau_max = tau_end when the sampled motion never comes within 1.2 gaps (tests/ccd.rs:221-243)."""
import numpy as np
import pytest

import ccd_scenes as S
import rs_oracle as O


@pytest.mark.parametrize("name", list(S.known_answer_scenes()))
def test_known_answer_scenes(name):
    f, p, v, tau_end, ell, *expect = S.known_answer_scenes()[name]
    r = O.ccd_first_contact(f, p, v, tau_end, reference_length=ell)
    for e in expect:
        if e[0] == "range":
            assert e[1] < r["tau_max"] <= e[2], r
            assert r["contact"] == 1
        elif e[0] == "end":
            assert r["tau_max"] == tau_end and r["contact"] == 0, r
        elif e[0] == "close":
            assert r["close_pairs"] == e[1], r
        elif e[0] == "touching":
            assert r["touching_pairs"] == e[1], r
        elif e[0] == "any":
            assert r["tau_max"] < tau_end or r["contact"] == 0
    if name == "head_on_vertex_face":
        assert (r["close_pairs"], r["touching_pairs"]) == (0, 0)


def test_option_and_input_errors():
    f, p, v, *_ = S.known_answer_scenes()["stationary"]
    for kw in ({"gap": 0.0}, {"gap": float("nan")}, {"max_iterations": 0}, {"close_factor": 1.0},
               {"reference_length": -1.0}):
        with pytest.raises(O.OracleError):
            O.ccd_first_contact(f, p, v, 1.0, **kw)
    with pytest.raises(O.OracleError):
        O.ccd_first_contact(f, p, v, -1.0)
    bad = v.copy()
    bad[2, 1] = np.nan
    with pytest.raises(O.OracleError):
        O.ccd_first_contact(f, p, bad, 1.0)


def _check_sampled(f, p, v, tau_end, ell, samples=120):
    gap = 0.05 * ell
    r = O.ccd_first_contact(f, p, v, tau_end, reference_length=ell)
    assert 0.0 <= r["tau_max"] <= tau_end
    ts = np.linspace(0.0, r["tau_max"], samples + 1)
    dmin = min(O.ccd_min_distance(p + t * v, f) for t in ts)
    assert dmin >= gap * (1 - 1e-6), (r, dmin)
    near = min(O.ccd_min_distance(p + t * v, f) for t in np.linspace(0.0, tau_end, samples + 1))
    if near >= 1.2 * gap:
        assert r["tau_max"] == tau_end, r
    return r


def test_random_soups_against_sampling():
    contacts = 0
    for seed in range(40):
        f, p, v, tau_end, ell = S.random_soup(1000 + seed)
        if O.ccd_min_distance(p, f) <= 1.5 * 0.05 * ell:  # start free, as the reference's soups
            continue
        contacts += _check_sampled(f, p, v, tau_end, ell)["contact"]
    assert contacts >= 3


def test_sphere_pairs_against_sampling():
    out = [_check_sampled(*S.sphere_pair(77 + seed)) for seed in range(6)]
    assert any(r["contact"] for r in out)


def test_torus_sweep_is_safe_and_uses_windows():
    f, p, v, tau_end, _ = S.torus_sweep(16, 8, reach=3.0)
    r = O.ccd_first_contact(f, p, v, tau_end)
    ts = np.linspace(0.0, r["tau_max"], 41)
    mel = S._mean_edge_length(f, p)
    assert min(O.ccd_min_distance(p + t * v, f) for t in ts) >= 0.05 * mel * (1 - 1e-6)
    assert r["windows"] >= 1 and r["pairs_tested"] > 0


def test_band_of_an_embedded_mesh_changes_nothing():
    f, p, v, tau_end, ell = S.embedded_spheres()
    assert len(O.ccd_intersecting_pairs(p, f)) == 0
    a = O.ccd_first_contact(f, p, v, tau_end, reference_length=ell)
    b = O.ccd_first_contact(f, p, v, tau_end, reference_length=ell, band=True)
    assert a["contact"] == 1 and b["band_vertices"] == 0 and b["exempt_pairs"] == 0
    assert {k: a[k] for k in a if k != "band_vertices"} == {k: b[k] for k in b if k != "band_vertices"}


def test_exemption_frees_the_intersection_curve_but_not_other_regions():
    f, p, r = S.overlapping_and_apart()
    ell = S._mean_edge_length(f, p)
    pairs = O.ccd_intersecting_pairs(p, f)
    assert len(pairs) > 0
    nf_sphere = len(f) // 4
    assert (pairs < 2 * nf_sphere).all()  # only faces of A and B intersect
    # B slides along A: the plain CCD stops it at once, the band frees it
    v = np.zeros_like(p)
    v[r[1].start:r[1].stop] = [0.0, 0.0, 0.4]
    plain = O.ccd_first_contact(f, p, v, 1.0, reference_length=ell)
    banded = O.ccd_first_contact(f, p, v, 1.0, reference_length=ell, band=True)
    assert banded["exempt_pairs"] > 0 and banded["band_vertices"] > 0
    assert banded["tau_max"] > plain["tau_max"]
    # C moves into D: the contact is that of C and D alone
    v = np.zeros_like(p)
    v[r[2].start:r[2].stop] = [0.0, 0.0, 1.0]
    banded = O.ccd_first_contact(f, p, v, 3.0, reference_length=ell, band=True)
    fc, pc = S.union(S._sphere(2, [0.0, 0.0, 6.0], 1.0), S._sphere(2, [0.0, 0.0, 9.0], 1.0))
    vc = np.zeros_like(pc)
    vc[: len(pc) // 2] = [0.0, 0.0, 1.0]
    alone = O.ccd_first_contact(fc, pc, vc, 3.0, reference_length=ell)
    assert alone["contact"] == 1 and banded["contact"] == 1
    assert abs(banded["tau_max"] - alone["tau_max"]) < 1e-6 * alone["tau_max"]


def test_coplanar_neighbours_do_not_intersect():
    hits = sum(len(O.ccd_intersecting_pairs(*reversed(S.flat_grid(12, seed)))) for seed in range(10))
    assert hits == 0
    f, p = S.soup([[[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]],
                   [[0.2, 0.2, 0.0], [1.2, 0.2, 0.0], [0.2, 1.2, 0.0]]])
    assert O.ccd_intersecting_pairs(p, f).tolist() == [[0, 1]]
