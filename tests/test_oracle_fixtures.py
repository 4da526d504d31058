"""Pins the FP64 oracle to the reference's own golden vectors (CPU only).

* Lean-oracle fixtures (lean/oracle/fixtures/rs, replayed by RS/tests/oracle.rs at 1e-12):
  energy and gradient of every ``energy`` case; error kinds of the error cases.
* The authors' C++ program dumps (RS/tests/reference_fixtures.rs:107-157): all-pairs energy
  1e-12 and differential 1e-11 (normwise); Barnes-Hut at theta 0.5 within the 1e-2 band the
  reference allows (different trees).
* Invariants of RS/tests/energy.rs and RS/tests/barnes_hut.rs: theta = 0 equals the exact
  energy; the BH gradient equals finite differences on frozen lists; scaling and the Euler
  identity; refit equals a fresh evaluation.
"""
import numpy as np
import pytest

import golden_io as G
import rs_oracle as O

ENERGY_TOL = 1e-12
GRAD_TOL = 1e-12


@pytest.mark.parametrize("name", G.lean_names("energy", "ok"))
def test_lean_energy_fixtures(name):
    c = G.LeanCase(name)
    E, dE = O.exact_energy(c.positions, c.faces, c.alpha, c.beta)
    want = c.scalar("energy")
    assert abs(E - want) <= ENERGY_TOL * max(abs(want), 1e-300)
    assert G.normwise(dE, c.vectors("d"), floor=1e-300) <= GRAD_TOL


ERROR_KIND_TO_CODE = {
    "DegenerateFace": 5,
    "InvalidExponents": 1,
    "NonFiniteEnergy": 6,
    "VertexOutOfRange": 7,
}


@pytest.mark.parametrize("name", [n for n in G.lean_names("energy", "error")
                                  if G.LeanCase(n).error_kind in ERROR_KIND_TO_CODE])
def test_lean_energy_error_fixtures(name):
    c = G.LeanCase(name)
    with pytest.raises(O.OracleError) as ei:
        O.exact_energy(c.positions, c.faces, c.alpha, c.beta)
    assert ei.value.code == ERROR_KIND_TO_CODE[c.error_kind]


@pytest.mark.parametrize("name", ["torus192", "torus504", "tube_regular"])
def test_authors_program_fixtures(name):
    m = G.reference_mesh(name)
    E, dE = O.exact_energy(m["positions"], m["faces"], m["alpha"], m["beta"])
    assert abs(E - m["all_pairs"]) / m["all_pairs"] < 1e-12
    assert G.normwise(dE, m["d_all"]) < 1e-11
    bh = O.BhTree(m["positions"], m["faces"], theta=m["theta"])
    Eb, dEb = bh.energy_and_differential(m["alpha"], m["beta"])
    assert abs(Eb - m["barnes_hut"]) / m["barnes_hut"] < 1e-2
    assert G.normwise(dEb, m["d_bh"]) < 1e-2
    # theta = 0 admits nothing: the exact energy up to summation order
    bh0 = O.BhTree(m["positions"], m["faces"], theta=0.0)
    E0, d0 = bh0.energy_and_differential(m["alpha"], m["beta"])
    assert abs(E0 - E) / E < 1e-12
    assert G.normwise(d0, dE) < 1e-11
    # value-only path performs the same operations as the gradient path
    assert bh.energy(m["alpha"], m["beta"]) == Eb


def _small_mesh():
    from rs_gb300 import generators as g

    return g.config_c1()


def test_bh_gradient_matches_finite_differences():
    P, F = _small_mesh()
    bh = O.BhTree(P, F, theta=0.5)
    E, dE = bh.energy_and_differential()
    rng = np.random.default_rng(3)
    for _ in range(4):
        d = rng.standard_normal(P.shape)
        d /= np.linalg.norm(d)
        h = 1e-6
        bh.refit(P + h * d)
        Ep = bh.energy()
        bh.refit(P - h * d)
        Em = bh.energy()
        fd = (Ep - Em) / (2 * h)
        assert abs(fd - np.sum(dE * d)) <= 1e-6 * np.abs(dE).sum()
    bh.refit(P)
    E2, d2 = bh.energy_and_differential()
    assert E2 == E and np.array_equal(d2, dE)  # refit equals the fresh evaluation


def test_energy_identities():
    """sum g = 0, sum f x g = 0, sum f . g = (4 + alpha - beta) E (RS/tests/energy.rs:250)."""
    P, F = _small_mesh()
    E, g = O.exact_energy(P, F, 6.0, 12.0)
    scale = np.abs(g).sum()
    assert np.abs(g.sum(0)).max() < 1e-10 * scale
    assert np.abs(np.cross(P, g).sum(0)).max() < 1e-10 * scale
    assert abs(np.sum(P * g) - (4 + 6 - 12) * E) < 1e-10 * abs(E)
    E2 = O.exact_energy(2.0 * P, F, 6.0, 12.0, gradient=False)
    assert abs(E2 - 2.0 ** (4 + 6 - 12) * E) < 1e-12 * abs(E)


def test_oracle_threads_bitwise():
    P, F = _small_mesh()
    O.set_threads(1)
    a = O.BhTree(P, F, theta=0.25).energy_and_differential()
    O.set_threads(4)
    b = O.BhTree(P, F, theta=0.25).energy_and_differential()
    assert a[0] == b[0] and np.array_equal(a[1], b[1])
