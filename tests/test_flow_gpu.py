"""One Hs descent step on the GPU (Session::step_inner without remeshing / collisions):
the energy decreases (Armijo), the held area and volume come back to their targets after the
projection (within the crate's NONLINEAR_TOLERANCE, 1e-8 relative), the barycenter stays put,
and the saddle solves converge. A cancel request stops a step cleanly at any point."""
import numpy as np
import pytest

import rs_oracle as O
import rs_gb300 as R
from rs_gb300 import generators as gen

pytestmark = pytest.mark.gpu


def _area_volume(P, F):
    a, _, _ = O.face_geometry(P, F)
    p0, p1, p2 = P[F[:, 0]], P[F[:, 1]], P[F[:, 2]]
    vol = np.sum(np.einsum("ij,ij->i", p0, np.cross(p1, p2))) / 6.0
    return a.sum(), vol


@pytest.mark.parametrize("hold", [(0, 0), (1, 1)])
def test_flow_steps(hold):
    P, F = gen.noisy_torus(48, 24, 1.0, 0.3, 0.003, 7)
    opts = R.flow_options(theta=0.5, hold_area=hold[0], hold_volume=hold[1], solver_tolerance=1e-6,
                          solver_restart=30)
    flow = R.Flow(F, P, opts)
    A0, V0 = _area_volume(P, F)
    a, _, _ = O.face_geometry(P, F)
    energies = []
    for _ in range(3):
        rep = flow.step()
        print(rep)
        assert rep["accepted"] == 1.0
        assert rep["energy_after"] < rep["energy_before"]
        assert rep["relative_residual"] <= 1e-6
        assert rep["slope"] > 0.0
        energies.append(rep["energy_after"])
    Q = flow.positions()
    A1, V1 = _area_volume(Q, F)
    if hold[0]:
        assert abs(A1 - A0) / A0 <= 1e-8
        assert abs(V1 - V0) / abs(V0) <= 1e-8
    mass = np.zeros(len(P))
    np.add.at(mass, F.ravel().astype(np.int64), np.repeat(a / 3.0, 3))
    a1, _, _ = O.face_geometry(Q, F)
    m1 = np.zeros(len(P))
    np.add.at(m1, F.ravel().astype(np.int64), np.repeat(a1 / 3.0, 3))
    b0 = (mass[:, None] * P).sum(0) / mass.sum()
    b1 = (m1[:, None] * Q).sum(0) / m1.sum()
    assert np.abs(b1 - b0).max() < 1e-10
    assert energies == sorted(energies, reverse=True)


def test_two_linked_tori_at_full_size():
    """One step on the geometry of the two-torus configuration: two 400 x 400 tori (640,000
    faces) linked as a Hopf pair, here with N(0, 0.0005) noise (the specified 0.01 is 2.5 minor
    edge lengths and crumples the surface). The global barycenter, total area and volume are
    held; the step is accepted and lowers the energy."""
    P, F = gen.torus(400, 400, 1.0, 0.25)
    Q = np.stack([P[:, 0] + 1.0, -P[:, 2], P[:, 1]], axis=1)
    P2 = np.vstack([P, Q])
    F2 = np.vstack([F, F + len(P)]).astype(np.uint32)
    P2 = P2 + 0.0005 * np.random.default_rng(5).standard_normal(P2.shape)
    assert len(F2) == 640_000
    A0, V0 = _area_volume(P2, F2)
    flow = R.Flow(F2, P2, R.flow_options(theta=0.25, hold_area=1, hold_volume=1))
    rep = flow.step()
    print(rep)
    assert rep["accepted"] == 1.0 and rep["energy_after"] < rep["energy_before"]
    Q2 = flow.positions()
    A1, V1 = _area_volume(Q2, F2)
    assert abs(A1 - A0) / A0 <= 1e-8 and abs(V1 - V0) / abs(V0) <= 1e-8
    a0, _, _ = O.face_geometry(P2, F2)
    a1, _, _ = O.face_geometry(Q2, F2)
    m0, m1 = np.zeros(len(P2)), np.zeros(len(P2))
    np.add.at(m0, F2.ravel().astype(np.int64), np.repeat(a0 / 3.0, 3))
    np.add.at(m1, F2.ravel().astype(np.int64), np.repeat(a1 / 3.0, 3))
    b0 = (m0[:, None] * P2).sum(0) / m0.sum()
    b1 = (m1[:, None] * Q2).sum(0) / m1.sum()
    assert np.abs(b1 - b0).max() < 1e-10


def test_cancel_flag():
    P, F = gen.noisy_torus(32, 16, 1.0, 0.3, 0.003, 2)
    flow = R.Flow(F, P, R.flow_options(theta=0.5))
    flow.step()
    Q = flow.positions()
    flow.cancel(True)
    with pytest.raises(R.RsError) as e:
        flow.step()
    assert e.value.kind == "Cancelled"
    assert flow.positions().tobytes() == Q.tobytes()
    flow.cancel(False)
    assert flow.step()["accepted"] == 1.0


def test_cancel_from_another_thread_during_a_step():
    """The flag set from a second thread while a step runs (between line-search trials the step
    reads it, session.rs:989-998): the step either completes or stops with Cancelled, and then
    the positions are bit for bit those before the step; after clearing the flag the next step
    is accepted. A long line search (an absolute start of 1e6, about 40 halvings on a
    51,200-face torus) gives the request time to land inside it."""
    import threading
    import time

    P, F = gen.noisy_torus(160, 160, 1.0, 0.3, 0.002, 4)
    flow = R.Flow(F, P, R.flow_options(theta=0.5, start_rule=R.START_ABSOLUTE, start_value=1e6,
                                       max_halvings=80))
    outcomes = []
    for delay in (0.05, 0.2, 0.35, 0.5, 0.8):
        before = flow.positions()
        timer = threading.Timer(delay, flow.cancel, args=(True,))
        timer.start()
        try:
            rep = flow.step()
            outcomes.append("completed")
            assert rep["accepted"] == 1.0
        except R.RsError as e:
            assert e.kind == "Cancelled"
            outcomes.append("cancelled")
            assert flow.positions().tobytes() == before.tobytes()
        timer.join()
        flow.cancel(False)
        time.sleep(0.01)
    print(outcomes)
    assert flow.step()["accepted"] == 1.0


def test_recovery_repeats_a_diverged_solve():
    """The recovery of RobustHierarchical (RS/src/step/direction.rs:269-379): a step whose solves
    end above the divergence threshold (here: one iteration allowed) is solved again with
    restart 60 and at least 800 iterations, counted in the report, and the step proceeds."""
    P, F = gen.noisy_torus(32, 16, 1.0, 0.3, 0.003, 2)
    flow = R.Flow(F, P, R.flow_options(theta=0.5, hold_volume=1, solver_max_iterations=1, solver_tolerance=1e-6))
    rep = flow.step()
    print(rep)
    assert rep["fallbacks"] == 1.0
    assert rep["accepted"] == 1.0 and rep["relative_residual"] <= 1e-6


def test_recovery_ends_with_the_dense_lu():
    """The whole recovery chain (RobustHierarchical::escalate, direction.rs:269-379): when the
    restart-60 retry diverges too (here one iteration each), a mesh of at most 6000 vertices
    is solved by the dense LU of the exact metric; both escalations are counted and the step
    proceeds with a direction that solves the dense system."""
    P, F = gen.noisy_torus(32, 16, 1.0, 0.3, 0.003, 2)
    flow = R.Flow(F, P, R.flow_options(theta=0.5, hold_volume=1, solver_max_iterations=1, solver_tolerance=1e-6,
                                       retry_max_iterations=1))
    rep = flow.step()
    print(rep)
    assert rep["fallbacks"] == 2.0
    assert rep["accepted"] == 1.0 and rep["relative_residual"] <= 1e-10
    # without the last stage the step fails with SolverDiverged
    flow = R.Flow(F, P, R.flow_options(theta=0.5, hold_volume=1, solver_max_iterations=1, solver_tolerance=1e-6,
                                       retry_max_iterations=1, dense_fallback=0))
    with pytest.raises(R.RsError) as e:
        flow.step()
    assert e.value.kind == "SolverDiverged"
