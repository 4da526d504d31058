"""The learned preconditioner's hand-written kernels against a plain PyTorch fp32 reference of
the same network (CPU autograd): forward output, loss and parameter gradient of one sample,
the Adam step, and its use as the flexible-GMRES preconditioner with the plain fallback."""
import numpy as np
import pytest

import rs_gb300 as R
from rs_gb300 import generators as gen

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

H, IN, OUT = 64, 13, 3


def unpack(w):
    """The parameter layout of rs_learned: W1s W1n b1 W2s W2n b2 W3s W3n b3 (row-major [out][in])."""
    sizes = [(H, IN), (H, IN), (H,), (H, H), (H, H), (H,), (OUT, H), (OUT, H), (OUT,)]
    out, k = [], 0
    for s in sizes:
        n = int(np.prod(s))
        out.append(w[k:k + n].reshape(s))
        k += n
    assert k == len(w)
    return out


def one_ring(F, nv):
    nb = [set() for _ in range(nv)]
    for a, b, c in F.astype(np.int64):
        for x, y in ((a, b), (b, c), (c, a)):
            nb[x].add(y), nb[y].add(x)
    rows = np.concatenate([[v] * len(s) for v, s in enumerate(nb)]).astype(np.int64)
    cols = np.concatenate([sorted(s) for s in nb]).astype(np.int64)
    deg = np.array([len(s) for s in nb], np.float32)
    A = torch.sparse_coo_tensor(torch.tensor(np.stack([rows, cols])), torch.tensor(1.0 / deg[rows]),
                                (nv, nv)).coalesce()
    return A


def static_features(P, F):
    import rs_oracle as O
    a, N, _ = O.face_geometry(P, F)
    nv = len(P)
    area = np.zeros(nv)
    nrm = np.zeros((nv, 3))
    Fi = F.astype(np.int64)
    for c in range(3):
        np.add.at(area, Fi[:, c], a / 3.0)
        np.add.at(nrm, Fi[:, c], a[:, None] * N)
    cen = P.mean(0)
    R_ = np.sqrt(((P - cen) ** 2).sum(1).mean())
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    return np.concatenate([(P - cen) / R_, nrm, (area / area.mean())[:, None]], 1).astype(np.float32)


def reference(w, stat, A, r, y, zt=None):
    """Forward (BF16-rounded weights, fp32 arithmetic), and loss + gradient if zt is given."""
    wt = torch.tensor(w, dtype=torch.float32).to(torch.bfloat16).to(torch.float32).requires_grad_(True)
    W1s, W1n, b1, W2s, W2n, b2, W3s, W3n, b3 = unpack(wt)
    rr = r.reshape(-1, 3)
    yy = y.reshape(-1, 3)
    sr = float(np.sqrt((r ** 2).mean()))
    sy = float(np.sqrt((y ** 2).mean()))
    X = torch.tensor(np.concatenate([stat, rr / sr, yy / sy], 1), dtype=torch.float32)
    silu = torch.nn.functional.silu
    h1 = silu(X @ W1s.T + torch.sparse.mm(A, X) @ W1n.T + b1)
    h2 = silu(h1 @ W2s.T + torch.sparse.mm(A, h1) @ W2n.T + b2)
    o = h2 @ W3s.T + torch.sparse.mm(A, h2) @ W3n.T + b3
    z = torch.tensor(yy) + sy * o.double()
    if zt is None:
        return z.detach().numpy().ravel(), None, None
    ztt = torch.tensor(zt.reshape(-1, 3))
    loss = ((z - ztt) ** 2).sum() / max(float((ztt ** 2).sum()), float((torch.tensor(yy) ** 2).sum()))
    loss.backward()
    return z.detach().numpy().ravel(), float(loss.detach()), wt.grad.numpy().astype(np.float64)


@pytest.fixture(scope="module")
def setup():
    ctx = R.Context(0)
    P, F = gen.noisy_torus(40, 20, 1.0, 0.35, 0.004, 21)
    g = R.SurfaceGraph(F, P, ctx)
    m = R.LearnedModel(seed=3, ctx=ctx)
    w = m.get_parameters()
    rng = np.random.default_rng(5)
    w = (w + 0.05 * rng.standard_normal(w.size)).astype(np.float32)  # an output layer far from zero
    m.set_parameters(w)
    return ctx, P, F, g, m, w


def test_forward_matches_torch(setup):
    ctx, P, F, g, m, w = setup
    rng = np.random.default_rng(1)
    r = rng.standard_normal(3 * len(P))
    y = rng.standard_normal(3 * len(P)) * 0.1
    rd, yd = torch.tensor(r).cuda(), torch.tensor(y).cuda()
    zd = torch.zeros_like(rd)
    torch.cuda.synchronize()
    m.apply_device(g, 1, rd.data_ptr(), yd.data_ptr(), zd.data_ptr())
    ctx.synchronize()
    z_ref, _, _ = reference(w, static_features(P, F), one_ring(F, len(P)), r, y)
    z = zd.cpu().numpy()
    assert np.linalg.norm(z - z_ref) <= 1e-5 * np.linalg.norm(z_ref)


def test_loss_and_gradient_match_torch(setup):
    ctx, P, F, g, m, w = setup
    rng = np.random.default_rng(2)
    r = rng.standard_normal(3 * len(P))
    y = rng.standard_normal(3 * len(P)) * 0.1
    zt = y + 0.02 * rng.standard_normal(3 * len(P))
    rd, yd, zd = (torch.tensor(v).cuda() for v in (r, y, zt))
    torch.cuda.synchronize()
    m.set_parameters(w)  # clears the accumulated gradient
    loss = m.loss_and_gradient_device(g, rd.data_ptr(), yd.data_ptr(), zd.data_ptr())
    _, loss_ref, grad_ref = reference(w, static_features(P, F), one_ring(F, len(P)), r, y, zt)
    assert abs(loss - loss_ref) <= 1e-5 * abs(loss_ref)
    grad = m.get_gradient().astype(np.float64)
    assert np.linalg.norm(grad - grad_ref) <= 1e-3 * np.linalg.norm(grad_ref)
    # a second sample accumulates
    m.loss_and_gradient_device(g, rd.data_ptr(), yd.data_ptr(), zd.data_ptr())
    assert np.linalg.norm(m.get_gradient() - 2 * grad) <= 1e-5 * np.linalg.norm(grad)


def test_training_reduces_the_loss(setup):
    ctx, P, F, g, m, w = setup
    rng = np.random.default_rng(3)
    r = rng.standard_normal(3 * len(P))
    y = rng.standard_normal(3 * len(P)) * 0.1
    zt = y + 0.05 * np.repeat(np.sin(3 * P[:, :1]), 3, 1).ravel()
    rd, yd, zd = (torch.tensor(v).cuda() for v in (r, y, zt))
    torch.cuda.synchronize()
    m.set_parameters(w)
    first = m.loss_and_gradient_device(g, rd.data_ptr(), yd.data_ptr(), zd.data_ptr())
    m.adam_step(3e-3, 1.0)
    for _ in range(60):
        last = m.loss_and_gradient_device(g, rd.data_ptr(), yd.data_ptr(), zd.data_ptr())
        m.adam_step(3e-3, 1.0)
    assert last < 0.5 * first


def test_learned_preconditioner_solves_with_fallback(setup):
    ctx, P, F, g, m, w = setup
    S = R.SaddleSolver(F, P, R.Exponents(), R.solver_options(tolerance=1e-6), ctx)
    rhs = np.zeros((1, S.n))
    rhs[0, :S.n_dofs] = np.random.default_rng(4).standard_normal(S.n_dofs)
    y_plain, rep_plain = S.solve_many(rhs)
    S.set_learned(m, g, cheap_steps=2, max_iterations=40)
    y, rep = S.solve_many(rhs)
    assert rep[0]["converged"] and rep[0]["relative_residual"] <= 1e-6
    solves, fallbacks = S.learned_counts()
    assert solves == 1 and fallbacks in (0, 1)
    assert np.linalg.norm(y - y_plain) <= 1e-4 * np.linalg.norm(y_plain)


def _ring_correlation(F, nv, e, rings=8, samples=64, seed=0):
    """corr[k] = mean over sampled vertices v of the mean over the vertices u at one-ring
    distance k of e_u . e_v / |e_v|^2 (so corr[0] = 1): how far the error field e stays
    correlated across the surface."""
    import scipy.sparse as sp
    Fi = F.astype(np.int64)
    rows = np.concatenate([Fi[:, 0], Fi[:, 1], Fi[:, 2], Fi[:, 1], Fi[:, 2], Fi[:, 0]])
    cols = np.concatenate([Fi[:, 1], Fi[:, 2], Fi[:, 0], Fi[:, 0], Fi[:, 1], Fi[:, 2]])
    A = sp.csr_matrix((np.ones(len(rows)), (rows, cols)), shape=(nv, nv))
    E = e.reshape(-1, 3)
    rng = np.random.default_rng(seed)
    acc = np.zeros(rings + 1)
    for v in rng.choice(nv, samples, replace=False):
        ev = E[v]
        den = float(ev @ ev)
        if den == 0.0:
            continue
        seen = {int(v)}
        front = np.array([v])
        acc[0] += 1.0
        for k in range(1, rings + 1):
            nxt = np.unique(A[front].indices)
            nxt = np.array([u for u in nxt if int(u) not in seen])
            if len(nxt) == 0:
                break
            seen.update(int(u) for u in nxt)
            acc[k] += float((E[nxt] @ ev).mean()) / den
            front = nxt
    return acc / samples


def test_held_out_c4_evaluation():
    """The trained network (rs_gb300/learned_params.npy) as the flexible-GMRES preconditioner on
    held-out seeded 204,800-face tori (320 x 320, R = 1, r = 0.3, N(0, 0.001) noise, seeds
    1000-1009, none of them a training mesh) at relative residual 1e-6 on the energy
    differential. Every solve in the production setting (learned, capped at 100 iterations,
    then the plain fallback) reaches the tolerance and the plain solution. Printed beside it,
    on the wall clock of the whole call: the plain solver (6 CG steps in L'^-1), the cheap
    preconditioner alone (2 CG steps) and the cheap preconditioner with the network, both
    uncapped: the ablation of what the network adds to the method it corrects. Also printed:
    the network's and the cheap preconditioner's error against the tight solution (relative
    squared error after the best scaling) and the one-ring correlation of the cheap
    preconditioner's error, which shows how far beyond the network's three-ring receptive
    field that error reaches."""
    import time

    from rs_gb300 import learned as L
    ctx = R.Context(0)
    m = R.LearnedModel(seed=0, ctx=ctx)
    assert L.load(m), "no trained parameters"
    rows = []
    corr = None

    def timed(S, rhs):
        t = time.perf_counter()
        y, rep = S.solve_many(rhs)
        return y, rep[0], time.perf_counter() - t

    for seed in range(1000, 1010):
        P, F = gen.noisy_torus(320, 320, 1.0, 0.3, 0.001, seed)
        bh = R.BhTree.build(F, P, R.BhOptions(0.25), ctx)
        dE = np.ravel(bh.energy_and_differential()[1])
        S = R.SaddleSolver(F, P, R.Exponents(), R.solver_options(tolerance=1e-6), ctx)
        rhs = np.zeros((1, S.n))
        rhs[0, :S.n_dofs] = dE
        y0, rep0, t0 = timed(S, rhs)
        assert rep0["converged"]
        g = R.SurfaceGraph(F, P, ctx)
        # production setting: learned capped at 100 iterations, plain fallback
        S.set_learned(m, g, cheap_steps=2, max_iterations=100)
        y1, rep1, t1 = timed(S, rhs)
        _, fallbacks = S.learned_counts()
        assert rep1["converged"] and rep1["relative_residual"] <= 1e-6
        assert np.linalg.norm(y1 - y0) <= 1e-4 * np.linalg.norm(y0)
        # ablation: the cheap preconditioner with and without the network, uncapped
        Sc = R.SaddleSolver(F, P, R.Exponents(), R.solver_options(tolerance=1e-6, vcycles=2, max_iterations=600), ctx)
        _, repc, tc = timed(Sc, rhs)
        yc = Sc.precondition(rhs)[0, :S.n_dofs]
        Sc.set_learned(m, g, cheap_steps=2, max_iterations=0)
        _, repl, tl = timed(Sc, rhs)
        _, lfb = Sc.learned_counts()
        # the network against the cheap preconditioner alone, on the tight solution
        St = R.SaddleSolver(F, P, R.Exponents(), R.solver_options(tolerance=1e-9, restart=60, max_iterations=600),
                            ctx)
        z, _ = St.solve_many(rhs)
        zt = z[0, :S.n_dofs]
        rd, yd = torch.tensor(dE).cuda(), torch.tensor(yc).cuda()
        zd = torch.zeros_like(rd)
        torch.cuda.synchronize()
        m.apply_device(g, 1, rd.data_ptr(), yd.data_ptr(), zd.data_ptr())
        ctx.synchronize()
        zp = zd.cpu().numpy()

        def rel(u):  # after the best scaling (a preconditioner's scale is free)
            a = float(u @ zt) / float(u @ u)
            return float(np.linalg.norm(a * u - zt) ** 2 / np.linalg.norm(zt) ** 2)
        if corr is None:
            corr = _ring_correlation(F, len(P), zt - yc * float(yc @ zt) / float(yc @ yc))
        rows.append((seed, rep0["iterations"], t0, t1, fallbacks, repc["iterations"], tc,
                     repl["iterations"] if lfb == 0 else -1, tl, rel(yc), rel(zp)))
    print("\nseed | plain it s | production s fallbacks | cheap it s | cheap+network it s | "
          "rel.sq.error cheap network")
    for r in rows:
        print(f"{r[0]} | {r[1]:4d} {r[2]:.3f} | {r[3]:.3f} {r[4]} | {r[5]:4d} {r[6]:.3f} | {r[7]:4d} {r[8]:.3f} | "
              f"{r[9]:.4f} {r[10]:.4f}")
    print(f"production / plain time: {sum(r[3] for r in rows) / sum(r[2] for r in rows):.2f}; "
          f"cheap+network / cheap time: {sum(r[8] for r in rows) / sum(r[6] for r in rows):.2f}")
    print("error correlation by ring: " + " ".join(f"{c:.2f}" for c in corr))
