"""Training of the learned preconditioner (no crate counterpart) on residual/solution pairs
that the plain solver produces on seeded meshes.

For every training mesh a plain solver (the fractional preconditioner, L'^-1 by multigrid CG)
solves A' z = r to a tight tolerance for residuals r drawn from the flow's own right-hand sides
(the energy differential, the area and volume gradients) mixed with seeded smooth fields and
noise; the cheap plain preconditioner gives y = P_cheap^-1 r. The network learns
z - y from (surface, r, y) with the relative squared error |z_pred - z|^2 / |z|^2, by the
library's hand-written forward/backward kernels and Adam (the relative error is taken against
the larger of |z| and |y|). The trained parameters are a flat
float32 array (``LearnedModel.get_parameters``), saved with ``save`` and read with ``load``.
"""
from __future__ import annotations

import time
from pathlib import Path

import numpy as np

from . import generators as gen

PARAMS_FILE = Path(__file__).resolve().parent / "learned_params.npy"


def _constraint_gradients(P, F):
    """Area and volume gradients per vertex (ConstraintSet, RS/src/constraints/mod.rs:519-655)."""
    Fi = F.astype(np.int64)
    p0, p1, p2 = P[Fi[:, 0]], P[Fi[:, 1]], P[Fi[:, 2]]
    n = np.cross(p1 - p0, p2 - p0)
    N = n / np.linalg.norm(n, axis=1)[:, None]
    ga = np.zeros_like(P)
    gv = np.zeros_like(P)
    for c, (a, b) in enumerate([(1, 2), (2, 0), (0, 1)]):
        np.add.at(ga, Fi[:, c], 0.5 * np.cross(N, P[Fi[:, b]] - P[Fi[:, a]]))
        np.add.at(gv, Fi[:, c], np.cross(P[Fi[:, a]], P[Fi[:, b]]) / 6.0)
    return ga, gv


# (major, minor) grid sizes of the training tori: 20,000 to 204,800 faces, up to the size of
# the 320 x 320 evaluation torus, so that the network sees the global smooth error of the
# largest surfaces it preconditions.
TRAIN_TORI = [(100, 100), (160, 100), (200, 128), (240, 160), (256, 200), (288, 240), (320, 320)]


def training_meshes(count: int = 8, seed: int = 100):
    """Seeded noisy tori and jittered icospheres: mesh i is an icosphere when i % 4 == 3 (level 5
    or 6: 20,480 or 81,920 faces), otherwise the torus of TRAIN_TORI taken in turn from the
    largest (204,800 faces) down, so that eight meshes span 20,000-204,800 faces; torus noise
    0.1-0.3 of the minor edge."""
    rng = np.random.default_rng(seed)
    out = []
    tori = TRAIN_TORI[::-1]
    t = 0
    for i in range(count):
        s = int(rng.integers(1 << 30))
        if i % 4 == 3:
            P, F = gen.icosphere(5 if (i // 4) % 2 else 6)
            P = P * (1.0 + float(rng.uniform(0.005, 0.02)) * gen.SplitMix64(s).normals(len(P))[:, None])
        else:
            nu, nv = tori[t % len(tori)]
            t += 1
            r = float(rng.uniform(0.25, 0.4))
            edge = 2.0 * np.pi * r / nv
            P, F = gen.noisy_torus(nu, nv, 1.0, r, float(rng.uniform(0.1, 0.3)) * edge, s)
        out.append((P, F))
    return out


def residuals(P, F, dE, count, rng):
    """Right-hand sides: mixtures of the flow's vectors, smooth fields and noise, unit norm."""
    ga, gv = _constraint_gradients(P, F)
    base = [dE, ga, gv]
    out = []
    for _ in range(count):
        r = np.zeros_like(P)
        for b in base:
            r += rng.standard_normal() * b / max(np.linalg.norm(b), 1e-300)
        for _ in range(3):
            k = rng.uniform(1.0, 12.0, size=3)
            ph = rng.uniform(0, 2 * np.pi, size=3)
            f = np.sin(P @ k + ph[0])[:, None] * rng.standard_normal(3)[None, :]
            r += rng.uniform(0.0, 1.0) * f / max(np.linalg.norm(f), 1e-300)
        noise = rng.standard_normal(P.shape)
        r += rng.uniform(0.0, 0.5) * noise / np.linalg.norm(noise)
        out.append((r / np.linalg.norm(r)).ravel())
    return out


def make_dataset(R, ctx, meshes, per_mesh: int, cheap_steps: int = 2, seed: int = 7, log=print):
    """[(graph, r, y, z)] with r, y, z device tensors (3V, float64)."""
    import torch

    rng = np.random.default_rng(seed)
    data = []
    dev = torch.device("cuda")
    for mi, (P, F) in enumerate(meshes):
        t0 = time.time()
        bh = R.BhTree.build(F, P, R.BhOptions(0.25), ctx)
        _, dE = bh.energy_and_differential()
        S = R.SaddleSolver(F, P, R.Exponents(), R.solver_options(tolerance=1e-7, restart=60, max_iterations=800), ctx)
        Sc = R.SaddleSolver(F, P, R.Exponents(), R.solver_options(vcycles=cheap_steps), ctx)
        g = R.SurfaceGraph(F, P, ctx)
        # batches of four right-hand sides until the mesh holds per_mesh pairs (a solve that misses
        # the tolerance is dropped and replaced), at most three times the batches needed
        kept, tries = 0, 0
        while kept < per_mesh and tries < 3 * ((per_mesh + 3) // 4):
            tries += 1
            batch = residuals(P, F, dE, min(4, per_mesh - kept), rng)
            rhs = np.zeros((len(batch), S.n))
            for k, r in enumerate(batch):
                rhs[k, :S.n_dofs] = r
            try:
                z, reps = S.solve_many(rhs)
            except R.RsError:
                continue
            y = Sc.precondition(rhs)
            for k, r in enumerate(batch):
                if not reps[k]["converged"]:
                    continue
                kept += 1
                data.append((g, torch.tensor(r, device=dev), torch.tensor(y[k, :S.n_dofs].copy(), device=dev),
                             torch.tensor(z[k, :S.n_dofs].copy(), device=dev)))
        log(f"mesh {mi}: {len(F)} faces, {len(data)} pairs, {time.time() - t0:.1f} s")
    return data


def train(model, data, epochs: int = 10, lr: float = 2e-3, batch: int = 8, seed: int = 0, log=print):
    """Adam over the pairs in seeded random order; returns the mean loss per epoch."""
    import torch

    rng = np.random.default_rng(seed)
    torch.cuda.synchronize()
    history = []
    for ep in range(epochs):
        order = rng.permutation(len(data))
        tot, cnt = 0.0, 0
        step_lr = lr * 0.5 * (1 + np.cos(np.pi * ep / max(epochs, 1)))
        for i, k in enumerate(order):
            g, r, y, z = data[k]
            tot += model.loss_and_gradient_device(g, r.data_ptr(), y.data_ptr(), z.data_ptr())
            cnt += 1
            if cnt % batch == 0 or i + 1 == len(order):
                model.adam_step(step_lr, 1.0)
        history.append(tot / max(cnt, 1))
        log(f"epoch {ep}: loss {history[-1]:.4f}")
    return history


def save(model, path: Path = PARAMS_FILE) -> None:
    np.save(path, model.get_parameters())


def load(model, path: Path = PARAMS_FILE) -> bool:
    if not Path(path).exists():
        return False
    model.set_parameters(np.load(path))
    return True


def main(argv=None) -> int:
    """Generates the pairs, trains, evaluates on held-out pairs and writes PARAMS_FILE:
    python -m rs_gb300.learned [--meshes 8] [--per-mesh 250] [--epochs 20]."""
    import argparse

    import rs_gb300 as R

    ap = argparse.ArgumentParser()
    ap.add_argument("--meshes", type=int, default=8)
    ap.add_argument("--per-mesh", type=int, default=250)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--cheap-steps", type=int, default=2)
    ap.add_argument("--out", default=str(PARAMS_FILE))
    args = ap.parse_args(argv)
    ctx = R.Context(0)
    meshes = training_meshes(args.meshes + 1)
    data = make_dataset(R, ctx, meshes[:-1], args.per_mesh, args.cheap_steps)
    held = make_dataset(R, ctx, meshes[-1:], 32, args.cheap_steps, seed=99)
    model = R.LearnedModel(seed=1, ctx=ctx)
    train(model, data, args.epochs, args.lr)
    import torch

    torch.cuda.synchronize()
    w = model.get_parameters()
    lh = []
    for g, r, y, z in held:
        lh.append(model.loss_and_gradient_device(g, r.data_ptr(), y.data_ptr(), z.data_ptr()))
    model.set_parameters(w)  # clears the gradient of the evaluation
    base = [float(((y - z) ** 2).sum() / max((z ** 2).sum(), (y ** 2).sum())) for g, r, y, z in held]
    print(f"held-out: loss {np.mean(lh):.4f} (cheap preconditioner alone {np.mean(base):.4f})")
    save(model, Path(args.out))
    return 0


if __name__ == "__main__":
    import sys

    sys.exit(main())
