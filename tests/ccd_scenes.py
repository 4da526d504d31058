"""Scenes for the continuous collision detection tests: the known-answer scenes of the
reference's tests (crates/ddg-repulsive-surfaces/tests/ccd.rs:80-390), seeded random triangle
soups, sphere pairs and a noisy torus with a smooth motion. Each scene is
(faces, start, velocity, tau_end, reference_length)."""
import numpy as np


def soup(tris):
    tris = np.asarray(tris, dtype=np.float64).reshape(-1, 3, 3)
    pos = tris.reshape(-1, 3).copy()
    faces = np.arange(len(pos), dtype=np.uint32).reshape(-1, 3)
    return faces, pos


def two_triangles(b, vb):
    """A fixed triangle A in z = 0 and a moving triangle B (tests/ccd.rs:80-89)."""
    a = [[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]]
    faces, pos = soup([a, b])
    vel = np.zeros((6, 3))
    vel[3:] = vb
    return faces, pos, vel


def known_answer_scenes():
    """name -> (faces, start, velocity, tau_end, reference_length, expectation)."""
    s = {}
    f, p, v = two_triangles([[0.2, 0.2, 1.0], [1.0, 1.0, 1.5], [-0.5, 1.2, 1.5]], [0.0, 0.0, -1.0])
    s["head_on_vertex_face"] = (f, p, v, 2.0, 1.0, ("range", 0.94, 0.95 + 1e-9))
    f, p, v = two_triangles([[0.5, -0.5, 1.0], [0.5, 0.5, 1.0], [3.0, 0.0, 1.0]], [0.0, 0.0, -1.0])
    s["edge_edge_crossing"] = (f, p, v, 2.0, 1.0, ("range", 0.94, 0.95 + 1e-9))
    f, p = soup([[[-1.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, -0.01, 0.0]],
                 [[0.005, -1.0, 1.0], [0.005, 1.0, 1.0], [0.015, 0.2, 1.0]]])
    v = np.zeros((6, 3))
    v[3:] = [0.0, 0.0, -1.0]
    s["pure_edge_edge"] = (f, p, v, 2.0, 1.0, ("range", 0.94, 0.95 + 1e-9))
    f, p, v = two_triangles([[0.2, 0.2, 1.0], [1.0, 1.0, 1.0], [-0.5, 1.2, 1.0]], [3.0, 0.0, 0.0])
    s["sliding_past"] = (f, p, v, 5.0, 1.0, ("end",))
    f, p, v = two_triangles([[2.0, 0.5, 0.0], [3.0, 0.5, 0.0], [2.5, 1.5, 0.0]], [-4.0, -1.5, 0.0])
    s["passing_in_plane"] = (f, p, v, 1.0, 1.0, ("any",))
    f, p, v = two_triangles([[0.2, 0.2, 1.0], [1.0, 1.0, 1.0], [-0.5, 1.2, 1.0]], [0.0, 0.0, 0.0])
    s["stationary"] = (f, p, np.zeros((6, 3)), 3.0, 1.0, ("end",))
    s["common_translation"] = (f, p, np.tile([1.0, 2.0, 3.0], (6, 1)), 3.0, 1.0, ("end",))
    f, p, v = two_triangles([[0.2, 0.2, 0.02], [1.0, 1.0, 0.5], [-0.5, 1.2, 0.5]], [0.0, 0.0, -1.0])
    s["initially_close"] = (f, p, v, 2.0, 1.0, ("range", 0.009, 0.01 + 1e-9), ("close", 1))
    s["initially_close_moving_apart"] = (f, p, -v, 2.0, 1.0, ("end",), ("close", 1))
    f, p, v = two_triangles([[0.2, 0.2, 0.0], [1.0, 1.0, 0.5], [-0.5, 1.2, 0.5]], [0.0, 0.0, 1.0])
    s["touching_vertex"] = (f, p, v, 1.0, 1.0, ("end",), ("touching", 1))
    return s


def _mean_edge_length(faces, pos):
    e = np.concatenate([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]]).astype(np.int64)
    e = np.unique(np.sort(e, axis=1), axis=0)
    return float(np.linalg.norm(pos[e[:, 0]] - pos[e[:, 1]], axis=1).sum() / len(e))


def random_soup(seed, k=8):
    """k triangles of side ~0.8 in [0, 2]^3 whose corners move with their own random velocities
    (the shape of the reference's random soups, tests/ccd.rs:258-279, with numpy's generator)."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(0.0, 2.0, (k, 1, 3))
    tris = c + rng.uniform(-0.4, 0.4, (k, 3, 3))
    faces, pos = soup(tris)
    vel = rng.uniform(-1.0, 1.0, (3 * k, 3))
    return faces, pos, vel, 0.6, _mean_edge_length(faces, pos)


def sphere_pair(seed, level=1):
    """A unit icosphere and a second, smaller one above it falling with a tilt
    (the shape of tests/ccd.rs:305-328)."""
    from rs_gb300 import generators as gen

    rng = np.random.default_rng(seed)
    pa, fa = gen.icosphere(level)
    pa = np.asarray(pa, dtype=np.float64)
    c = np.array([rng.uniform(-0.5, 0.5), rng.uniform(-0.5, 0.5), 2.6])
    pb = c + rng.uniform(0.7, 1.0) * pa
    faces = np.concatenate([fa, fa + len(pa)]).astype(np.uint32)
    pos = np.concatenate([pa, pb])
    speed = rng.uniform(0.5, 2.0)
    tilt = rng.uniform(-0.3, 0.3, 2)
    vel = np.zeros_like(pos)
    vel[len(pa):] = [speed * tilt[0], speed * tilt[1], -speed]
    return faces, pos, vel, 2.5, _mean_edge_length(faces, pos)


def torus_sweep(nu=24, nv=12, reach=3.0, seed=5):
    """A noisy torus moving along a smooth, seeded velocity field scaled so that the fastest
    vertex travels `reach` mean edge lengths by tau_end = 1: several windows, many close
    approaches of neighbouring non-adjacent elements."""
    from rs_gb300 import generators as gen

    pos, faces = gen.noisy_torus(nu, nv, 1.0, 0.35, 0.002, seed)
    pos = np.asarray(pos, dtype=np.float64)
    faces = np.asarray(faces, dtype=np.uint32)
    rng = np.random.default_rng(seed)
    k = rng.normal(size=(4, 3))
    ph = rng.uniform(0, 2 * np.pi, (4, 3))
    vel = sum(np.sin(pos @ k[i][:, None] * 2.0 + ph[i]) for i in range(4))
    vel = np.asarray(vel, dtype=np.float64)
    mel = _mean_edge_length(faces, pos)
    vel *= reach * mel / np.linalg.norm(vel, axis=1).max()
    return faces, pos, vel, 1.0, 0.0


def _sphere(level, center, radius):
    from rs_gb300 import generators as gen

    p, f = gen.icosphere(level)
    return np.asarray(f, np.uint32), np.asarray(center) + radius * np.asarray(p, np.float64)


def union(*meshes):
    faces, pos, n = [], [], 0
    for f, p in meshes:
        faces.append(f + n)
        pos.append(p)
        n += len(p)
    return np.concatenate(faces).astype(np.uint32), np.concatenate(pos)


def embedded_spheres():
    """Two level-2 spheres 4 apart moving towards each other (tests/ccd.rs:641-662)."""
    f, p = union(_sphere(2, [0.0, 0.0, 0.0], 1.0), _sphere(2, [4.0, 0.0, 0.0], 1.0))
    n = len(p) // 2
    vel = np.zeros_like(p)
    vel[:n] = [1.0, 0.0, 0.0]
    vel[n:] = [-1.0, 0.0, 0.0]
    return f, p, vel, 3.0, _mean_edge_length(f, p)


def overlapping_and_apart():
    """Overlapping spheres A, B (an intersecting input) and C, D far from them
    (tests/ccd.rs:664-672); returns faces, positions and the vertex ranges of A, B, C, D."""
    parts = [_sphere(2, c, 1.0) for c in ([0.0, 0.0, 0.0], [1.2, 0.0, 0.0], [0.0, 0.0, 6.0], [0.0, 0.0, 9.0])]
    f, p = union(*parts)
    n = len(parts[0][1])
    return f, p, [range(k * n, (k + 1) * n) for k in range(4)]


def flat_grid(n, seed):
    """An n x n grid of squares split into triangles, placed in a random plane."""
    rng = np.random.default_rng(seed)
    i, j = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    uv = np.stack([i.ravel(), j.ravel()], 1) / n
    u, w = rng.uniform(-0.5, 0.5, 3), rng.uniform(-0.5, 0.5, 3)
    pos = 0.3 + uv[:, :1] * u + uv[:, 1:] * w
    idx = lambda a, b: a * (n + 1) + b
    faces = []
    for a in range(n):
        for b in range(n):
            faces.append([idx(a, b), idx(a + 1, b), idx(a + 1, b + 1)])
            faces.append([idx(a, b), idx(a + 1, b + 1), idx(a, b + 1)])
    return np.asarray(faces, np.uint32), pos
