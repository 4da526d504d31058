"""Readers for the golden fixtures committed under tests/golden/ (see make_golden.py)."""
from __future__ import annotations

import json
import struct
from functools import lru_cache
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"


def hexf(s: str) -> float:
    """A double from its 16-digit big-endian hex bit pattern (the Lean fixtures' format)."""
    return struct.unpack(">d", bytes.fromhex(s))[0]


@lru_cache(None)
def lean_cases() -> dict:
    return json.loads((GOLDEN / "lean_rs.json").read_text())


class LeanCase:
    """One Lean-oracle case: the input mesh and exponents, and the output lines by key."""

    def __init__(self, name: str):
        c = lean_cases()[name]
        self.name, self.task = name, c["task"]
        self.alpha, self.beta = 6.0, 12.0
        pos, faces = [], []
        self.inputs: dict[str, list[list[str]]] = {}
        for line in c["in"].splitlines():
            t = line.split()
            if not t:
                continue
            if t[0] == "exponents":
                self.alpha, self.beta = hexf(t[1]), hexf(t[2])
            elif t[0] == "p":
                pos.append([hexf(x) for x in t[1:4]])
            elif t[0] == "f":
                faces.append([int(x) for x in t[1:4]])
            else:
                self.inputs.setdefault(t[0], []).append(t[1:])
        self.positions = np.array(pos, dtype=np.float64).reshape(-1, 3)
        self.faces = np.array(faces, dtype=np.uint32).reshape(-1, 3)
        self.out: dict[str, list[list[str]]] = {}
        for line in c["out"].splitlines():
            t = line.split()
            if t:
                self.out.setdefault(t[0], []).append(t[1:])

    @property
    def status(self) -> str:
        return self.out["status"][0][0]

    @property
    def error_kind(self) -> str | None:
        s = self.out["status"][0]
        return s[1] if s[0] == "error" else None

    def scalar(self, key: str) -> float:
        return hexf(self.out[key][0][0])

    def vectors(self, key: str) -> np.ndarray:
        """Rows ``key i x y z`` as an (n, 3) array ordered by i."""
        rows = sorted(self.out[key], key=lambda r: int(r[0]))
        return np.array([[hexf(x) for x in r[1:]] for r in rows])

    def matrix(self, key: str) -> np.ndarray:
        rows = sorted(self.out[key], key=lambda r: int(r[0]))
        return np.array([[hexf(x) for x in r[1:]] for r in rows])


    def constraint_items(self) -> list[tuple[str, int | None, list[float], list[int]]]:
        """The ``c`` lines in order as (kind, component or None, targets, pinned vertices).

        ``c barycenter all`` holds every component's barycenter separately (the Lean oracle's
        reading, the crate's ``BarycenterMode::PerComponent``)."""
        out = []
        for t in self.inputs.get("c", []):
            kind = t[0]
            if kind == "pins":
                n = int(t[1])
                verts = [int(x) for x in t[2:2 + n]]
                targets = [hexf(x) for x in t[2 + n:]]
                out.append((kind, None, targets, verts))
            else:
                comp = None if t[1] == "all" else int(t[1])
                out.append((kind, comp, [hexf(x) for x in t[2:]], []))
        return out

    def line(self, key: str) -> list[str] | None:
        v = self.inputs.get(key)
        return v[0] if v else None


def lean_names(task: str, status: str | None = "ok") -> list[str]:
    out = []
    for name, c in sorted(lean_cases().items()):
        if c["task"] != task:
            continue
        st = next(l.split()[1] for l in c["out"].splitlines() if l.startswith("status"))
        if status is None or st == status:
            out.append(name)
    return out


@lru_cache(None)
def reference_meshes() -> dict:
    return json.loads((GOLDEN / "reference_meshes.json").read_text())


def reference_mesh(name: str) -> dict:
    """An authors'-program fixture: positions, faces, exponents, energies, differentials."""
    m = reference_meshes()[name]
    pos, faces = [], []
    for line in m["obj"].splitlines():
        t = line.split()
        if not t:
            continue
        if t[0] == "v":
            pos.append([float(x) for x in t[1:4]])
        elif t[0] == "f":
            faces.append([int(x.split("/")[0]) - 1 for x in t[1:4]])
    kv = {}
    for line in m["txt"].splitlines():
        t = line.split()
        if len(t) >= 2:
            kv[t[0]] = float(t[1])

    def triples(text):
        return np.array([[float(x) for x in l.split()] for l in text.splitlines() if l.strip()])

    return dict(positions=np.array(pos), faces=np.array(faces, dtype=np.uint32), alpha=kv["alpha"],
                beta=kv["beta"], theta=kv["theta"], all_pairs=kv["tpe_all_pairs"],
                barnes_hut=kv["tpe_barnes_hut"], d_all=triples(m["dE_all.txt"]),
                d_bh=triples(m["dE_bh.txt"]))


def normwise(got, want, floor=1e-300) -> float:
    """max|got - want| / max(max|want|, floor) -- the reference tests' comparison."""
    got = np.asarray(got, dtype=np.float64).ravel()
    want = np.asarray(want, dtype=np.float64).ravel()
    return float(np.max(np.abs(got - want)) / max(np.max(np.abs(want)), floor)) if want.size else 0.0
