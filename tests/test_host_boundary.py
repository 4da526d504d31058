"""CPU tests of the product library's host side: it loads, exports every symbol of
include/rsgpu.h, validates surfaces with the crate's error kinds, and builds the face BVH
bit for bit as the oracle (no device work)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import golden_io as G
import rs_oracle as O
import rs_gb300 as R
from rs_gb300 import generators as gen

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    text = "\n".join(p.read_text() for p in (ROOT / "include").glob("*.h"))
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rs_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = R.load_library()
    names = declared_symbols()
    assert len(names) > 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


@pytest.mark.parametrize("name", G.lean_names("energy", "error"))
def test_surface_validation_error_kinds(name):
    c = G.LeanCase(name)
    kind = c.error_kind
    if kind in ("InvalidExponents", "NonFiniteEnergy"):
        R.validate_surface(c.faces, c.positions)  # raised by the energy, not the surface
        return
    with pytest.raises(R.RsError) as ei:
        R.validate_surface(c.faces, c.positions)
    assert ei.value.kind == kind


def test_surface_validation_accepts_fixture_meshes():
    for name in G.lean_names("energy", "ok"):
        c = G.LeanCase(name)
        R.validate_surface(c.faces, c.positions)


def test_topology_errors():
    P, F = gen.icosphere(1)
    with pytest.raises(R.RsError, match="RepeatedVertex"):
        R.validate_surface(np.vstack([F, [[0, 0, 1]]]), P)
    with pytest.raises(R.RsError, match="DuplicateFace"):
        R.validate_surface(np.vstack([F, F[3][::-1][None]]), P)
    with pytest.raises(R.RsError, match="NoFaces"):
        R.validate_surface(np.zeros((0, 3), np.uint32), P)
    Q = P.copy()
    Q[F[5][1]] = Q[F[5][0]]
    with pytest.raises(R.RsError, match="DegenerateFace"):
        R.validate_surface(F, Q)
    Q = P.copy()
    Q[2, 1] = np.nan
    with pytest.raises(R.RsError, match="NonFinitePosition"):
        R.validate_surface(F, Q)


def _meshes():
    yield "c1", gen.config_c1()
    yield "c2-level4", gen.config_c2(level=4)
    yield "torus40", gen.noisy_torus(40, 24, 1.0, 0.3, 0.01, 11)
    for name in ["torus192", "tube_regular"]:
        m = G.reference_mesh(name)
        yield name, (m["positions"], m["faces"])
    for name in G.lean_names("energy", "ok"):
        c = G.LeanCase(name)
        yield name, (c.positions, c.faces)


@pytest.mark.parametrize("name,mesh", list(_meshes()))
@pytest.mark.parametrize("leaf", [1, 3, 8])
def test_face_tree_matches_oracle_bitwise(name, mesh, leaf):
    P, F = mesh
    T = R.face_tree(F, P, leaf_size=leaf)
    bh = O.BhTree(P, F, theta=0.5, leaf_size=leaf)
    U, Cl = bh.tree(), bh.clusters()
    for k in ("start", "end", "right", "order"):
        assert np.array_equal(T[k], U[k]), k
    assert np.array_equal(T["box"], Cl["bbox"])
    assert np.array_equal(T["radius"], Cl["radius"])


@pytest.mark.parametrize("name", ["c2", "c3s"])
def test_large_face_tree_matches_oracle_bitwise(name):
    """Sizes where the build sorts the three axes concurrently and splits the top subtrees as
    parallel tasks (81,920 and 204,800 faces)."""
    P, F = gen.CONFIGS[name]()
    T = R.face_tree(F, P, leaf_size=8)
    bh = O.BhTree(P, F, theta=0.5, leaf_size=8)
    U = bh.tree()
    for k in ("start", "end", "right", "order"):
        assert np.array_equal(T[k], U[k]), k


def test_generators_match_reference_recipes():
    P, F = gen.icosphere(3)
    assert P.shape == (642, 3) and F.shape == (1280, 3)
    assert np.allclose(np.linalg.norm(P, axis=1), 1.0)
    P, F = gen.torus(6, 4, 1.0, 0.3)
    assert P.shape == (24, 3) and F.shape == (48, 3)
    assert F[0].tolist() == [0, 4, 5] and F[1].tolist() == [0, 5, 1]
    r = gen.SplitMix64(1)
    seq = [r.next_u64() for _ in range(3)]
    assert np.array_equal(gen.SplitMix64(1).draws(3), np.array(seq, dtype=np.uint64))


@pytest.mark.parametrize("py_name, c_name", [("SolverOptions", "rs_solver_options"),
                                             ("FlowOptions", "rs_flow_options"),
                                             ("CcdOptions", "rs_ccd_options")])
def test_option_structs_match_the_header(tmp_path, py_name, c_name):
    """The ctypes mirrors of the option structs have the C header's size and field offsets
    (compiled against include/rsgpu.h with the host compiler)."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    py = getattr(R, py_name)
    fields = [f[0] for f in py._fields_]
    src = tmp_path / "layout.c"
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "rsgpu.h"', "int main(void) {",
             f'  printf("%zu\\n", sizeof({c_name}));']
    lines += [f'  printf("%zu\\n", offsetof({c_name}, {f}));' for f in fields]
    lines += ["  return 0;", "}"]
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    inc = Path(__file__).resolve().parents[1] / "include"
    subprocess.run([cc, f"-I{inc}", str(src), "-o", str(exe)], check=True, capture_output=True)
    out = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert out[0] == C.sizeof(py)
    assert out[1:] == [getattr(py, f).offset for f in fields]
