"""OBJ input and output of triangle meshes (RS/src/io.rs:1-99 over the OBJ reader and writer of
crates/ddg-core/src/io.rs:150-430). Host code: no device work.

* ``parse_obj(text)`` / ``read_obj(path)`` -> (positions V x 3 float64, faces F x 3 uint32).
  ``v``, ``vt`` and polygonal ``f`` statements with corners ``v``, ``v/vt``, ``v//vn`` and
  ``v/vt/vn``; 1-based and negative (relative) indices; ``#`` comments; a trailing backslash
  continues a line; every other statement is skipped. Only triangles are accepted: another
  polygon raises ``RsError`` of kind ``PolygonFace`` naming the face.
* ``obj_to_string(positions, faces)`` / ``write_obj(path, positions, faces)``: a comment line,
  ``v`` lines with every coordinate in its shortest round-trip decimal (no exponent, ``1`` for
  1.0, as the reference formats an f64), and 1-based ``f`` lines.

Positions are read as they are. The functions that use them validate them (finite, no
degenerate face), and the topology too (``validate_surface``, ``BhTree``, ``Flow``).
"""
from __future__ import annotations

from decimal import Decimal
from pathlib import Path

import numpy as np

from . import RsError


def _parse_error(line: int, message: str) -> RsError:
    return RsError(1, "Parse", "io", f"line {line}: {message}")


def _number(token: str, line: int) -> float:
    if "_" in token:  # Python accepts digit separators; an f64 parse does not
        raise _parse_error(line, f"cannot parse '{token}' as a number")
    try:
        x = float(token)
    except ValueError:
        raise _parse_error(line, f"cannot parse '{token}' as a number") from None
    if not np.isfinite(x):
        raise _parse_error(line, f"non-finite number '{token}'")
    return x


def _index(token: str, defined: int, what: str, line: int) -> int:
    """A 1-based or negative OBJ index as a 0-based one; negative indices count back from the
    `defined` elements so far (ddg-core io.rs resolve_index)."""
    try:
        if "_" in token:
            raise ValueError
        i = int(token)
    except ValueError:
        raise _parse_error(line, f"cannot parse '{token}' as a {what} index") from None
    if i > 0:
        if i >= 0xFFFFFFFF:
            raise _parse_error(line, f"{what} index {i} is too large")
        return i - 1
    if i < 0:
        if -i > defined:
            raise _parse_error(line, f"{what} index {i} refers before the first {what} ({defined} defined)")
        return defined + i
    raise _parse_error(line, f"{what} index 0 is not valid (indices start at 1)")


def parse_obj(text: str):
    """(positions, faces) of OBJ text; see the module documentation."""
    positions, texcoords, faces, face_lines = [], [], [], []
    pending, start = None, 0
    lines = text.splitlines()
    stmts = []
    for i, raw in enumerate(lines, 1):
        raw = raw.rstrip()
        if raw.endswith("\\"):
            if pending is None:
                pending, start = [], i
            pending.append(raw[:-1] + " ")
            continue
        if pending is not None:
            pending.append(raw)
            stmts.append(("".join(pending), start))
            pending = None
        else:
            stmts.append((raw, i))
    if pending is not None:
        stmts.append(("".join(pending), start))
    for line, n in stmts:
        tokens = line.split("#", 1)[0].split()
        if not tokens:
            continue
        kw, rest = tokens[0], tokens[1:]
        if kw == "v":
            if len(rest) < 3:
                raise _parse_error(n, f"vertex needs 3 coordinates, found {len(rest)}")
            positions.append([_number(t, n) for t in rest[:3]])
        elif kw == "vt":
            if not rest:
                raise _parse_error(n, "texture coordinate needs at least 1 value")
            texcoords.append([_number(rest[0], n), _number(rest[1], n) if len(rest) > 1 else 0.0])
        elif kw == "f":
            corners = []
            for tok in rest:
                parts = tok.split("/")
                v = _index(parts[0], len(positions), "vertex", n)
                if len(parts) > 1 and parts[1] != "":
                    t = _index(parts[1], len(texcoords), "texture coordinate", n)
                    corners.append((v, t))
                else:
                    corners.append((v, None))
            if len(corners) < 3:
                raise _parse_error(n, f"face has {len(corners)} corners, at least 3 are required")
            faces.append(corners)
            face_lines.append(n)
    for corners, n in zip(faces, face_lines):
        for v, t in corners:
            if v >= len(positions):
                raise _parse_error(n, f"face refers to vertex {v + 1}, but the file defines {len(positions)} vertices")
            if t is not None and t >= len(texcoords):
                raise _parse_error(n, f"face refers to texture coordinate {t + 1}, but the file defines {len(texcoords)}")
    out = np.zeros((len(faces), 3), np.uint32)
    for f, corners in enumerate(faces):
        if len(corners) != 3:
            raise RsError(1, "PolygonFace", "io", f"face {f} has {len(corners)} corners; only triangles are accepted")
        out[f] = [v for v, _ in corners]
    return np.asarray(positions, np.float64).reshape(-1, 3), out


def read_obj(path):
    """(positions, faces) of an OBJ file; see ``parse_obj``."""
    try:
        text = Path(path).read_text()
    except OSError as e:
        raise RsError(1, "Io", "io", f"{path}: {e}") from None
    return parse_obj(text)


def _fmt(x: float) -> str:
    """An f64 as the reference prints it: the shortest round-trip digits in plain decimal."""
    s = format(Decimal(repr(float(x))), "f")
    if "." in s:
        s = s.rstrip("0").rstrip(".")
    return s


def obj_to_string(positions, faces) -> str:
    """OBJ text of a triangle mesh: ``v`` lines, then 1-based ``f`` lines."""
    p = np.asarray(positions, dtype=np.float64).reshape(-1, 3)
    f = np.asarray(faces, dtype=np.int64).reshape(-1, 3)
    bad = np.flatnonzero(~np.isfinite(p).all(axis=1))
    if bad.size:
        raise RsError(1, "NonFinitePosition", "io", f"position of vertex {int(bad[0])} is not finite")
    if f.size and (f.min() < 0 or f.max() >= len(p)):
        raise RsError(1, "InvalidOption", "io", "a face refers to a vertex that does not exist")
    out = ["# written by rs_gb300\n"]
    out += [f"v {_fmt(a)} {_fmt(b)} {_fmt(c)}\n" for a, b, c in p.tolist()]
    out += [f"f {a + 1} {b + 1} {c + 1}\n" for a, b, c in f.tolist()]
    return "".join(out)


def write_obj(path, positions, faces) -> None:
    """Writes ``obj_to_string(positions, faces)`` to `path`."""
    text = obj_to_string(positions, faces)
    try:
        Path(path).write_text(text)
    except OSError as e:
        raise RsError(1, "Io", "io", f"{path}: {e}") from None
