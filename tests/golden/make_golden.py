"""Regenerates the golden fixtures under tests/golden/ from the reference project's own
fixture files (run in a container where the reference is mounted; the tests only read the
JSON written here, never the reference tree).

Sources (data, not code):

* ``lean/oracle/fixtures/rs/*.in|*.out`` -- the Lean Float oracle's answers (bit-exact hex
  doubles) for the tasks ``energy``, ``df``, ``metric``, ``constraints``, ``saddle``,
  ``precond`` and ``step``, replayed by the reference's ``RS/tests/oracle.rs``;
* ``crates/ddg-repulsive-surfaces/tests/fixtures/reference/{torus192,torus504,tube_regular}.*``
  -- dumps of the authors' C++ program (all-pairs and Barnes-Hut energies and differentials),
  replayed by ``RS/tests/reference_fixtures.rs``.

Usage: ``python tests/golden/make_golden.py REFERENCE_ROOT`` (the root of the reference
project's checkout).
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

TASKS = {"energy", "df", "metric", "constraints", "precond", "saddle", "step"}
REF_MESHES = ["torus192", "torus504", "tube_regular"]


def main(root: Path) -> None:
    out_dir = Path(__file__).resolve().parent
    lean = root / "lean" / "oracle" / "fixtures" / "rs"
    cases = {}
    for f_in in sorted(lean.glob("*.in")):
        text_in = f_in.read_text()
        task = next(l.split()[1] for l in text_in.splitlines() if l.startswith("task "))
        if task not in TASKS:
            continue
        text_out = f_in.with_suffix(".out").read_text()
        cases[f_in.stem] = {"task": task, "in": text_in, "out": text_out}
    (out_dir / "lean_rs.json").write_text(json.dumps(cases, indent=0, sort_keys=True))

    ref = root / "crates" / "ddg-repulsive-surfaces" / "tests" / "fixtures" / "reference"
    meshes = {}
    for name in REF_MESHES:
        meshes[name] = {ext: (ref / f"{name}.{ext}").read_text()
                        for ext in ("obj", "txt", "dE_all.txt", "dE_bh.txt")}
    (out_dir / "reference_meshes.json").write_text(json.dumps(meshes, indent=0, sort_keys=True))
    print(f"{len(cases)} Lean cases, {len(meshes)} reference meshes -> {out_dir}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py REFERENCE_ROOT")
    main(Path(sys.argv[1]))
