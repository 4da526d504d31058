"""OBJ input and output (RS/src/io.rs over crates/ddg-core/src/io.rs:150-430) on the CPU."""
import numpy as np
import pytest

import rs_gb300 as R
from rs_gb300 import generators as gen
from rs_gb300 import obj


def test_round_trip_is_exact(tmp_path):
    P, F = gen.noisy_torus(16, 8, 1.0, 0.3, 0.01, 4)
    obj.write_obj(tmp_path / "t.obj", P, F)
    Q, G = obj.read_obj(tmp_path / "t.obj")
    assert Q.tobytes() == np.ascontiguousarray(P, np.float64).tobytes()
    assert G.tolist() == np.asarray(F).tolist()


@pytest.mark.parametrize("x, s", [(1.0, "1"), (-0.0, "-0"), (0.1, "0.1"), (1e-7, "0.0000001"),
                                  (1e22, "10000000000000000000000"), (123.456, "123.456"), (-2.5, "-2.5")])
def test_numbers_are_written_as_the_reference_prints_them(x, s):
    assert obj._fmt(x) == s


def test_parser_features():
    text = """# a comment
v 0 0 0
v 1 0 0 # trailing comment
v 0 1 0 1.0
vt 0.5
vn 0 0 1
v 0 0 \\
  1
f 1/1 2//1 3/1/1
f -4 -2 -1
g group ignored
"""
    P, F = obj.parse_obj(text)
    assert P.tolist() == [[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]]
    assert F.tolist() == [[0, 1, 2], [0, 2, 3]]


@pytest.mark.parametrize("text, kind, what", [
    ("v 0 0 0\nv 1 0 0\nv 0 1 0\nv 1 1 0\nf 1 2 4 3\n", "PolygonFace", "face 0"),
    ("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 0\n", "Parse", "line 4"),
    ("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 5\n", "Parse", "line 4"),
    ("v 0 0\n", "Parse", "line 1"),
    ("v 0 inf 0\n", "Parse", "line 1"),
    ("v 0 0 0\nf 1 2\n", "Parse", "line 2"),
    ("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 -4\n", "Parse", "line 4"),
])
def test_errors_name_the_line_or_face(text, kind, what):
    with pytest.raises(R.RsError) as e:
        obj.parse_obj(text)
    assert e.value.kind == kind and what in str(e.value)


def test_writer_rejects_bad_input():
    with pytest.raises(R.RsError):
        obj.obj_to_string([[0, 0, np.nan]], [[0, 0, 0]])
    with pytest.raises(R.RsError):
        obj.obj_to_string([[0, 0, 0]], [[0, 1, 2]])
