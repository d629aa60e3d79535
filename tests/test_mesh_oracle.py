"""OBJ input on the CPU: the library's reader (crt_obj_parse, host code) against
the oracle's restatement of Mesh::load (srcCommon/scene/geometry/mesh.cpp:
186-263), on generated OBJ text in every corner syntax and, where the
reference checkout exists, on the reference's own model files."""
import os

import numpy as np
import pytest

from oracle import obj_oracle as OO
from realtimeraytracing_gb300 import crt
from realtimeraytracing_gb300 import scenes as S

from oracle import oracle as O

MODELS = os.path.join(O.REFERENCE_DIR, "resources", "models")


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from realtimeraytracing_gb300 import build
    build.build()


def test_generated_mesh_all_corner_syntaxes():
    v, f = S.icosphere(3)
    text = OO.to_obj_text(v, f)
    gv, gi = crt.parse_obj(text)
    ov, oi = OO.parse_obj(text)
    np.testing.assert_array_equal(gv.view(np.uint32), ov.view(np.uint32))
    np.testing.assert_array_equal(gi, oi)
    np.testing.assert_array_equal(gv, np.asarray(v, np.float32))
    np.testing.assert_array_equal(gi, np.asarray(f, np.uint32))


def test_polygons_become_fans_and_other_statements_are_skipped():
    text = """# a quad, a pentagon and a triangle
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
v 2 0.5 0
vn 0 0 1
g group
usemtl red
s off
f 1 2 3 4
f 1/1 2/1 5/1 3/1 4/1
f -1 -2 -3
"""
    gv, gi = crt.parse_obj(text)
    ov, oi = OO.parse_obj(text)
    np.testing.assert_array_equal(gi, oi)
    assert gi.tolist() == [[0, 1, 2], [0, 2, 3], [0, 1, 4], [0, 4, 2], [0, 2, 3], [4, 3, 2]]
    assert gv.shape == (5, 3)


def test_numbers_read_as_double_then_float():
    text = "v 0.1 -2.5e-3 +7\nv 1e30 3.4028235677973366e38 -0.0\nv 16777217 0.333333333333333314829616256247 1\nf 1 2 3\n"
    gv, _ = crt.parse_obj(text)
    ov, _ = OO.parse_obj(text)
    np.testing.assert_array_equal(gv.view(np.uint32), ov.view(np.uint32))
    assert gv[0, 2] == 7.0 and np.signbit(gv[1, 2])


@pytest.mark.parametrize("bad", ["v 1 2\n", "v 0 0 0\nv 1 0 0\nf 1 2\n", "v 0 0 0\nf 1 2 3\n",
                                 "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 0 1 2\n", "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 x\n",
                                 "v 0 0 zero\n"])
def test_malformed_input_is_an_error(bad):
    with pytest.raises(crt.CrtError) as e:
        crt.parse_obj(bad)
    assert e.value.status == 7
    with pytest.raises(ValueError):
        OO.parse_obj(bad)


@pytest.mark.skipif(not os.path.isdir(MODELS), reason="reference checkout not present")
@pytest.mark.parametrize("name,n_verts,n_tris", [("teapot.obj", 3644, 6320), ("stanford-bunny.obj", 35947, 69451),
                                                 ("suzanne.obj", 507, 968)])
def test_reference_models(name, n_verts, n_tris):
    path = os.path.join(MODELS, name)
    gv, gi = crt.parse_obj(path)
    with open(path) as fh:
        ov, oi = OO.parse_obj(fh.read())
    assert gv.shape == (n_verts, 3) and gi.shape == (n_tris, 3)
    np.testing.assert_array_equal(gv.view(np.uint32), ov.view(np.uint32))
    np.testing.assert_array_equal(gi, oi)
