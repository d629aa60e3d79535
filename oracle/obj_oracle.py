"""ORACLE — test infrastructure, never part of the product path.

Restatement of the mesh input the reference performs on the CPU:
  * Mesh::load (srcCommon/scene/geometry/mesh.cpp:186-263): tinyobjloader
    reads the file; every face becomes Triangle(v0, v1, v2, meshId) in file
    order.  tinyobjloader (a third-party dependency the reference does not
    vendor or pin) reads numbers as double and stores them as float, takes
    1-based or negative (relative) vertex indices from "v", "v/vt", "v//vn"
    and "v/vt/vn" corners, and triangulates larger faces itself; this
    restatement takes the fan (0, i, i+1) for those (the reference's teapot
    and bunny have triangles only).
  * Triangle's constructor (triangle.cpp:18-25): vertices as vec4(p, 1),
    the model id, zero padding — TriangleGPU, 64 bytes.
Only tests/ import this module.
"""
from __future__ import annotations

import numpy as np


def parse_obj(text: str):
    verts, tris = [], []
    for line_no, line in enumerate(text.split("\n"), 1):
        tok = line.split()
        if not tok:
            continue
        if tok[0] == "v":
            if len(tok) < 4:
                raise ValueError(f"OBJ line {line_no}: bad vertex")
            with np.errstate(over="ignore"):  # out-of-range literals become +-inf, as a float cast does
                verts.append([np.float32(float(t)) for t in tok[1:4]])
        elif tok[0] == "f":
            corners = []
            for c in tok[1:]:
                v = int(c.split("/")[0])
                if v == 0:
                    raise ValueError(f"OBJ line {line_no}: bad face corner")
                idx = v - 1 if v > 0 else len(verts) + v
                if not 0 <= idx < len(verts):
                    raise ValueError(f"OBJ line {line_no}: face corner past the vertices read so far")
                corners.append(idx)
            if len(corners) < 3:
                raise ValueError(f"OBJ line {line_no}: face with fewer than 3 corners")
            for i in range(1, len(corners) - 1):
                tris.append([corners[0], corners[i], corners[i + 1]])
    return np.array(verts, np.float32).reshape(-1, 3), np.array(tris, np.uint32).reshape(-1, 3)


def triangles_from_indexed(verts, indices, model_id=0):
    """TriangleGPU records (n, 16) float32 of an indexed mesh."""
    n = indices.shape[0]
    out = np.zeros((n, 16), np.float32)
    for k in range(3):
        out[:, 4 * k:4 * k + 3] = verts[indices[:, k]]
        out[:, 4 * k + 3] = 1.0
    out.view(np.uint32)[:, 12] = model_id
    return out


def to_obj_text(verts, indices, style: int = 0) -> str:
    """OBJ text of an indexed mesh; style varies the corner syntax per face
    (v, v/vt, v//vn, v/vt/vn, negative indices) to exercise the reader."""
    lines = ["# generated mesh", "o mesh", "mtllib none.mtl"]
    for v in np.asarray(verts, np.float32):
        lines.append("v " + " ".join(repr(float(c)) for c in v))
    lines.append("vn 0 0 1")
    lines.append("vt 0.5 0.5")
    nv = len(verts)
    for i, f in enumerate(np.asarray(indices)):
        s = (style + i) % 5
        if s == 0:
            c = [str(int(x) + 1) for x in f]
        elif s == 1:
            c = [f"{int(x) + 1}/1" for x in f]
        elif s == 2:
            c = [f"{int(x) + 1}//1" for x in f]
        elif s == 3:
            c = [f"{int(x) + 1}/1/1" for x in f]
        else:
            c = [str(int(x) - nv) for x in f]
        lines.append("f " + " ".join(c))
    return "\r\n".join(lines) + "\n"
