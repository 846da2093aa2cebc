"""OBJ mesh input/output for UnitWorld.

The reference loads meshes with assimp (lib/osr/scene.cc:78-156) using
GenNormals | Triangulate | JoinIdenticalVertices | SortByPType |
OptimizeGraph, and takes the robot's centre as the float mean of the
resulting vertices (scene.cc:40-50, 141-145).  assimp is not available
here, so ``load_obj`` reproduces the vertex list that pipeline yields for
plain OBJ files: one vertex per distinct (position, texcoord, normal)
reference in order of first use by the faces, polygons fan-triangulated.
Vertices never referenced by a face are dropped, as assimp drops them.
"""
from __future__ import annotations

import numpy as np


def load_obj(path: str):
    """Return (V float32 [n, 3], F uint32 [m, 3]) in assimp's joined-vertex order."""
    pos, uv, nrm = [], [], []
    keys = {}
    verts = []
    faces = []
    with open(path, "r", errors="replace") as fh:
        for line in fh:
            if not line or line[0] == "#":
                continue
            parts = line.split()
            if not parts:
                continue
            tag = parts[0]
            if tag == "v":
                pos.append((float(parts[1]), float(parts[2]), float(parts[3])))
            elif tag == "vt":
                uv.append(tuple(float(x) for x in parts[1:3]))
            elif tag == "vn":
                nrm.append((float(parts[1]), float(parts[2]), float(parts[3])))
            elif tag == "f":
                corner = []
                for tok in parts[1:]:
                    fields = tok.split("/")
                    vi = int(fields[0])
                    vi = vi - 1 if vi > 0 else len(pos) + vi
                    ti = ni = -1
                    if len(fields) > 1 and fields[1]:
                        ti = int(fields[1])
                        ti = ti - 1 if ti > 0 else len(uv) + ti
                    if len(fields) > 2 and fields[2]:
                        ni = int(fields[2])
                        ni = ni - 1 if ni > 0 else len(nrm) + ni
                    key = (pos[vi], uv[ti] if ti >= 0 else None, nrm[ni] if ni >= 0 else None)
                    idx = keys.get(key)
                    if idx is None:
                        idx = len(verts)
                        keys[key] = idx
                        verts.append(pos[vi])
                    corner.append(idx)
                for k in range(1, len(corner) - 1):
                    faces.append((corner[0], corner[k], corner[k + 1]))
    V = np.asarray(verts, dtype=np.float32).reshape(-1, 3)
    F = np.asarray(faces, dtype=np.uint32).reshape(-1, 3)
    return V, F


def save_obj(path: str, V, F) -> None:
    """Write a plain triangle OBJ (so other tools can read the synthetic meshes)."""
    V = np.asarray(V)
    F = np.asarray(F)
    with open(path, "w") as fh:
        for v in V:
            fh.write("v %.9g %.9g %.9g\n" % (v[0], v[1], v[2]))
        for f in F:
            fh.write("f %d %d %d\n" % (f[0] + 1, f[1] + 1, f[2] + 1))
