"""STL meshes for mesh drivers (register_stl_mesh): the reader of
stl_mesh_reader.hpp:25-132, the shape conversion of stl_mesh_to_driver.hpp:26-121
and shape::rescale (shape.hpp:605-618, vertices only).

The conversion is restated as it runs on one thread (its OpenMP loops then
follow the file order):

* vertices: every face vertex, sorted and made unique (onika's Vec3d ordering,
  restated here as lexicographic x, y, z; onika is not part of the reference
  sources);
* faces: in file order, each the indices of its vertices;
* edges: per face, (v_k, v_{k+1}) around the face in face order, with only
  consecutive duplicates removed (std::unique on the unsorted list), so an
  edge shared by two faces appears once per face.
"""
from __future__ import annotations

import struct

import numpy as np


def read_stl(path: str, binary: bool) -> list:
    """Faces of an STL file, each an (k, 3) float64 array (binary STL stores float32)."""
    faces = []
    if binary:
        with open(path, "rb") as f:
            f.read(80)
            (nt,) = struct.unpack("<I", f.read(4))
            rec = np.frombuffer(f.read(50 * nt), dtype=np.dtype([("n", "<f4", 3), ("v", "<f4", (3, 3)),
                                                                 ("a", "<u2")]), count=nt)
        for t in range(nt):
            faces.append(rec["v"][t].astype(np.float64))
        return faces
    with open(path) as f:
        tok = f.read().split()
    k = 0
    while k < len(tok):
        if tok[k] == "outer":
            verts = []
            k += 1
            while k < len(tok) and tok[k] != "endloop":
                if tok[k] == "vertex":
                    verts.append([float(tok[k + 1]), float(tok[k + 2]), float(tok[k + 3])])
                    k += 4
                else:
                    k += 1
            faces.append(np.asarray(verts, dtype=np.float64))
        k += 1
    return faces


def build_shape(faces: list) -> dict:
    """build_shape (stl_mesh_to_driver.hpp:26-121): vertices (nv, 3), edges (ne, 2),
    faces (list of vertex index lists)."""
    allv = np.concatenate(faces, axis=0) if faces else np.zeros((0, 3))
    uniq = sorted({(float(x), float(y), float(z)) for x, y, z in allv})
    index = {v: k for k, v in enumerate(uniq)}
    fl, edges = [], []
    for face in faces:
        idx = [index[(float(x), float(y), float(z))] for x, y, z in face]
        fl.append(idx)
        for k in range(len(idx)):
            edges.append((idx[k], idx[(k + 1) % len(idx)]))
    kept = [e for k, e in enumerate(edges) if k == 0 or e != edges[k - 1]]
    return {"vertices": np.asarray(uniq, dtype=np.float64).reshape(-1, 3),
            "edges": np.asarray(kept, dtype=np.int32).reshape(-1, 2), "faces": fl}


def rescale(shape: dict, scale: float) -> dict:
    """shape::rescale(scale, false): every vertex s * v; the Minkowski radius is kept."""
    out = dict(shape)
    out["vertices"] = scale * np.asarray(shape["vertices"], dtype=np.float64)
    return out


def load_stl_mesh(path: str, binary: bool, scale: float | None = None) -> dict:
    """register_stl_mesh's shape: read, convert, then rescale when scale != 1."""
    shp = build_shape(read_stl(path, binary))
    if scale is not None and scale > 0.0 and scale != 1.0:
        shp = rescale(shp, scale)
    return shp


def write_stl_binary(path: str, triangles: np.ndarray) -> None:
    """A binary STL of (nt, 3, 3) triangles (float32 vertices, zero normals)."""
    tri = np.asarray(triangles, dtype=np.float32).reshape(-1, 3, 3)
    with open(path, "wb") as f:
        f.write(b"\0" * 80)
        f.write(struct.pack("<I", len(tri)))
        for t in tri:
            f.write(struct.pack("<3f", 0.0, 0.0, 0.0))
            f.write(t.astype("<f4").tobytes())
            f.write(struct.pack("<H", 0))
