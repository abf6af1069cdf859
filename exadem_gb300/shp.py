"""Reader of the Rockable/exaDEM ``.shp`` shape format.

Follows ``read_shp`` / ``read_shps`` (src/shape/include/exaDEM/shape_reader.hpp:36-150):
a file holds shapes between a line ``<`` and a token ``>``; inside, keys are
read token by token:

- ``name`` <word>; ``radius`` <Minkowski radius>; ``volume`` <v>; ``I/m`` <3 values>;
- ``preCompDone`` must be ``y`` (volume and I/m given), otherwise the shape is refused;
- ``nv`` n, then one vertex per line (3 values); ``ne`` n, then one edge per line
  (2 vertex indices); ``nf`` n, then one face per line (its vertex count, then
  the indices);
- any other token is skipped (``position``, ``orientation``, ``obb.*``: the
  reference recomputes the OBB from the vertices with build_OBB and ignores the
  file's).

Each vertex, edge and face record starts after the end of the current line, as
the reference's ``getline`` before each one.  The returned dicts have the keys of
``workloads._shape`` (name, vertices, edges, faces, radius, obb, volume,
i_over_m, max_rcut); ``i_over_m`` is the file's 3-vector.
"""
from __future__ import annotations

import numpy as np

from .workloads import build_obb, max_rcut


class _Stream:
    """Whitespace tokens and rest-of-line skips over a text, like std::istream >> and getline."""

    def __init__(self, text: str):
        self.s = text
        self.i = 0

    def token(self) -> str | None:
        s, i, n = self.s, self.i, len(self.s)
        while i < n and s[i].isspace():
            i += 1
        if i >= n:
            self.i = n
            return None
        j = i
        while j < n and not s[j].isspace():
            j += 1
        self.i = j
        return s[i:j]

    def skip_line(self) -> None:
        k = self.s.find("\n", self.i)
        self.i = len(self.s) if k < 0 else k + 1

    def line(self) -> str | None:
        if self.i >= len(self.s):
            return None
        k = self.s.find("\n", self.i)
        if k < 0:
            out, self.i = self.s[self.i:], len(self.s)
        else:
            out, self.i = self.s[self.i:k], k + 1
        return out

    def need(self, conv, what: str):
        t = self.token()
        if t is None:
            raise ValueError(f".shp: unexpected end of file reading {what}")
        try:
            return conv(t)
        except ValueError:
            raise ValueError(f".shp: bad value {t!r} for {what}") from None


def _read_one(st: _Stream) -> dict:
    name, radius, volume = "undefined", 0.0, 0.0
    iom = [0.0, 0.0, 0.0]
    verts: list = []
    edges: list = []
    faces: list = []
    while True:
        key = st.token()
        if key is None:
            raise ValueError(".shp: unexpected end of file or malformed shape (no closing '>')")
        if key == "name":
            name = st.need(str, "name")
        if key == "preCompDone":
            if st.need(str, "preCompDone") != "y":
                raise ValueError(".shp: preCompDone must be 'y' (volume and I/m precomputed)")
        elif key == "radius":
            radius = st.need(float, "radius")
        elif key == "volume":
            volume = st.need(float, "volume")
        elif key == "I/m":
            iom = [st.need(float, "I/m") for _ in range(3)]
        elif key == "position":
            for _ in range(3):
                st.need(float, "position")
        elif key == "nv":
            for _ in range(st.need(int, "nv")):
                st.skip_line()
                verts.append([st.need(float, "vertex") for _ in range(3)])
        elif key == "ne":
            for _ in range(st.need(int, "ne")):
                st.skip_line()
                edges.append([st.need(int, "edge"), st.need(int, "edge")])
        elif key == "nf":
            for _ in range(st.need(int, "nf")):
                st.skip_line()
                k = st.need(int, "face size")
                if k <= 0:
                    raise ValueError(".shp: a face needs at least one vertex")
                faces.append([st.need(int, "face vertex") for _ in range(k)])
        elif key == ">":
            break
    if not verts:
        raise ValueError(f".shp: shape {name!r} has no vertices")
    v = np.asarray(verts, dtype=np.float64)
    nv = len(v)
    for e in edges:
        if not (0 <= e[0] < nv and 0 <= e[1] < nv):
            raise ValueError(f".shp: shape {name!r}: edge {e} refers to a missing vertex")
    for f in faces:
        if any(not (0 <= x < nv) for x in f):
            raise ValueError(f".shp: shape {name!r}: face {f} refers to a missing vertex")
    return {"name": name, "vertices": v, "edges": np.asarray(edges, dtype=np.int32).reshape(-1, 2),
            "faces": faces, "radius": radius, "obb": build_obb(v, radius), "volume": volume,
            "i_over_m": tuple(iom), "max_rcut": max_rcut(v, radius)}


def parse_shps(text: str) -> list[dict]:
    """Every shape of a .shp text, in file order (read_shps, shape_reader.hpp:121-140)."""
    st = _Stream(text)
    out = []
    while True:
        line = st.line()
        if line is None:
            return out
        if line == "<":
            out.append(_read_one(st))


def read_shps(path) -> list[dict]:
    with open(path, "r") as f:
        return parse_shps(f.read())


def read_shp(path) -> dict:
    """The first shape of a .shp file (read_shp(file_name), shape_reader.hpp:148-158)."""
    shapes = read_shps(path)
    if not shapes:
        raise ValueError(f".shp: no shape in {path}")
    return shapes[0]


def format_shp(shape: dict) -> str:
    """A shape dict written in the .shp format (keys as read by read_shp)."""
    lines = ["<", f"name {shape['name']}", f"radius {float(shape['radius'])!r}", "preCompDone y"]
    v = np.asarray(shape["vertices"], dtype=np.float64)
    lines.append(f"nv {len(v)}")
    lines += [" ".join(repr(float(x)) for x in row) for row in v]
    e = np.asarray(shape["edges"]).reshape(-1, 2)
    lines.append(f"ne {len(e)}")
    lines += [f"{int(a)} {int(b)}" for a, b in e]
    lines.append(f"nf {len(shape['faces'])}")
    lines += [" ".join(str(int(x)) for x in [len(f), *f]) for f in shape["faces"]]
    lines.append(f"volume {float(shape['volume'])!r}")
    iom = shape["i_over_m"]
    iom = (iom, iom, iom) if np.isscalar(iom) else iom
    lines.append("I/m " + " ".join(repr(float(x)) for x in iom))
    lines.append(">")
    return "\n".join(lines) + "\n"
