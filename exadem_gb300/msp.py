"""Reader of exaDEM ``.msp`` input decks (the subset the hot path needs).

An ``.msp`` deck is YAML read by onika's operator graph: top-level keys name
operators or operator blocks, ``includes`` pulls other decks in first, a key
defined later replaces an earlier one, and a key written ``+name`` appends its
list to the earlier ``name``.  Quantities may carry units (``9 m``, ``1e-4 s``).

``load_deck(path, config_dirs)`` resolves a deck into one dict (includes
searched in the deck's folder, then in ``config_dirs``, e.g. exaDEM's
``data/config``).  ``deck_workload(deck, base_dir)`` turns the resolved deck
into a ``Workload`` for this library, reading the keys the default Verlet deck
uses on the hot path:

- ``domain``: bounds, periodic, cell_size;
- ``global``: dt, rcut_inc, simulation_end_iteration;
- ``setup_drivers``: register_surface / register_cylinder (state: offset,
  normal, center, radius, axis, vel, vrot) and register_stl_mesh (filename,
  minkowski, binary, scale, state center and quat); stationary motion only;
- ``compute_force``: gravity_force (default gravity (0, 0, -9.807)), the
  contact operator (contact_sphere / contact_polyhedron and their
  ``*_hooke``, ``*_hooke_cohesive``, ``*_hooke_dmt`` variants) with its
  ``config`` and ``config_driver`` blocks and ``symetric``;
- ``input_data``: particle_type, read_shape_file, lattice (optionally inside a
  box region of ``particle_regions``), set_fields.

``set_fields`` follows src/field/set_fields.cu:238-330: a sphere of radius r and
density d gets m = (4/3) pi r^3 d (pi = 4 atan 1) and inertia 0.4 m r^2; a
polyhedron gets m = d V(h), inertia m I/m(h) and radius compute_max_rcut.
Defaults are those of the operator (density 1, velocity 0, identity
quaternion, group 0).  Restated from exaNBody (not part of exaDEM's sources):
``lattice`` places one particle of the type list per structure site at
(cell index + site offset) x size, the cell index running over the domain
bounds, sites SC (0.5, 0.5, 0.5), BCC (+ corner), FCC (4 sites).
``sigma_velocity`` and ``random_quaternion`` draw from this library's own
seeded generator (exaDEM draws from std::default_random_engine, an
implementation-defined stream), so those initial values follow the same
distributions, not the same numbers.
"""
from __future__ import annotations

import math
import re
from pathlib import Path

import numpy as np

# ------------------------------------------------------------------ YAML subset
_UNIT = re.compile(r"^([-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?)\s*([A-Za-z/^0-9.*]+)?$")


def _scalar(tok: str):
    t = tok.strip()
    if t == "":
        return None
    if (t[0] == t[-1]) and t[0] in "\"'" and len(t) >= 2:
        return t[1:-1]
    low = t.lower()
    if low in ("true", "yes", "on"):
        return True
    if low in ("false", "no", "off"):
        return False
    if low in ("null", "~"):
        return None
    try:
        return int(t)
    except ValueError:
        pass
    try:
        return float(t)
    except ValueError:
        pass
    m = _UNIT.match(t)
    if m:  # a quantity with a unit: its value in SI (the units the decks use are SI)
        return float(m.group(1))
    return t


def _strip_comment(line: str) -> str:
    out, q = [], None
    for i, ch in enumerate(line):
        if q:
            if ch == q:
                q = None
        elif ch in "\"'":
            q = ch
        elif ch == "#" and (i == 0 or line[i - 1] in " \t"):
            break
        out.append(ch)
    return "".join(out).rstrip()


def _split_flow(s: str):
    """Split the inside of a flow collection on top-level commas."""
    parts, depth, cur, q = [], 0, [], None
    for ch in s:
        if q:
            cur.append(ch)
            if ch == q:
                q = None
            continue
        if ch in "\"'":
            q = ch
        elif ch in "[{":
            depth += 1
        elif ch in "]}":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
    if "".join(cur).strip():
        parts.append("".join(cur))
    return parts


def _flow(s: str):
    s = s.strip()
    if s.startswith("["):
        if not s.endswith("]"):
            raise ValueError(f"unterminated flow sequence: {s}")
        return [_flow(p) for p in _split_flow(s[1:-1])]
    if s.startswith("{"):
        if not s.endswith("}"):
            raise ValueError(f"unterminated flow mapping: {s}")
        out = {}
        for p in _split_flow(s[1:-1]):
            k, _, v = p.partition(":")
            out[k.strip()] = _flow(v)
        return out
    return _scalar(s)


def _key_split(text: str):
    """'key: value' -> (key, value) when the line is a mapping entry, else None."""
    q = None
    for i, ch in enumerate(text):
        if q:
            if ch == q:
                q = None
            continue
        if ch in "\"'":
            q = ch
        elif ch in "[{":
            return None
        elif ch == ":" and (i + 1 == len(text) or text[i + 1] in " \t"):
            return text[:i].strip(), text[i + 1:].strip()
    return None


def _depth(s: str) -> int:
    d, q = 0, None
    for ch in s:
        if q:
            if ch == q:
                q = None
        elif ch in "\"'":
            q = ch
        elif ch in "[{":
            d += 1
        elif ch in "]}":
            d -= 1
    return d


def parse_yaml(text: str):
    """The YAML subset of the decks: block mappings and sequences, flow
    collections, block literals (``|``), comments, scalars with units."""
    lines = []
    raw = text.splitlines()
    i = 0
    while i < len(raw):
        line = raw[i]
        body = _strip_comment(line)
        if body.strip():
            ind = len(body) - len(body.lstrip(" "))
            s = body.strip()
            while _depth(s) > 0 and i + 1 < len(raw):  # a flow collection continued on the next lines
                i += 1
                s = s + " " + _strip_comment(raw[i]).strip()
            kv = _key_split(s[2:] if s.startswith("- ") else s)
            if kv and kv[1] in ("|", ">", "|-", ">-"):  # block literal: keep its lines as text
                j = i + 1
                block = []
                while j < len(raw) and (not raw[j].strip() or len(raw[j]) - len(raw[j].lstrip(" ")) > ind):
                    block.append(raw[j])
                    j += 1
                lines.append((ind, s, "\n".join(block)))
                i = j
                continue
            lines.append((ind, s, None))
        i += 1
    pos = [0]

    def block(ind):
        if pos[0] >= len(lines):
            return None
        if lines[pos[0]][1].startswith("- ") or lines[pos[0]][1] == "-":
            return seq(lines[pos[0]][0])
        return mapping(lines[pos[0]][0])

    def value_after(rest, ind, literal):
        if literal is not None:
            return literal
        if rest == "":
            if pos[0] < len(lines) and (lines[pos[0]][0] > ind or
                                        (lines[pos[0]][0] == ind and lines[pos[0]][1].startswith("- "))):
                return block(lines[pos[0]][0])
            return None
        return _flow(rest)

    def mapping(ind):
        out = {}
        while pos[0] < len(lines):
            li, s, lit = lines[pos[0]]
            if li != ind or s.startswith("- "):
                break
            kv = _key_split(s)
            if kv is None:
                raise ValueError(f"expected 'key: value', got {s!r}")
            pos[0] += 1
            out[kv[0]] = value_after(kv[1], ind, lit)
        return out

    def seq(ind):
        out = []
        while pos[0] < len(lines):
            li, s, lit = lines[pos[0]]
            if li != ind or not (s.startswith("- ") or s == "-"):
                break
            item = s[2:].strip() if s != "-" else ""
            pos[0] += 1
            kv = _key_split(item) if item else None
            if kv is None:
                out.append(_flow(item) if item else (block(lines[pos[0]][0]) if pos[0] < len(lines)
                                                      and lines[pos[0]][0] > ind else None))
                continue
            # a mapping that starts on the dash line; its other keys are indented past the dash
            d = {kv[0]: value_after(kv[1], ind + 2, lit)}
            if pos[0] < len(lines) and lines[pos[0]][0] > ind and not lines[pos[0]][1].startswith("- "):
                d.update(mapping(lines[pos[0]][0]))
            out.append(d)
        return out

    doc = block(0) if lines else {}
    if pos[0] != len(lines):
        raise ValueError(f"cannot parse near {lines[pos[0]][1]!r}")
    return doc or {}


# ------------------------------------------------------------------- deck merge
def load_deck(path, config_dirs=(), defaults: bool = True) -> dict:
    """A deck with its includes resolved: includes first, in order, then the
    deck's own keys (a key replaces an earlier one, ``+key`` appends).  With
    ``defaults``, exaDEM's main-config.msp (found in ``config_dirs``) is read
    first, as the exaDEM executable does."""
    path = Path(path)
    dirs = [path.parent] + [Path(d) for d in config_dirs]
    seen = set()

    def find(name):
        for d in dirs:
            p = d / name
            if p.exists():
                return p
        return None

    def load(p: Path, out: dict):
        if p.resolve() in seen:
            return
        seen.add(p.resolve())
        doc = parse_yaml(p.read_text())
        for inc in doc.get("includes", []) or []:
            q = find(inc)
            if q is None:
                out.setdefault("_missing_includes", []).append(inc)
                continue
            load(q, out)
        for k, v in doc.items():
            if k == "includes":
                continue
            if k.startswith("+"):
                base = out.get(k[1:])
                base = list(base) if isinstance(base, list) else ([] if base in (None, "nop") else [base])
                out[k[1:]] = base + (v if isinstance(v, list) else [v])
            elif k in ("global", "domain") and isinstance(v, dict) and isinstance(out.get(k), dict):
                out[k] = {**out[k], **v}  # these blocks are slot assignments: merged key by key
            else:
                out[k] = v

    out: dict = {}
    if defaults:
        for d in config_dirs:
            if (Path(d) / "main-config.msp").exists():
                load(Path(d) / "main-config.msp", out)
                break
    load(path, out)
    return out


# ------------------------------------------------------------- deck -> workload
def _items(block):
    """A deck block (list of operators) as (name, params) pairs."""
    if block in (None, "nop"):
        return []
    if isinstance(block, (dict, str)):
        block = [block]
    out = []
    for it in block:
        if isinstance(it, str):
            out.append((it, {}))
        elif isinstance(it, dict):
            for k, v in it.items():
                out.append((k, v if isinstance(v, dict) else {}))
    return out


def _expand(deck, name, depth=0):
    """Operator entries of a block, with named sub-blocks of the deck expanded."""
    out = []
    for op, prm in _items(deck.get(name)):
        if depth < 8 and not prm and op in deck and isinstance(deck[op], (list, dict)) and op != name:
            out += _expand(deck, op, depth + 1)
        else:
            out.append((op, prm))
    return out


_SITES = {"SC": [(0.5, 0.5, 0.5)], "BCC": [(0.0, 0.0, 0.0), (0.5, 0.5, 0.5)],
          "FCC": [(0.0, 0.0, 0.0), (0.5, 0.5, 0.0), (0.5, 0.0, 0.5), (0.0, 0.5, 0.5)]}


def _vec(v, n=3):
    return [float(x) for x in (v if isinstance(v, (list, tuple)) else [v] * n)]


def deck_workload(deck: dict, base_dir=".", seed: int = 1, **flags):
    """The Workload (exadem_gb300.workloads) a resolved deck describes."""
    from . import _abi as A
    from .shp import read_shps
    from .system import make_params
    from .workloads import Workload

    base_dir = Path(base_dir)
    dom = deck.get("domain", {}) or {}
    glob = deck.get("global", {}) or {}
    lo, hi = (_vec(b) for b in dom["bounds"])
    periodic = [bool(x) for x in dom.get("periodic", [False] * 3)]
    dt = float(glob.get("dt", 1e-4))
    rcut_inc = float(glob.get("rcut_inc", 0.0))
    notes = []

    # force field
    gravity = (0.0, 0.0, -9.807)  # gravity_force default (gravity_force.cu)
    law, cfg, cfg_d, contact_op = A.LAW_HOOKE_NONE, None, None, None
    for op, prm in _expand(deck, "compute_force"):
        if op == "gravity_force":
            if "gravity" in prm:
                gravity = tuple(_vec(prm["gravity"]))
        elif op == "inner_bond_polyhedron" or op in ("rebind", "body", "condition"):
            pass  # bonds: run by every step of a system with bonds; the others: block structure
        elif not op.startswith("contact_"):
            notes.append(f"compute_force: operator {op} ignored")
        elif op.startswith("contact_"):
            contact_op = op
            cfg = prm.get("config", {}) or {}
            cfg_d = prm.get("config_driver", cfg) or cfg
            if op.endswith("_cohesive"):
                law = A.LAW_HOOKE_COHESIVE
            elif op.endswith("_dmt"):
                law = A.LAW_HOOKE_DMT
            if prm.get("symetric", True) is not True:
                raise ValueError(f"{op}: only symetric: true is supported")
    if contact_op is None:
        raise ValueError("the deck defines no contact operator in compute_force")
    keys = ("kn", "kt", "kr", "mu", "damp_rate", "fc", "dncut", "gamma")

    def params(c):
        return {k: float(c[k]) for k in keys if k in c}

    # particles
    types: list = []
    groups: dict = {}
    shapes: list = []
    polyhedra = contact_op.startswith("contact_polyhedron") or "polyhedron" in contact_op
    lattices, fields = [], []
    ibp = None
    for op, prm in _expand(deck, "input_data"):
        if op == "add_cube":  # AddShapeCubeOperator (src/shape/add_cube.cpp:31-58)
            from .workloads import exadem_cube

            name = str(prm.get("name", "cube"))
            shapes.append(exadem_cube(name, float(prm.get("length", 1.0)), float(prm.get("minkowski", 0.01))))
            if name not in types:
                types.append(name)
            for k in prm:
                if k not in ("name", "length", "minkowski"):
                    notes.append(f"add_cube: key {k} is not a slot of add_cube; ignored")
        elif op == "inner_bond_params":
            ibp = _inner_bond_params(prm)
        elif op == "particle_type":
            for t in prm.get("type", []):
                if t not in types:
                    types.append(t)
        elif op == "read_shape_file":
            for s in read_shps(base_dir / prm["filename"]):
                shapes.append(s)
                if s["name"] not in types:
                    types.append(s["name"])
        elif op == "lattice":
            lattices.append(prm)
        elif op == "set_fields":
            fields.append(prm)
        elif op not in ("init_rcb_grid", "domain", "message"):
            notes.append(f"input_data: operator {op} ignored")
    if not lattices:
        raise ValueError("the deck places no particles (no lattice in input_data)")
    regions = {}
    for ent in (deck.get("particle_regions") or []):
        if isinstance(ent, dict):
            for rname, rdef in ent.items():
                regions[rname] = rdef
    rng = np.random.default_rng(seed)
    pos, ptype = [], []
    for L in lattices:
        size = _vec(L.get("size", [1.0, 1.0, 1.0]))
        ltypes = L.get("types", types[:1])
        for t in ltypes:
            if t not in types:
                types.append(t)
        enl = float(L.get("enlarge_bounds", 0.0) or 0.0)
        sites = _SITES.get(str(L.get("structure", "SC")).upper())
        if sites is None:
            raise ValueError(f"lattice structure {L.get('structure')} not supported")
        llo = [lo[d] - enl for d in range(3)]
        cnt = [max(0, int(math.floor((hi[d] + enl - llo[d]) / size[d] + 1e-9))) for d in range(3)]
        box = None
        if L.get("region") is not None:  # a region given by its bounds (particle_regions: NAME: {bounds: ...})
            rdef = regions.get(L["region"])
            if not isinstance(rdef, dict) or "bounds" not in rdef:
                raise ValueError(f"lattice: region {L['region']} is not a box region (bounds)")
            box = [_vec(b) for b in rdef["bounds"]]
        k = 0
        for iz in range(cnt[2]):
            for iy in range(cnt[1]):
                for ix in range(cnt[0]):
                    for s in sites:
                        x = [llo[0] + (ix + s[0]) * size[0], llo[1] + (iy + s[1]) * size[1],
                             llo[2] + (iz + s[2]) * size[2]]
                        if box is not None and not all(box[0][d] <= x[d] <= box[1][d] for d in range(3)):
                            continue
                        pos.append(x)
                        ptype.append(types.index(ltypes[k % len(ltypes)]))
                        k += 1
    n = len(pos)
    from .system import empty_particles

    arr = empty_particles(n)
    P = np.asarray(pos, dtype=np.float64).reshape(n, 3)
    arr["rx"], arr["ry"], arr["rz"] = (np.ascontiguousarray(P[:, d]) for d in range(3))
    arr["id"] = np.arange(n, dtype=np.uint64)
    arr["qw"] = np.ones(n)
    arr["homothety"] = np.ones(n)
    ptype = np.asarray(ptype, dtype=np.uint32)
    shape_index = {s["name"]: k for k, s in enumerate(shapes)}
    arr["type"] = np.array([shape_index.get(types[t], 0) for t in ptype], dtype=np.uint32) if polyhedra else \
        np.zeros(n, dtype=np.uint32)
    if not fields:
        raise ValueError("the deck sets no particle fields (no set_fields)")
    for F in fields:
        ftypes = F.get("type", [])
        for i, tname in enumerate(ftypes):
            if tname not in types:
                raise ValueError(f"set_fields: type {tname} is not defined")
            sel = ptype == types.index(tname)
            m = int(sel.sum())
            if m == 0:
                continue

            def pick(key, default):
                v = F.get(key)
                return v[i] if isinstance(v, list) and i < len(v) else default

            d = float(pick("density", 1.0))
            h = float(pick("homothety", 1.0))
            vel = _vec(pick("velocity", [0.0, 0.0, 0.0]))
            sig = pick("sigma_velocity", None)
            arr["group"][sel] = int(pick("group", 0))
            arr["homothety"][sel] = h
            v = np.tile(np.asarray(vel), (m, 1))
            if sig is not None:
                v = v + rng.normal(0.0, float(sig), (m, 3))
            for c, k in enumerate(("vx", "vy", "vz")):
                arr[k][sel] = v[:, c]
            rq = pick("random_quaternion", False)
            if "random_quaterion" in F:
                notes.append("set_fields: key random_quaterion is not a slot of set_fields; ignored")
            q = pick("quaternion", None)
            if rq:
                qq = rng.standard_normal((m, 4))
                qq /= np.linalg.norm(qq, axis=1)[:, None]
            else:
                qq = np.tile(np.asarray(_vec(q, 4) if q is not None else [1.0, 0.0, 0.0, 0.0]), (m, 1))
            for c, k in enumerate(("qw", "qx", "qy", "qz")):
                arr[k][sel] = qq[:, c]
            if polyhedra:
                s = shapes[shape_index[tname]]
                vol = h * h * h * s["volume"]              # shape::get_volume(h)
                mass = d * vol
                iom = s["i_over_m"]
                iom = (iom, iom, iom) if np.isscalar(iom) else iom
                arr["mass"][sel] = mass
                for c, k in enumerate(("inertiax", "inertiay", "inertiaz")):
                    arr[k][sel] = mass * (h * h * iom[c])  # m * get_Im(h)
                arr["radius"][sel] = s["max_rcut"]          # compute_max_rcut
            else:
                r = pick("radius", None)
                if r is None:
                    raise ValueError("set_fields: spheres need a radius")
                r = float(r)
                pi = 4 * math.atan(1)
                V = ((4.0) / (3.0)) * pi * r * r * r
                mass = V * d
                arr["radius"][sel] = r
                arr["mass"][sel] = mass
                for k in ("inertiax", "inertiay", "inertiaz"):
                    arr[k][sel] = 0.4 * mass * r * r

    p = make_params(lo, hi, periodic, rcut_inc=rcut_inc, dt=dt, gravity=gravity, law=law,
                    config=params(cfg), config_driver=params(cfg_d), cell_size=float(dom.get("cell_size", 0.0) or 0.0),
                    **flags)
    # drivers
    surfaces, cylinders, meshes = [], [], []
    for op, prm in _expand(deck, "setup_drivers"):
        st = prm.get("state", {}) or {}
        motion = str((prm.get("params", {}) or {}).get("motion_type", "STATIONARY")).upper()
        if op in ("register_surface", "register_cylinder") and motion != "STATIONARY":
            raise ValueError(f"{op}: motion_type {motion} is not supported (stationary drivers only)")
        if op == "register_surface":
            surfaces.append(dict(offset=float(st["offset"]), normal=tuple(_vec(st["normal"])),
                                 center=tuple(_vec(st.get("center", [0, 0, 0]))),
                                 vel=tuple(_vec(st.get("vel", [0, 0, 0]))), vrot=tuple(_vec(st.get("vrot", [0, 0, 0])))))
        elif op == "register_cylinder":
            cylinders.append(dict(radius=float(st["radius"]), axis=tuple(_vec(st["axis"])),
                                  center=tuple(_vec(st["center"])), vel=tuple(_vec(st.get("vel", [0, 0, 0]))),
                                  vrot=tuple(_vec(st.get("vrot", [0, 0, 0])))))
        elif op == "register_stl_mesh":
            from .stl import load_stl_mesh

            if motion != "STATIONARY" or prm.get("deform") is not None:
                raise ValueError("register_stl_mesh: stationary, undeformed meshes only")
            sc = prm.get("scale")
            m = load_stl_mesh(str(base_dir / prm["filename"]), bool(prm.get("binary", False)),
                              float(sc) if sc is not None else None)
            meshes.append(dict(vertices=m["vertices"], edges=m["edges"], faces=m["faces"],
                               minkowski=float(prm["minkowski"]), center=tuple(_vec(st.get("center", [0, 0, 0]))),
                               quat=tuple(_vec(st.get("quat", [1, 0, 0, 0]), 4))))
        else:
            notes.append(f"setup_drivers: operator {op} ignored")
    steps = int(glob.get("simulation_end_iteration", 1000))
    w = Workload("deck", p, arr, surfaces=surfaces, cylinders=cylinders, meshes=meshes, steps=steps,
                 info={"contact_operator": contact_op, "types": types, "notes": notes})
    w.shapes = shapes if polyhedra else None
    # fragmentation (config_fragmentation.msp prepro_fragmentation): stick_polyhedra
    # when apply_particle_sticking is set; the cluster field is 0 for the particles
    # a lattice places (one cluster)
    if polyhedra and glob.get("apply_particle_sticking") is True:
        if ibp is None:
            raise ValueError("apply_particle_sticking needs inner_bond_params in input_data")
        w.bonds = {"params": ibp, "cluster": np.zeros(n), "threshold": float(glob.get("sticking_threshold", 2e-5))}
    return w


def _inner_bond_params(prm: dict):
    """inner_bond_params (src/forcefield/multimat_inner_bond.cpp:104-200): a
    default_config dict, or per group pair lists (group1, group2, kn, kt,
    damp_rate and g, gn + gt or g + sigma), as System.set_inner_bond_params takes."""
    def one(c):
        out = {k: float(c[k]) for k in ("kn", "kt", "damp_rate") if k in c}
        for k in ("g", "gn", "gt", "sigma"):
            if k in c:
                out[k] = float(c[k])
        if not {"kn", "kt", "damp_rate"} <= set(out) or not ("g" in out or {"gn", "gt"} <= set(out)):
            raise ValueError(f"inner_bond_params: incomplete parameters {c}")
        return out

    default = prm.get("default_config")
    if prm.get("group1") is None:
        if default is None:
            raise ValueError("inner_bond_params: define group1/group2 lists or a default_config")
        return one(default)
    g1, g2 = [int(x) for x in prm["group1"]], [int(x) for x in prm["group2"]]
    ng = max(g1 + g2) + 1
    table = [[one(default) if default is not None else None for _ in range(ng)] for _ in range(ng)]
    for p_, (a, b) in enumerate(zip(g1, g2)):
        c = {k: prm[k][p_] for k in ("kn", "kt", "damp_rate", "g", "gn", "gt", "sigma") if prm.get(k) is not None}
        table[a][b] = table[b][a] = one(c)
    if any(x is None for row in table for x in row):
        raise ValueError("inner_bond_params: a group pair has no parameters and there is no default_config")
    return table
