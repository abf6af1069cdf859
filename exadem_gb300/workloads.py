"""Seeded synthetic workloads of the benchmark configurations.

No public dataset is involved: every input is generated from a fixed seed by
random sequential addition (``dem_generate_rsa_spheres``, include/dem_workloads.h,
built as its own host library ``libdem_workloads.so``, apart from the product library).

* ``spheres_box``     -- config 1: monodisperse spheres in a walled box.
* ``spheres_floor``   -- config 2: polydisperse spheres, periodic in x/y,
                          floor wall, Hooke + linear cohesion, rolling kr.
* ``spheres_drum``    -- one rotating drum of config 5.
Where a configuration leaves a value open it is stated in the function.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _abi as A
from .system import System, contact_params, empty_particles, make_params


@dataclass
class Workload:
    name: str
    params: A.Params
    particles: dict
    surfaces: list = field(default_factory=list)   # kwargs of System.register_surface
    cylinders: list = field(default_factory=list)  # kwargs of System.register_cylinder
    meshes: list = field(default_factory=list)     # kwargs of System.register_mesh
    steps: int = 1000
    info: dict = field(default_factory=dict)
    shapes: list = None  # polyhedron shapes (System.set_shapes), None for spheres
    # fragmentation: {"params": inner bond parameters (System.set_inner_bond_params),
    # "cluster": cluster of each particle, "threshold": sticking threshold}
    bonds: dict = None

    @property
    def n(self) -> int:
        return len(self.particles["rx"])

    def build(self, system_factory=None) -> System:
        """Creates a System (native by default) loaded with this workload."""
        s = system_factory(self.params) if system_factory else System(self.params)
        if self.shapes:
            s.set_shapes(self.shapes)
        s.set_particles(self.particles)
        for kw in self.surfaces:
            s.register_surface(**kw)
        for kw in self.cylinders:
            s.register_cylinder(**kw)
        for kw in self.meshes:
            s.register_mesh(**kw)
        if self.bonds:
            s.set_inner_bond_params(self.bonds["params"])
            ids = self.particles.get("id")
            ids = np.arange(self.n, dtype=np.uint64) if ids is None else ids
            s.stick_polyhedra(ids, self.bonds["cluster"], self.bonds["threshold"])
        return s


def save_workload(w: Workload, path) -> None:
    """A workload in one .npz file: particle arrays, parameters, drivers, shapes, meshes."""
    import json

    meta = {"name": w.name, "steps": w.steps, "surfaces": w.surfaces, "cylinders": w.cylinders,
            "info": {k: v for k, v in w.info.items() if isinstance(v, (int, float, str, list, dict, bool))},
            "params": {f: (list(getattr(w.params, f)) if hasattr(getattr(w.params, f), "__len__") else
                           getattr(w.params, f)) for f, _ in A.Params._fields_ if f not in ("config", "config_driver")},
            "config": {f: getattr(w.params.config, f) for f, _ in A.ContactParams._fields_},
            "config_driver": {f: getattr(w.params.config_driver, f) for f, _ in A.ContactParams._fields_},
            "shapes": [], "meshes": []}
    arrays = {f"p/{k}": np.asarray(v) for k, v in w.particles.items()}
    for k, s in enumerate(w.shapes or []):
        meta["shapes"].append({"name": s["name"], "radius": s["radius"], "volume": s["volume"],
                               "i_over_m": list(np.atleast_1d(s["i_over_m"]).astype(float)), "faces": s["faces"]})
        arrays[f"s{k}/vertices"] = np.asarray(s["vertices"], dtype=np.float64)
        arrays[f"s{k}/edges"] = np.asarray(s["edges"], dtype=np.int32)
    for k, m in enumerate(w.meshes):
        meta["meshes"].append({"faces": [list(map(int, f)) for f in m["faces"]], "minkowski": m["minkowski"],
                               "center": list(m.get("center", (0, 0, 0))), "quat": list(m.get("quat", (1, 0, 0, 0)))})
        arrays[f"m{k}/vertices"] = np.asarray(m["vertices"], dtype=np.float64)
        arrays[f"m{k}/edges"] = np.asarray(m["edges"], dtype=np.int32)
    if w.bonds:
        meta["bonds"] = {"params": w.bonds["params"], "threshold": float(w.bonds["threshold"])}
        arrays["b/cluster"] = np.asarray(w.bonds["cluster"], dtype=np.float64)
    arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(path, **arrays)


def load_workload(path) -> Workload:
    """The workload save_workload wrote."""
    import json

    z = np.load(path)
    meta = json.loads(z["meta"].tobytes().decode())
    p = A.Params()
    for f, v in meta["params"].items():
        cur = getattr(p, f)
        if hasattr(cur, "__len__"):
            cur[:] = v
        else:
            setattr(p, f, v)
    p.config = contact_params(**meta["config"])
    p.config_driver = contact_params(**meta["config_driver"])
    parts = {k[2:]: np.ascontiguousarray(z[k]) for k in z.files if k.startswith("p/")}
    shapes = []
    for k, s in enumerate(meta["shapes"]):
        iom = s["i_over_m"]
        shapes.append(_shape(s["name"], z[f"s{k}/vertices"], z[f"s{k}/edges"], s["faces"], s["radius"], s["volume"],
                             tuple(iom) if len(iom) == 3 else iom[0]))
    meshes = [dict(vertices=z[f"m{k}/vertices"], edges=z[f"m{k}/edges"], faces=m["faces"], minkowski=m["minkowski"],
                   center=tuple(m["center"]), quat=tuple(m["quat"])) for k, m in enumerate(meta["meshes"])]
    w = Workload(meta["name"], p, parts, surfaces=[{k: (tuple(v) if isinstance(v, list) else v) for k, v in d.items()}
                                                   for d in meta["surfaces"]],
                 cylinders=[{k: (tuple(v) if isinstance(v, list) else v) for k, v in d.items()}
                            for d in meta["cylinders"]],
                 meshes=meshes, steps=meta["steps"], info=meta["info"])
    w.shapes = shapes or None
    if "bonds" in meta:
        w.bonds = {"params": meta["bonds"]["params"], "threshold": meta["bonds"]["threshold"],
                   "cluster": np.ascontiguousarray(z["b/cluster"])}
    return w


def rsa(n, rmin, rmax, density, lo, hi, periodic=(0, 0, 0), grow_axis=-1, seed=1, vmin=0.0, vmax=0.0,
        region=0, cyl_center=(0.0, 0.0), cyl_radius=0.0, max_attempts=64, id_offset=0, radii=None):
    lib = A.load_workloads()
    spec = A.RsaSpec()
    spec.n = n
    spec.rmin, spec.rmax, spec.density = rmin, rmax, density
    spec.lo[:] = list(lo)
    spec.hi[:] = list(hi)
    spec.periodic[:] = list(periodic)
    spec.grow_axis = grow_axis
    spec.region = region
    spec.cyl_center[:] = list(cyl_center)
    spec.cyl_radius = cyl_radius
    spec.vmin, spec.vmax = vmin, vmax
    spec.seed = seed
    spec.max_attempts = max_attempts
    spec.id_offset = id_offset
    if radii is not None:
        spec.radii = A.ptr(radii)
    arr = empty_particles(n)
    st = A.particles_struct(arr, n)
    top = C.c_double(0.0)
    rc = lib.dem_generate_rsa_spheres(C.byref(spec), C.byref(st), C.byref(top))
    if rc != A.DEM_OK:
        raise A.DemError(rc, "dem_generate_rsa_spheres", "could not place the spheres")
    return arr, top.value


def spheres_box(n=10_000, box=30.0, radius=0.5, density=2500.0, seed=1, steps=1000, dt=1e-3, skin=0.05,
                **flags) -> Workload:
    """Config 1: n monodisperse spheres r=0.5, density 2500, non-overlapping uniform
    random placement in a box x box x box walled box, velocities uniform in
    [-0.1, 0.1], gravity -9.81 z; Hooke kn=1e4, kt=8e3, kr=0, mu=0.3,
    damp_rate=0.9 for particles and walls; dt=1e-3, skin 0.05."""
    arr, _ = rsa(n, radius, radius, density, (0, 0, 0), (box, box, box), seed=seed, vmin=-0.1, vmax=0.1,
                 max_attempts=100000)
    cfg = dict(kn=1e4, kt=8e3, kr=0.0, mu=0.3, damp_rate=0.9)
    p = make_params((0, 0, 0), (box, box, box), (0, 0, 0), rcut_inc=skin, dt=dt, gravity=(0, 0, -9.81),
                    config=cfg, config_driver=cfg, **flags)
    walls = []
    for ax in range(3):
        nrm = [0.0, 0.0, 0.0]
        nrm[ax] = 1.0
        walls.append(dict(offset=0.0, normal=tuple(nrm)))
        walls.append(dict(offset=box, normal=tuple(nrm)))
    return Workload("spheres_box", p, arr, surfaces=walls, steps=steps, info={"box": box})


def spheres_floor(n=2_000_000, side=400.0, rmin=0.4, rmax=0.6, phi=0.55, density=2.0, seed=2, steps=1000,
                  dt=5e-4, skin=0.05, rsa_attempts=400, **flags) -> Workload:
    """Config 2: n polydisperse spheres, radii uniform in [0.4, 0.6], in a
    side x side x H domain periodic in x/y with a floor wall at z = 0.
    Random sequential addition jams near phi = 0.38, below the 0.55 target, so
    the spheres are added inside a window at the fill front that moves up
    each time rsa_attempts draws find no room (400 draws: phi = 0.295 at 2M,
    1500 draws: 0.319 but four times the generation time); the column height
    and the achieved fraction are reported in ``info``.  Hooke kn=1e4, kt=8e3, mu=0.3,
    damp 0.9, linear cohesion kc=1e3 over dncut=0.01 (fc = kc*dncut = 10),
    rolling kr=100, dt=5e-4.  Open values: density 2 (cohesion and weight of
    the same order, overlaps ~2% of r), zero initial velocity, skin 0.05."""
    ev = 4.0 / 3.0 * math.pi * (rmax ** 4 - rmin ** 4) / (4 * (rmax - rmin))
    h0 = n * ev / (phi * side * side)
    arr, top = rsa(n, rmin, rmax, density, (0, 0, 0), (side, side, 4 * rmax), periodic=(1, 1, 0), grow_axis=2,
                   seed=seed, max_attempts=rsa_attempts)
    cfg = dict(kn=1e4, kt=8e3, kr=100.0, mu=0.3, damp_rate=0.9, fc=10.0, dncut=0.01)
    p = make_params((0, 0, 0), (side, side, top + 2 * rmax), (1, 1, 0), rcut_inc=skin, dt=dt,
                    gravity=(0, 0, -9.81), law=A.LAW_HOOKE_COHESIVE, config=cfg, config_driver=cfg, **flags)
    vol = float(np.sum(4.0 / 3.0 * math.pi * arr["radius"] ** 3))
    info = {"height": top, "phi_achieved": vol / (side * side * top), "phi_target": phi}
    return Workload("spheres_floor", p, arr, surfaces=[dict(offset=0.0, normal=(0.0, 0.0, 1.0))], steps=steps,
                    info=info)


def spheres_drum(n=20_000, rmin=0.45, rmax=0.55, fill=0.30, density=2.0, length=None, omega=2.0, seed=5,
                 steps=2000, dt=5e-4, skin=0.05, id_offset=0, **flags) -> Workload:
    """One drum of config 5: n spheres, radii uniform in [0.45, 0.55], in a
    cylinder (axis y) whose radius is set so the solid volume is `fill` of the
    drum volume; the drum turns at `omega` rad/s (Cylinder vrot); Hooke
    kn=1e4, kt=8e3, mu=0.4, damp 0.9, dt=5e-4.  Open values: density 2,
    drum length = 2 x radius (when not given), zero initial velocity."""
    ev = 4.0 / 3.0 * math.pi * (rmax ** 4 - rmin ** 4) / (4 * (rmax - rmin))
    vs = n * ev
    # pi R^2 * (2R) * fill = vs  (length 2R) or pi R^2 L fill = vs
    if length is None:
        R = (vs / (fill * 2 * math.pi)) ** (1.0 / 3.0)
        length = 2 * R
    else:
        R = math.sqrt(vs / (fill * math.pi * length))
    c = R + 1.0
    lo, hi = (0.0, 0.0, 0.0), (2 * c, length, 2 * c)
    arr, _ = rsa(n, rmin, rmax, density, lo, hi, periodic=(0, 1, 0), seed=seed, region=1, cyl_center=(c, c),
                 cyl_radius=R, max_attempts=100000, id_offset=id_offset)
    cfg = dict(kn=1e4, kt=8e3, kr=0.0, mu=0.4, damp_rate=0.9)
    p = make_params(lo, hi, (0, 1, 0), rcut_inc=skin, dt=dt, gravity=(0, 0, -9.81), config=cfg, config_driver=cfg,
                    **flags)
    cyl = dict(radius=R, axis=(1.0, 0.0, 1.0), center=(c, 0.0, c), vrot=(0.0, omega, 0.0))
    return Workload("spheres_drum", p, arr, cylinders=[cyl], steps=steps, info={"drum_radius": R, "length": length})


def terrain_triangles(side, m, amp, waves, z0):
    """(2 m^2, 3, 3) triangles of the height field z0 + amp sin(2 pi w x / side)
    sin(2 pi w y / side) over [-side/2, side/2]^2 (a square grid, two triangles
    per square)."""
    xs = np.linspace(-side / 2, side / 2, m + 1)
    h = lambda x, y: z0 + amp * math.sin(2 * math.pi * waves * x / side) * math.sin(2 * math.pi * waves * y / side)
    tri = []
    for i in range(m):
        for j in range(m):
            p = [(xs[a], xs[b], h(xs[a], xs[b])) for a, b in ((i, j), (i + 1, j), (i + 1, j + 1), (i, j + 1))]
            tri.append([p[0], p[1], p[2]])
            tri.append([p[0], p[2], p[3]])
    return np.asarray(tri, dtype=np.float64)


def spheres_mesh_terrain(n=3000, side=16.0, height=None, rmin=0.4, rmax=0.5, density=2.0, m=16, amp=0.8,
                         waves=2, minkowski=0.05, vz=-3.0, seed=9, steps=400, dt=1e-3, skin=0.1,
                         **flags) -> Workload:
    """Spheres falling on a triangulated height field (a mesh driver,
    register_stl_mesh with its STL conversion: every sphere against the mesh's
    vertices, edges and faces) inside four walls.  The mesh is built about the
    origin and placed by its center (side/2, side/2, amp + 0.2) and a quarter
    turn about z.  Hooke kn=1e4, kt=8e3, kr=0, mu=0.4, damp 0.9 for pairs and walls; the
    spheres start above the terrain moving down at vz."""
    from exadem_gb300.stl import build_shape

    ev = 4.0 / 3.0 * math.pi * (rmax ** 4 - rmin ** 4) / (4 * (rmax - rmin))
    zc = amp + 0.2
    z_lo = zc + amp + minkowski + rmax + 0.2
    if height is None:
        height = z_lo + n * ev / (0.25 * (side - 2 * rmax) ** 2) + 2 * rmax
    arr, _ = rsa(n, rmin, rmax, density, (rmax, rmax, z_lo), (side - rmax, side - rmax, height - rmax), seed=seed,
                 max_attempts=100000)
    arr["vz"] = arr["vz"] + vz
    cfg = dict(kn=1e4, kt=8e3, kr=0.0, mu=0.4, damp_rate=0.9)
    p = make_params((0, 0, 0), (side, side, height), (0, 0, 0), rcut_inc=skin, dt=dt, gravity=(0, 0, -9.81),
                    config=cfg, config_driver=cfg, **flags)
    shp = build_shape(list(terrain_triangles(side, m, amp, waves, 0.0)))
    c45 = math.cos(math.pi / 4)
    mesh = dict(vertices=shp["vertices"], edges=shp["edges"], faces=shp["faces"], minkowski=minkowski,
                center=(side / 2, side / 2, zc), quat=(c45, 0.0, 0.0, c45))
    walls = [dict(offset=0.0, normal=(1.0, 0.0, 0.0)), dict(offset=-side, normal=(-1.0, 0.0, 0.0)),
             dict(offset=0.0, normal=(0.0, 1.0, 0.0)), dict(offset=-side, normal=(0.0, -1.0, 0.0))]
    return Workload("spheres_mesh_terrain", p, arr, surfaces=walls, meshes=[mesh], steps=steps,
                    info={"mesh_vertices": len(shp["vertices"]), "mesh_edges": len(shp["edges"]),
                          "mesh_faces": len(shp["faces"])})


@dataclass
class BatchWorkload:
    """Independent systems run in one context (dem_set_systems): the particle
    arrays are concatenated system after system, each system keeps its own
    domain and drivers; `members` are the systems as standalone workloads."""
    name: str
    params: A.Params
    members: list
    steps: int = 1000
    info: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return sum(m.n for m in self.members)

    def particles(self) -> dict:
        keys = self.members[0].particles.keys()
        return {k: np.concatenate([m.particles[k] for m in self.members]) for k in keys}

    def systems(self) -> list:
        out, first, dfirst = [], 0, 0
        for m in self.members:
            nd = len(m.surfaces) + len(m.cylinders)
            p = m.params
            out.append(dict(first=first, count=m.n, bounds_lo=list(p.bounds_lo), bounds_hi=list(p.bounds_hi),
                            periodic=list(p.periodic), driver_first=dfirst, driver_count=nd))
            first += m.n
            dfirst += nd
        return out

    def build(self, system_factory=None) -> System:
        s = system_factory(self.params) if system_factory else System(self.params)
        s.set_particles(self.particles())
        for m in self.members:
            for kw in m.surfaces:
                s.register_surface(**kw)
            for kw in m.cylinders:
                s.register_cylinder(**kw)
        s.set_systems(self.systems())
        return s


def drums_batch(nsys=256, nmin=2_000, nmax=200_000, seed=5, steps=2000, **kw) -> BatchWorkload:
    """Config 5: nsys rotating drums (spheres_drum) with sphere counts
    log-uniform in [nmin, nmax] (seeded), each drum its own system with its
    own domain (periodic along its axis) and its own rotating cylinder.
    Drum k uses seed seed * 1000 + k and ids offset by the spheres before it."""
    import concurrent.futures as cf
    import os

    rng = np.random.default_rng(seed)
    counts = np.exp(rng.uniform(math.log(nmin), math.log(nmax), nsys)).astype(np.int64)
    offsets = np.concatenate([[0], np.cumsum(counts)[:-1]])
    # the drums are independent: generate them in parallel (the C generator releases the GIL)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(nsys, os.cpu_count() or 1))) as ex:
        members = list(ex.map(lambda k: spheres_drum(n=int(counts[k]), seed=seed * 1000 + k, steps=steps,
                                                     id_offset=int(offsets[k]), **kw), range(nsys)))
    return BatchWorkload("drums_batch", members[0].params, members, steps=steps,
                         info={"systems": nsys, "counts": counts.tolist()})


# ------------------------------------------------------------------ polyhedra
def _sym_eigen(C):
    """Jacobi eigen decomposition of a symmetric 3x3 matrix, restating
    mat9::sym_eigen (src/shape/include/exaDEM/type/mat9.hpp:278-376).
    C is a flat list of 9 floats (row major); returns (V flat 9, D 3)."""
    A = list(C)
    V = [1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0]
    B = [A[0], A[4], A[8]]
    D = [A[0], A[4], A[8]]
    Z = [0.0, 0.0, 0.0]
    for sweep in range(1, 51):
        sm = abs(A[1]) + abs(A[2]) + abs(A[5])
        if abs(sm) < 1.0e-15:
            return V, D
        thresh = sm * 0.2 / 9.0 if sweep < 4 else 0.0
        for p in range(2):
            for q in range(p + 1, 3):
                g = 100.0 * abs(A[p * 3 + q])
                if sweep > 4 and g < 1.0e-15:
                    A[p * 3 + q] = 0.0
                elif abs(A[p * 3 + q]) > thresh:
                    h = D[q] - D[p]
                    if g < 1.0e-20:
                        t = A[p * 3 + q] / h
                    else:
                        theta = 0.5 * h / A[p * 3 + q]
                        t = 1.0 / (abs(theta) + math.sqrt(1.0 + theta * theta))
                        if theta < 0.0:
                            t = -t
                    c = 1.0 / math.sqrt(1.0 + t * t)
                    s = t * c
                    tau = s / (1.0 + c)
                    h = t * A[p * 3 + q]
                    Z[p] -= h
                    Z[q] += h
                    D[p] -= h
                    D[q] += h
                    A[p * 3 + q] = 0.0
                    for j in range(0, p):
                        g, h = A[j * 3 + p], A[j * 3 + q]
                        A[j * 3 + p] = g - s * (h + g * tau)
                        A[j * 3 + q] = h + s * (g - h * tau)
                    for j in range(p + 1, q):
                        g, h = A[p * 3 + j], A[j * 3 + q]
                        A[p * 3 + j] = g - s * (h - g * tau)
                        A[j * 3 + q] = h + s * (g - h * tau)
                    for j in range(q + 1, 3):
                        g, h = A[p * 3 + j], A[q * 3 + j]
                        A[p * 3 + j] = g - s * (h + g * tau)
                        A[q * 3 + j] = h + s * (g - h * tau)
                    for j in range(3):
                        g, h = V[j * 3 + p], V[j * 3 + q]
                        V[j * 3 + p] = g - s * (h + g * tau)
                        V[j * 3 + q] = h + s * (g - h * tau)
        B = [B[k] + Z[k] for k in range(3)]
        D = list(B)
        Z = [0.0, 0.0, 0.0]
    return V, D


def build_obb(vertices, radius):
    """Shape OBB from the covariance of the vertices, restating build_OBB
    (src/shape/include/exaDEM/shape_prepro.hpp:26-97); extents include the radius."""
    vs = [tuple(map(float, v)) for v in vertices]
    n = len(vs)
    mu = [0.0, 0.0, 0.0]
    for v in vs:
        mu = [mu[0] + v[0], mu[1] + v[1], mu[2] + v[2]]
    inv_n = 1.0 / float(n)  # vec3::operator/= multiplies by the reciprocal (type/vec3.hpp:179-185)
    mu = [mu[0] * inv_n, mu[1] * inv_n, mu[2] * inv_n]
    cxx = cxy = cxz = cyy = cyz = czz = 0.0
    for p in vs:
        cxx += p[0] * p[0] - mu[0] * mu[0]
        cxy += p[0] * p[1] - mu[0] * mu[1]
        cxz += p[0] * p[2] - mu[0] * mu[2]
        cyy += p[1] * p[1] - mu[1] * mu[1]
        cyz += p[1] * p[2] - mu[1] * mu[2]
        czz += p[2] * p[2] - mu[2] * mu[2]
    V, _ = _sym_eigen([cxx, cxy, cxz, cxy, cyy, cyz, cxz, cyz, czz])

    def normalized(a):  # vec3::normalize (type/vec3.hpp:257-265)
        n2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2]
        if n2 > 0.0:
            inv = 1.0 / math.sqrt(n2)
            return [a[0] * inv, a[1] * inv, a[2] * inv]
        return list(a)

    r = normalized([V[0], V[3], V[6]])
    u = normalized([V[1], V[4], V[7]])
    f = normalized([V[2], V[5], V[8]])
    dot = lambda a, b: a[0] * b[0] + a[1] * b[1] + a[2] * b[2]
    mn, mx = [1e20] * 3, [-1e20] * 3
    for p in vs:
        pp = [dot(r, p), dot(u, p), dot(f, p)]
        mn = [min(mn[k], pp[k]) for k in range(3)]
        mx = [max(mx[k], pp[k]) for k in range(3)]
    half = [0.5 * (mx[k] + mn[k]) for k in range(3)]
    center = [V[0] * half[0] + V[1] * half[1] + V[2] * half[2], V[3] * half[0] + V[4] * half[1] + V[5] * half[2],
              V[6] * half[0] + V[7] * half[1] + V[8] * half[2]]
    extent = [0.5 * (mx[k] - mn[k]) + radius for k in range(3)]
    return {"center": center, "e1": r, "e2": u, "e3": f, "extent": extent}


def _shape(name, vertices, edges, faces, radius, volume, i_over_m):
    v = np.asarray(vertices, dtype=np.float64)
    return {"name": name, "vertices": v, "edges": np.asarray(edges, dtype=np.int32), "faces": faces,
            "radius": radius, "obb": build_obb(v, radius), "volume": volume, "i_over_m": i_over_m,
            "max_rcut": max_rcut(v, radius)}


def max_rcut(vertices, radius) -> float:
    """shape::compute_max_rcut (shape.hpp:479-489): max over vertices of |v| + radius."""
    rc = 0.0
    for x, y, z in np.asarray(vertices, dtype=np.float64).tolist():
        rc = max(rc, math.sqrt(x * x + y * y + z * z) + radius)
    return rc


def shape_cube(a=1.0, radius=0.01):
    h = 0.5 * a
    v = [[-h, -h, -h], [h, -h, -h], [h, h, -h], [-h, h, -h], [-h, -h, h], [h, -h, h], [h, h, h], [-h, h, h]]
    e = [[0, 1], [1, 2], [2, 3], [3, 0], [4, 5], [5, 6], [6, 7], [7, 4], [0, 4], [1, 5], [2, 6], [3, 7]]
    f = [[0, 3, 2, 1], [4, 5, 6, 7], [0, 1, 5, 4], [1, 2, 6, 5], [2, 3, 7, 6], [3, 0, 4, 7]]
    return _shape("Cube", v, e, f, radius, a ** 3, a * a / 6.0)


def shape_tetrahedron(a=1.2, radius=0.01):
    s = a / (2.0 * math.sqrt(2.0))
    v = [[s, s, s], [s, -s, -s], [-s, s, -s], [-s, -s, s]]
    e = [[0, 1], [0, 2], [0, 3], [1, 2], [1, 3], [2, 3]]
    f = [[0, 1, 2], [0, 3, 1], [0, 2, 3], [1, 3, 2]]
    return _shape("Tetrahedron", v, e, f, radius, a ** 3 / (6.0 * math.sqrt(2.0)), a * a / 20.0)


def shape_octahedron(a=1.0, radius=0.01):
    d = a / math.sqrt(2.0)
    v = [[d, 0, 0], [-d, 0, 0], [0, d, 0], [0, -d, 0], [0, 0, d], [0, 0, -d]]
    e = [[0, 2], [2, 1], [1, 3], [3, 0], [0, 4], [2, 4], [1, 4], [3, 4], [0, 5], [2, 5], [1, 5], [3, 5]]
    f = [[0, 2, 4], [2, 1, 4], [1, 3, 4], [3, 0, 4], [0, 5, 2], [2, 5, 1], [1, 5, 3], [3, 5, 0]]
    return _shape("Octahedron", v, e, f, radius, math.sqrt(2.0) / 3.0 * a ** 3, a * a / 10.0)


def exadem_cube(name="cube", length=1.0, minkowski=0.01):
    """The cube of exaDEM's add_cube operator, restating basic_shape::create_cube
    (src/shape/include/exaDEM/shape/basic_shape/cube.hpp:14-88): unit-cube
    vertices scaled by the length, its edge and face order, the volume and the
    inertia over mass of the Minkowski-rounded cube."""
    c, r, pi = float(length), float(minkowski), math.pi
    volume = c * c * c + 6.0 * c * c * r + 3.0 * pi * r * r * c + (4.0 / 3.0) * pi * r * r * r
    inertia = (1.0 / 6.0) * math.pow(c, 5)
    d = 0.5 * (c + r)
    i_face = (1.0 / 12.0) * c * c * r * (c * c + r * r)
    v_face = c * c * r
    inertia += 6.0 * (i_face + v_face * d * d)
    v_edges = 3.0 * pi * r * r * c
    inertia += v_edges * ((c * c) / 12.0 + (r * r) / 2.0)
    inertia += (8.0 / 15.0) * pi * math.pow(r, 5)
    iom = inertia / (1.0 * 1.0 * 1.0 * volume) * 1.0  # I / get_volume() * (1, 1, 1)
    unit = [[-0.5, -0.5, -0.5], [0.5, -0.5, -0.5], [0.5, 0.5, -0.5], [-0.5, 0.5, -0.5],
            [-0.5, -0.5, 0.5], [0.5, -0.5, 0.5], [0.5, 0.5, 0.5], [-0.5, 0.5, 0.5]]
    v = [[x * c for x in p] for p in unit]
    e = [[0, 1], [1, 2], [2, 3], [3, 0], [4, 5], [5, 6], [6, 7], [7, 4], [0, 4], [1, 5], [2, 6], [3, 7]]
    f = [[3, 2, 1, 0], [4, 5, 6, 7], [0, 1, 5, 4], [2, 3, 7, 6], [4, 7, 3, 0], [1, 2, 6, 5]]
    return _shape(name, v, e, f, r, volume, (iom, iom, iom))


def polyhedra_floor(n=200_000, side=None, density=0.02, seed=3, steps=2000, dt=1e-4, skin=0.05,
                    radius=0.01, walls=True, rsa_attempts=1500, **flags) -> Workload:
    """Config 3: n convex polyhedra, an equal mix of cubes (edge 1.0), regular
    tetrahedra (edge 1.2) and octahedra (edge 1.0) with Minkowski radius 0.01;
    orientations uniform on SU(2) (normalised 4-D Gaussian); positions by random
    sequential addition of the circumscribed spheres, a floor wall and four side
    walls; Hooke kn=1e5, kt=8e4, mu=0.5, damp 0.9, dt=1e-4, gravity deposition.
    The RSA runs in a window moving up the column (as for spheres) with
    rsa_attempts draws per particle before the window moves; 1500 draws give a
    solid fraction of the circumscribed spheres of 0.351 at 200k (0.35 asked),
    reported as info["phi_spheres"].
    Open values: density 0.02 (the reference's polyhedron examples), zero initial
    velocity, skin 0.05, footprint side = (n / 14)^(1/2) * 1.0 (about 120 for 200k)."""
    shapes = [shape_cube(1.0, radius), shape_tetrahedron(1.2, radius), shape_octahedron(1.0, radius)]
    if side is None:
        side = max(8.0, math.sqrt(n / 14.0))
    types = (np.arange(n) % 3).astype(np.uint32)
    radii = np.array([shapes[t]["max_rcut"] for t in types], dtype=np.float64)
    rmax = float(radii.max())
    arr, top = rsa(n, float(radii.min()), rmax, density, (0, 0, 0), (side, side, 4 * rmax), grow_axis=2, seed=seed,
                   max_attempts=rsa_attempts, radii=np.ascontiguousarray(radii))
    rng = np.random.default_rng(seed)
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1)[:, None]
    arr["qw"], arr["qx"], arr["qy"], arr["qz"] = (np.ascontiguousarray(q[:, k]) for k in range(4))
    arr["type"] = types
    arr["radius"] = radii
    vol = np.array([shapes[t]["volume"] for t in types])
    iom = np.array([shapes[t]["i_over_m"] for t in types])
    arr["mass"] = density * vol
    for ax in ("inertiax", "inertiay", "inertiaz"):
        arr[ax] = arr["mass"] * iom
    arr["homothety"] = np.ones(n)
    for k in ("vx", "vy", "vz"):
        arr[k] = np.zeros(n)
    cfg = dict(kn=1e5, kt=8e4, kr=0.0, mu=0.5, damp_rate=0.9)
    hi = (side, side, top + 2 * rmax)
    p = make_params((0, 0, 0), hi, (0, 0, 0), rcut_inc=skin, dt=dt, gravity=(0, 0, -9.81), config=cfg,
                    config_driver=cfg, **flags)
    surfaces = [dict(offset=0.0, normal=(0.0, 0.0, 1.0))]
    if walls:
        surfaces += [dict(offset=0.0, normal=(1.0, 0.0, 0.0)), dict(offset=side, normal=(1.0, 0.0, 0.0)),
                     dict(offset=0.0, normal=(0.0, 1.0, 0.0)), dict(offset=side, normal=(0.0, 1.0, 0.0))]
    sphere_vol = float(np.sum(4.0 / 3.0 * math.pi * radii ** 3))
    w = Workload("polyhedra_floor", p, arr, surfaces=surfaces, steps=steps,
                 info={"height": top, "phi_spheres": sphere_vol / (side * side * top), "side": side})
    w.shapes = shapes
    return w


def polyhedra_lattice(nx=8, ny=8, nz=6, spacing=1.3, density=1.0, seed=7, radius=0.01, vmax=0.5, dt=1e-4,
                      skin=0.05, kn=1e4, **flags) -> Workload:
    """Dense test arrangement: polyhedra (cube / tetrahedron / octahedron mix) on
    a cubic lattice whose spacing is below the circumscribed diameters, with
    random orientations and velocities, inside a walled box.  Many vertex,
    edge and face features are within the skin from the first step."""
    shapes = [shape_cube(1.0, radius), shape_tetrahedron(1.2, radius), shape_octahedron(1.0, radius)]
    rng = np.random.default_rng(seed)
    n = nx * ny * nz
    g = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"), -1).reshape(-1, 3)
    pos = (g + 1.0) * spacing + rng.uniform(-0.05, 0.05, (n, 3))
    types = rng.integers(0, 3, n).astype(np.uint32)
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1)[:, None]
    arr = empty_particles(n)
    arr["rx"], arr["ry"], arr["rz"] = (np.ascontiguousarray(pos[:, k]) for k in range(3))
    arr["qw"], arr["qx"], arr["qy"], arr["qz"] = (np.ascontiguousarray(q[:, k]) for k in range(4))
    arr["vx"], arr["vy"], arr["vz"] = (rng.uniform(-vmax, vmax, n) for _ in range(3))
    arr["vrotx"], arr["vroty"], arr["vrotz"] = (rng.uniform(-1.0, 1.0, n) for _ in range(3))
    arr["type"] = types
    arr["id"] = np.arange(n, dtype=np.uint64)
    arr["radius"] = np.array([shapes[t]["max_rcut"] for t in types])
    vol = np.array([shapes[t]["volume"] for t in types])
    iom = np.array([shapes[t]["i_over_m"] for t in types])
    arr["mass"] = density * vol
    for ax in ("inertiax", "inertiay", "inertiaz"):
        arr[ax] = arr["mass"] * iom
    arr["homothety"] = np.ones(n)
    hi = ((nx + 1) * spacing, (ny + 1) * spacing, (nz + 1) * spacing)
    cfg = dict(kn=kn, kt=0.8 * kn, kr=0.0, mu=0.5, damp_rate=0.9)
    p = make_params((0, 0, 0), hi, (0, 0, 0), rcut_inc=skin, dt=dt, gravity=(0, 0, -9.81), config=cfg,
                    config_driver=cfg, **flags)
    surfaces = [dict(offset=0.0, normal=(0.0, 0.0, 1.0)), dict(offset=0.0, normal=(1.0, 0.0, 0.0)),
                dict(offset=hi[0], normal=(1.0, 0.0, 0.0)), dict(offset=0.0, normal=(0.0, 1.0, 0.0)),
                dict(offset=hi[1], normal=(0.0, 1.0, 0.0))]
    w = Workload("polyhedra_lattice", p, arr, surfaces=surfaces, steps=100)
    w.shapes = shapes
    return w


def fragment_blocks(nblocks=2, nx=3, ny=3, nz=3, edge=1.0, radius=0.01, density=1.0, seed=5, vz=-3.0, tilt=0.3,
                    gap=0.05, dt=1e-4, skin=0.05, kn=1e5, bond=None, threshold=1e-4, steps=400,
                    **flags) -> Workload:
    """Fragmentation: nblocks blocks of nx x ny x nz cubes (edge `edge`, Minkowski
    radius `radius`), the cubes of a block face to face (centres 2 radius +
    edge apart, so bonded vertices touch: dn 0), each block one cluster and
    turned as a whole by a random rotation of angle up to `tilt`, its lowest
    corner gap to 2 gap above a floor, falling at vz under gravity.  The pairs of touching faces of a block are
    bonded by stick_polyhedra (sticking threshold `threshold`) with the inner
    bond parameters `bond` (default kn 1e4, kt 8e3, damp_rate 0.87 as in
    exaDEM's two-fragments example, mixed mode g 0.05: at vz -3 part of the
    interfaces break at the impact); contacts: Hooke kn, kt = 0.8 kn, mu 0.3,
    damp_rate 0.87.  The bond damping is not scaled by the bond weight
    (inner_bond_force.hpp:45), so kn must stay small enough for the explicit
    step: damp_rate 2 sqrt(kn m/2) dt x bonds per particle well below 2 m."""
    shp = shape_cube(edge, radius)
    rng = np.random.default_rng(seed)
    pitch = edge + 2 * radius
    pos, cl, q = [], [], []
    ext = np.array([nx, ny, nz], dtype=np.float64) * pitch
    span = float(np.linalg.norm(ext))
    per_row = max(1, int(math.ceil(math.sqrt(nblocks))))
    for b in range(nblocks):
        ax = rng.standard_normal(3)
        ax /= np.linalg.norm(ax)
        ang = rng.uniform(-tilt, tilt)
        qb = np.array([math.cos(ang / 2), *(math.sin(ang / 2) * ax)])
        w, x, y, z = qb
        R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                      [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                      [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
        g = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"), -1).reshape(-1, 3)
        local = (g - (np.array([nx, ny, nz]) - 1) / 2.0) * pitch
        corners = np.array([[sx, sy, sz] for sx in (-1, 1) for sy in (-1, 1) for sz in (-1, 1)]) * (0.5 * ext)
        low = float(min((R @ c)[2] for c in corners))  # lowest point of the turned block above its centre
        centre = np.array([(b % per_row + 0.5) * (span + 1.0), (b // per_row + 0.5) * (span + 1.0),
                           -low + gap + rng.uniform(0, gap)])
        for p in local:
            pos.append(centre + R @ p)
            cl.append(float(b))
            q.append(qb)
    pos, q = np.asarray(pos), np.asarray(q)
    n = len(pos)
    arr = empty_particles(n)
    arr["rx"], arr["ry"], arr["rz"] = (np.ascontiguousarray(pos[:, k]) for k in range(3))
    arr["qw"], arr["qx"], arr["qy"], arr["qz"] = (np.ascontiguousarray(q[:, k]) for k in range(4))
    arr["vz"] = np.full(n, float(vz))
    arr["vx"], arr["vy"] = np.zeros(n), np.zeros(n)
    arr["type"] = np.zeros(n, dtype=np.uint32)
    arr["id"] = np.arange(n, dtype=np.uint64)
    arr["radius"] = np.full(n, shp["max_rcut"])
    arr["mass"] = np.full(n, density * shp["volume"])
    for ax_ in ("inertiax", "inertiay", "inertiaz"):
        arr[ax_] = arr["mass"] * shp["i_over_m"]
    arr["homothety"] = np.ones(n)
    side = per_row * (span + 1.0)
    hi = (side, side, float(pos[:, 2].max()) + span)
    cfg = dict(kn=kn, kt=0.8 * kn, kr=0.0, mu=0.3, damp_rate=0.87)
    p = make_params((0, 0, 0), hi, (0, 0, 0), rcut_inc=skin, dt=dt, gravity=(0, 0, -9.81), config=cfg,
                    config_driver=cfg, **flags)
    w = Workload("fragment_blocks", p, arr, surfaces=[dict(offset=0.0, normal=(0.0, 0.0, 1.0))], steps=steps)
    w.shapes = [shp]
    w.bonds = {"params": bond or dict(kn=1e4, kt=8e3, damp_rate=0.87, g=0.05), "cluster": np.asarray(cl),
               "threshold": threshold}
    return w


def polyhedra_mesh_terrain(nx=6, ny=6, nz=2, spacing=1.6, density=1.0, seed=11, radius=0.01, amp=0.3, waves=2,
                           m=14, minkowski=0.02, vz=-3.0, dt=5e-4, skin=0.05, kn=1e4, steps=300,
                           **flags) -> Workload:
    """Polyhedra (cube / tetrahedron / octahedron mix, random orientations) on a
    lattice above a triangulated height field (a mesh driver: interaction types
    7-12 against its vertices, edges and faces) inside four walls, falling at
    vz.  The mesh is built about the origin and placed by its center and a
    quarter turn about z.  Hooke kn, kt = 0.8 kn, mu 0.5, damp 0.9."""
    from exadem_gb300.stl import build_shape

    shapes = [shape_cube(1.0, radius), shape_tetrahedron(1.2, radius), shape_octahedron(1.0, radius)]
    rng = np.random.default_rng(seed)
    n = nx * ny * nz
    side = (nx + 1) * spacing
    zc = amp + 0.2
    z0 = zc + amp + minkowski + 1.0
    g = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"), -1).reshape(-1, 3)
    pos = np.stack([(g[:, 0] + 1.0) * spacing, (g[:, 1] + 1.0) * spacing, z0 + g[:, 2] * spacing], 1)
    pos = pos + rng.uniform(-0.05, 0.05, (n, 3))
    types = rng.integers(0, 3, n).astype(np.uint32)
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1)[:, None]
    arr = empty_particles(n)
    arr["rx"], arr["ry"], arr["rz"] = (np.ascontiguousarray(pos[:, k]) for k in range(3))
    arr["qw"], arr["qx"], arr["qy"], arr["qz"] = (np.ascontiguousarray(q[:, k]) for k in range(4))
    arr["vx"], arr["vy"] = (rng.uniform(-0.2, 0.2, n) for _ in range(2))
    arr["vz"] = np.full(n, vz) + rng.uniform(-0.2, 0.2, n)
    arr["vrotx"], arr["vroty"], arr["vrotz"] = (rng.uniform(-1.0, 1.0, n) for _ in range(3))
    arr["type"] = types
    arr["id"] = np.arange(n, dtype=np.uint64)
    arr["radius"] = np.array([shapes[t]["max_rcut"] for t in types])
    vol = np.array([shapes[t]["volume"] for t in types])
    iom = np.array([shapes[t]["i_over_m"] for t in types])
    arr["mass"] = density * vol
    for ax in ("inertiax", "inertiay", "inertiaz"):
        arr[ax] = arr["mass"] * iom
    arr["homothety"] = np.ones(n)
    hi = (side, side, z0 + nz * spacing + 1.0)
    cfg = dict(kn=kn, kt=0.8 * kn, kr=0.0, mu=0.5, damp_rate=0.9)
    p = make_params((0, 0, 0), hi, (0, 0, 0), rcut_inc=skin, dt=dt, gravity=(0, 0, -9.81), config=cfg,
                    config_driver=cfg, **flags)
    walls = [dict(offset=0.0, normal=(1.0, 0.0, 0.0)), dict(offset=side, normal=(1.0, 0.0, 0.0)),
             dict(offset=0.0, normal=(0.0, 1.0, 0.0)), dict(offset=side, normal=(0.0, 1.0, 0.0))]
    shp = build_shape(list(terrain_triangles(side, m, amp, waves, 0.0)))
    c45 = math.cos(math.pi / 4)
    mesh = dict(vertices=shp["vertices"], edges=shp["edges"], faces=shp["faces"], minkowski=minkowski,
                center=(side / 2, side / 2, zc), quat=(c45, 0.0, 0.0, c45))
    w = Workload("polyhedra_mesh_terrain", p, arr, surfaces=walls, meshes=[mesh], steps=steps)
    w.shapes = shapes
    return w


def mixer_triangles(radius=100.0, z0=30.0, z1=170.0, nseg=96, nring=10, blades=4, blade_len=80.0,
                    blade_w=4.0, blade_h=2.5, angle=0.0):
    """(nt, 3, 3) triangles of a synthetic mixer: a cylinder wall (nseg x nring
    quads), a bottom disk (nseg triangles) and `blades` box blades on the
    bottom, the shapes of the reference's mixer deck (its STL files are not
    part of this build)."""
    tri = []
    th = np.linspace(0.0, 2 * math.pi, nseg + 1)
    zs = np.linspace(z0, z1, nring + 1)
    ring = lambda t, z: (radius * math.cos(t), radius * math.sin(t), z)
    for a in range(nseg):
        for b in range(nring):
            p = [ring(th[a], zs[b]), ring(th[a + 1], zs[b]), ring(th[a + 1], zs[b + 1]), ring(th[a], zs[b + 1])]
            tri += [[p[0], p[1], p[2]], [p[0], p[2], p[3]]]
        tri.append([(0.0, 0.0, z0), ring(th[a + 1], z0), ring(th[a], z0)])
    for k in range(blades):
        t = angle + 2 * math.pi * k / blades
        c, s_ = math.cos(t), math.sin(t)
        loc = [(x, y, z) for z in (z0 + 0.5, z0 + 0.5 + blade_h) for (x, y) in
               ((2.0, -blade_w / 2), (blade_len, -blade_w / 2), (blade_len, blade_w / 2), (2.0, blade_w / 2))]
        v = [(x * c - y * s_, x * s_ + y * c, z) for x, y, z in loc]
        for f in ((0, 2, 1), (0, 3, 2), (4, 5, 6), (4, 6, 7), (0, 1, 5), (0, 5, 4), (1, 2, 6), (1, 6, 5),
                  (2, 3, 7), (2, 7, 6), (3, 0, 4), (3, 4, 7)):
            tri.append([v[f[0]], v[f[1]], v[f[2]]])
    return np.asarray(tri, dtype=np.float64)


def spheres_mixer(spacing=4.1, radius=2.0, density=0.0028, cyl_radius=92.0, z_lo=36.0, z_hi=166.3, minkowski=0.1,
                  dt=1e-3, skin=1.2, seed=13, steps=1000, n=None, **flags) -> Workload:
    """The mixer deck's shapes with spheres (example/spheres/mixer, 57k spheres):
    a simple-cubic lattice of spacing 4.1 inside a cylinder of radius 92 between
    z = 36 and 166.3 (about 51k spheres of radius 2, density 0.0028, velocity
    (0, 0, -1) with a 0.001 spread), falling into a synthetic mixer mesh
    (wall, bottom and four blades, Minkowski radius 0.1, mixer_triangles).
    Hooke kn 1000, kt 1000, mu 0.5, damp 0.999 (pairs), kt 800 for the mesh;
    dt 1e-3 (the deck's README), rcut_inc 1.2, 10 m cells.  n limits the count."""
    from exadem_gb300.stl import build_shape

    rng = np.random.default_rng(seed)
    ax = np.arange(-cyl_radius, cyl_radius + 1e-9, spacing)
    az = np.arange(z_lo, z_hi + 1e-9, spacing)
    gx, gy, gz = np.meshgrid(ax, ax, az, indexing="ij")
    keep = gx ** 2 + gy ** 2 < cyl_radius ** 2
    pos = np.stack([gx[keep], gy[keep], gz[keep]], 1)
    pos = pos[np.lexsort((pos[:, 0], pos[:, 1], pos[:, 2]))]
    if n is not None:
        pos = pos[:n]
    m = len(pos)
    arr = empty_particles(m)
    arr["rx"], arr["ry"], arr["rz"] = (np.ascontiguousarray(pos[:, k]) for k in range(3))
    arr["vx"], arr["vy"] = (rng.normal(0.0, 0.001, m) for _ in range(2))
    arr["vz"] = -1.0 + rng.normal(0.0, 0.001, m)
    arr["radius"] = np.full(m, radius)
    arr["mass"] = np.full(m, density * 4.0 / 3.0 * math.pi * radius ** 3)
    for a in ("inertiax", "inertiay", "inertiaz"):
        arr[a] = 0.4 * arr["mass"] * radius * radius
    arr["qw"] = np.ones(m)
    arr["homothety"] = np.ones(m)
    arr["id"] = np.arange(m, dtype=np.uint64)
    cfg = dict(kn=1000.0, kt=1000.0, kr=0.0, mu=0.5, damp_rate=0.999)
    cfgd = dict(kn=1000.0, kt=800.0, kr=0.0, mu=0.5, damp_rate=0.999)
    p = make_params((-105.0, -105.0, 28.0), (105.0, 105.0, 172.0), (0, 0, 0), rcut_inc=skin, dt=dt,
                    gravity=(0, 0, -9.81), config=cfg, config_driver=cfgd, cell_size=10.0, **flags)
    shp = build_shape(list(mixer_triangles()))
    mesh = dict(vertices=shp["vertices"], edges=shp["edges"], faces=shp["faces"], minkowski=minkowski)
    return Workload("spheres_mixer", p, arr, meshes=[mesh], steps=steps,
                    info={"mesh_vertices": len(shp["vertices"]), "mesh_edges": len(shp["edges"]),
                          "mesh_faces": len(shp["faces"])})

