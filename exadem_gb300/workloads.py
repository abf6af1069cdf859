"""Seeded synthetic workloads of the benchmark configurations.

No public dataset is involved: every input is generated from a fixed seed by
random sequential addition (``dem_generate_rsa_spheres``, include/dem_workloads.h).

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
    steps: int = 1000
    info: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return len(self.particles["rx"])

    def build(self, system_factory=None) -> System:
        """Creates a System (native by default) loaded with this workload."""
        s = system_factory(self.params) if system_factory else System(self.params)
        s.set_particles(self.particles)
        for kw in self.surfaces:
            s.register_surface(**kw)
        for kw in self.cylinders:
            s.register_cylinder(**kw)
        return s


def rsa(n, rmin, rmax, density, lo, hi, periodic=(0, 0, 0), grow_axis=-1, seed=1, vmin=0.0, vmax=0.0,
        region=0, cyl_center=(0.0, 0.0), cyl_radius=0.0, max_attempts=64, id_offset=0):
    lib = A.load()
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
                  dt=5e-4, skin=0.05, **flags) -> Workload:
    """Config 2: n polydisperse spheres, radii uniform in [0.4, 0.6], in a
    side x side x H domain periodic in x/y with a floor wall at z = 0.
    Random sequential addition jams near phi = 0.38, below the 0.55 target, so
    the spheres are added inside a window at the fill front that moves up
    each time 400 draws find no room; the column height and the achieved
    fraction are reported in ``info``.  Hooke kn=1e4, kt=8e3, mu=0.3,
    damp 0.9, linear cohesion kc=1e3 over dncut=0.01 (fc = kc*dncut = 10),
    rolling kr=100, dt=5e-4.  Open values: density 2 (cohesion and weight of
    the same order, overlaps ~2% of r), zero initial velocity, skin 0.05."""
    ev = 4.0 / 3.0 * math.pi * (rmax ** 4 - rmin ** 4) / (4 * (rmax - rmin))
    h0 = n * ev / (phi * side * side)
    arr, top = rsa(n, rmin, rmax, density, (0, 0, 0), (side, side, 4 * rmax), periodic=(1, 1, 0), grow_axis=2,
                   seed=seed, max_attempts=400)
    cfg = dict(kn=1e4, kt=8e3, kr=100.0, mu=0.3, damp_rate=0.9, fc=10.0, dncut=0.01)
    p = make_params((0, 0, 0), (side, side, top + 2 * rmax), (1, 1, 0), rcut_inc=skin, dt=dt,
                    gravity=(0, 0, -9.81), law=A.LAW_HOOKE_COHESIVE, config=cfg, config_driver=cfg, **flags)
    vol = float(np.sum(4.0 / 3.0 * math.pi * arr["radius"] ** 3))
    info = {"height": top, "phi_achieved": vol / (side * side * top), "phi_target": phi}
    return Workload("spheres_floor", p, arr, surfaces=[dict(offset=0.0, normal=(0.0, 0.0, 1.0))], steps=steps,
                    info=info)


def spheres_drum(n=20_000, rmin=0.45, rmax=0.55, fill=0.30, density=2.0, length=None, omega=2.0, seed=5,
                 steps=2000, dt=5e-4, skin=0.05, **flags) -> Workload:
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
                 cyl_radius=R, max_attempts=100000)
    cfg = dict(kn=1e4, kt=8e3, kr=0.0, mu=0.4, damp_rate=0.9)
    p = make_params(lo, hi, (0, 1, 0), rcut_inc=skin, dt=dt, gravity=(0, 0, -9.81), config=cfg, config_driver=cfg,
                    **flags)
    cyl = dict(radius=R, axis=(1.0, 0.0, 1.0), center=(c, 0.0, c), vrot=(0.0, omega, 0.0))
    return Workload("spheres_drum", p, arr, cylinders=[cyl], steps=steps, info={"drum_radius": R, "length": length})
