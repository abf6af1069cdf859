"""Host-side mirror of exaDEM's operator interface for the per-timestep hot path.

``System`` owns one native context (``dem_ctx``) and exposes one method per
reference operator, under the reference's operator name:

=============================  ==================================================
method                          reference operator (exaDEM / exaNBody)
=============================  ==================================================
``update_particle_neighbors``   move_particles + chunk_neighbors_contact +
                                nbh_sphere (or nbh_polyhedron) + classify_interactions
                                + backup_r / backup_dem
``set_shapes``                  shape files of the deck (.shp)
``compute_vertices``            compute_vertices
``vertex_displ_over``           vertex_displ_over
``contact_polyhedron``          contact_polyhedron / contact_singlemat_polyhedron_hooke*
``particle_displ_over``         particle_displ_over
``reset_force_moment``          reset_force_moment
``gravity_force``               gravity_force
``contact_sphere``              contact_sphere / contact_singlemat_sphere_hooke_*
``force_to_accel``              force_to_accel
``combined_compute_prolog``     combined_compute_prolog
``combined_compute_epilog``     combined_compute_epilog
``simulation_state``            simulation_state
``first_iteration``             first_iteration block of main-config.msp
``step``                        compute_loop x n with numerical_scheme_verlet
=============================  ==================================================

Errors are raised as ``DemError`` (the reference prints and exits).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi as A


def make_params(bounds_lo, bounds_hi, periodic=(0, 0, 0), rcut_inc=0.05, dt=1e-3, gravity=(0.0, 0.0, -9.807),
                law=A.LAW_HOOKE_NONE, config=None, config_driver=None, cell_size=0.0, fp32_broad_phase=0,
                fp32_contact_screen=0, fused_step=0, graph_step=0, learned_sizing=0) -> A.Params:
    p = A.Params()
    p.bounds_lo[:] = list(map(float, bounds_lo))
    p.bounds_hi[:] = list(map(float, bounds_hi))
    p.periodic[:] = [int(bool(x)) for x in periodic]
    p.rcut_inc = rcut_inc
    p.cell_size = cell_size
    p.dt = dt
    p.gravity[:] = list(map(float, gravity))
    p.symetric = 1
    p.law = law
    p.config = contact_params(**(config or {}))
    p.config_driver = contact_params(**(config_driver or config or {}))
    p.fp32_broad_phase = int(fp32_broad_phase)
    p.fp32_contact_screen = int(fp32_contact_screen)
    p.fused_step = int(fused_step)
    p.graph_step = int(graph_step)
    p.learned_sizing = int(learned_sizing)
    return p


def contact_params(kn=1e4, kt=8e3, kr=0.0, mu=0.3, damp_rate=0.9, fc=0.0, dncut=0.0, gamma=0.0) -> A.ContactParams:
    """ContactParams YAML keys (contact_parameters.hpp:138-190); gamma: DMT adhesion energy."""
    return A.ContactParams(kn, kt, kr, mu, damp_rate, fc, dncut, gamma)


def empty_particles(n: int) -> dict:
    a = {f: np.zeros(n) for f in A.PARTICLE_FIELDS}
    a["id"] = np.zeros(n, dtype=np.uint64)
    a["type"] = np.zeros(n, dtype=np.uint32)
    a["group"] = np.zeros(n, dtype=np.uint32)
    return a


def _contig(arrays: dict) -> dict:
    out = {}
    for k, v in arrays.items():
        if v is None:
            continue
        if k == "id":
            out[k] = np.ascontiguousarray(v, dtype=np.uint64)
        elif k in ("type", "group"):
            out[k] = np.ascontiguousarray(v, dtype=np.uint32)
        else:
            out[k] = np.ascontiguousarray(v, dtype=np.float64)
    return out


class _Backend:
    """Function table: the native library (``dem_*``).  Tests build the same
    table over the oracle so both sides are driven by identical code."""

    prefix = "dem_"

    def __init__(self, lib):
        self.lib = lib

    def __getattr__(self, name):
        return getattr(self.lib, self.prefix + name)


class System:
    def __init__(self, params: A.Params, backend=None):
        self.b = backend or _Backend(A.load())
        self.params = params
        h = C.c_void_p()
        self._check(self.b.ctx_create(C.byref(params), C.byref(h)), "ctx_create")
        self.h = h
        self.n = 0

    # ------------------------------------------------------------ plumbing
    def _check(self, rc: int, where: str) -> None:
        if rc != A.DEM_OK:
            msg = ""
            if getattr(self, "h", None):
                try:
                    msg = (self.b.last_error(self.h) or b"").decode()
                except Exception:  # noqa: BLE001
                    msg = ""
            raise A.DemError(rc, where, msg)

    def close(self) -> None:
        if getattr(self, "h", None):
            self.b.ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -------------------------------------------------------------- state
    def set_params(self, params: A.Params) -> None:
        self._check(self.b.set_params(self.h, C.byref(params)), "set_params")
        self.params = params

    def set_particles(self, arrays: dict) -> None:
        arrays = _contig(arrays)
        n = len(arrays["rx"])
        st = A.particles_struct(arrays, n)
        self._check(self.b.set_particles(self.h, C.byref(st), 0), "set_particles")
        self.n = n

    def register_surface(self, offset, normal, center=(0, 0, 0), vel=(0, 0, 0), vrot=(0, 0, 0)) -> None:
        s = A.Surface(offset, (C.c_double * 3)(*normal), (C.c_double * 3)(*center), (C.c_double * 3)(*vel),
                      (C.c_double * 3)(*vrot))
        self._check(self.b.register_surface(self.h, C.byref(s)), "register_surface")

    def register_cylinder(self, radius, axis, center, vel=(0, 0, 0), vrot=(0, 0, 0)) -> None:
        c = A.Cylinder(radius, (C.c_double * 3)(*axis), (C.c_double * 3)(*center), (C.c_double * 3)(*vel),
                       (C.c_double * 3)(*vrot))
        self._check(self.b.register_cylinder(self.h, C.byref(c)), "register_cylinder")

    def register_mesh(self, vertices, edges, faces, minkowski, center=(0, 0, 0), quat=(1, 0, 0, 0)) -> None:
        """register_stl_mesh / register_rshape with STATIONARY motion: vertices (nv, 3) in
        the mesh frame, edges (ne, 2), faces (list of vertex lists), Minkowski radius,
        position and orientation (w, x, y, z).  exadem_gb300.stl builds these arrays
        from an STL file the way the reference converts it."""
        v = np.ascontiguousarray(np.asarray(vertices, dtype=np.float64).reshape(-1))
        e = np.ascontiguousarray(np.asarray(edges, dtype=np.int32).reshape(-1))
        off = np.zeros(len(faces) + 1, dtype=np.int32)
        off[1:] = np.cumsum([len(f) for f in faces])
        fv = np.ascontiguousarray(np.concatenate([np.asarray(f, dtype=np.int32) for f in faces])
                                  if len(faces) else np.zeros(0, np.int32))
        m = A.Mesh(len(v) // 3, len(e) // 2, len(faces), A.ptr(v), A.ptr(e, C.POINTER(C.c_int32)),
                   A.ptr(off, C.POINTER(C.c_int32)), A.ptr(fv, C.POINTER(C.c_int32)), float(minkowski),
                   (C.c_double * 3)(*center), (C.c_double * 4)(*quat))
        self._check(self.b.register_mesh(self.h, C.byref(m)), "register_mesh")

    def set_shapes(self, shapes: list) -> None:
        """shapes: dicts with vertices (nv,3), edges (ne,2), faces (list of vertex lists), radius,
        obb = dict(center, e1, e2, e3, extent) -- exaDEM's .shp content."""
        keep = []
        arr = (A.Shape * len(shapes))()
        for k, sh in enumerate(shapes):
            v = np.ascontiguousarray(np.asarray(sh["vertices"], dtype=np.float64).reshape(-1))
            e = np.ascontiguousarray(np.asarray(sh["edges"], dtype=np.int32).reshape(-1))
            fs = np.ascontiguousarray(np.array([len(f) for f in sh["faces"]], dtype=np.int32))
            fv = np.ascontiguousarray(np.concatenate([np.asarray(f, dtype=np.int32) for f in sh["faces"]]))
            keep += [v, e, fs, fv]
            o = sh["obb"]
            arr[k] = A.Shape(len(v) // 3, len(e) // 2, len(fs), A.ptr(v), A.ptr(e, C.POINTER(C.c_int32)),
                             A.ptr(fs, C.POINTER(C.c_int32)), A.ptr(fv, C.POINTER(C.c_int32)), float(sh["radius"]),
                             (C.c_double * 3)(*o["center"]), (C.c_double * 3)(*o["e1"]), (C.c_double * 3)(*o["e2"]),
                             (C.c_double * 3)(*o["e3"]), (C.c_double * 3)(*o["extent"]))
        self._check(self.b.set_shapes(self.h, arr, len(shapes)), "set_shapes")
        self._shapes_keep = keep

    def particles(self, sort_by_id: bool = True) -> dict:
        a = {f: np.zeros(self.n) for f in A.PARTICLE_FIELDS}
        a["id"] = np.zeros(self.n, dtype=np.uint64)
        a["type"] = np.zeros(self.n, dtype=np.uint32)
        a["group"] = np.zeros(self.n, dtype=np.uint32)
        st = A.particles_struct(a, self.n)
        self._check(self.b.get_particles(self.h, C.byref(st), 0), "get_particles")
        if sort_by_id:
            o = np.argsort(a["id"], kind="stable")
            a = {k: v[o] for k, v in a.items()}
        return a

    # ---------------------------------------------------------- operators
    def update_particle_neighbors(self) -> None:
        self._check(self.b.update_particle_neighbors(self.h), "update_particle_neighbors")

    def particle_displ_over(self) -> bool:
        r = C.c_int()
        self._check(self.b.particle_displ_over(self.h, C.byref(r)), "particle_displ_over")
        return bool(r.value)

    def reset_force_moment(self) -> None:
        self._check(self.b.reset_force_moment(self.h), "reset_force_moment")

    def gravity_force(self) -> None:
        self._check(self.b.gravity_force(self.h), "gravity_force")

    def contact_sphere(self) -> None:
        self._check(self.b.contact_sphere(self.h), "contact_sphere")

    def contact_polyhedron(self) -> None:
        self._check(self.b.contact_polyhedron(self.h), "contact_polyhedron")

    def compute_vertices(self) -> None:
        self._check(self.b.compute_vertices(self.h), "compute_vertices")

    def vertex_displ_over(self) -> bool:
        r = C.c_int()
        self._check(self.b.vertex_displ_over(self.h, C.byref(r)), "vertex_displ_over")
        return bool(r.value)

    def force_to_accel(self) -> None:
        self._check(self.b.force_to_accel(self.h), "force_to_accel")

    def combined_compute_prolog(self) -> None:
        self._check(self.b.combined_compute_prolog(self.h), "combined_compute_prolog")

    def combined_compute_epilog(self) -> None:
        self._check(self.b.combined_compute_epilog(self.h), "combined_compute_epilog")

    def first_iteration(self) -> None:
        self._check(self.b.first_iteration(self.h), "first_iteration")

    def step(self, nsteps: int = 1) -> None:
        self._check(self.b.step(self.h, int(nsteps)), "step")

    def rebuild_count(self) -> int:
        v = C.c_uint64()
        self._check(self.b.rebuild_count(self.h, C.byref(v)), "rebuild_count")
        return int(v.value)

    def simulation_state(self) -> dict:
        s = A.State()
        self._check(self.b.simulation_state(self.h, C.byref(s)), "simulation_state")
        return {"kinetic_energy": np.array(s.kinetic_energy[:]), "rotation_energy": np.array(s.rotation_energy[:]),
                "mass": s.mass, "n_particles": s.n_particles, "n_interactions": s.n_interactions,
                "n_active_interactions": s.n_active_interactions}

    # ------------------------------------------------------------ batching
    def set_systems(self, systems: list) -> None:
        """Independent systems in one context (dem_set_systems).  Each entry:
        dict(first, count, bounds_lo, bounds_hi, periodic, driver_first, driver_count)."""
        arr = (A.SystemDesc * len(systems))()
        for k, d in enumerate(systems):
            q = arr[k]
            q.first, q.count = int(d["first"]), int(d["count"])
            q.bounds_lo[:] = list(map(float, d["bounds_lo"]))
            q.bounds_hi[:] = list(map(float, d["bounds_hi"]))
            q.periodic[:] = [int(bool(x)) for x in d.get("periodic", (0, 0, 0))]
            q.driver_first = int(d.get("driver_first", 0))
            q.driver_count = int(d.get("driver_count", 0))
        self._check(self.b.set_systems(self.h, arr, len(systems)), "set_systems")

    def autotune(self, steps_per_trial: int = 5, skin_policy: int = 1) -> dict:
        """dem_autotune: cell size, launch shapes and (skin_policy) the skin."""
        r = A.TuneResult()
        self._check(self.b.autotune(self.h, int(steps_per_trial), int(skin_policy), C.byref(r)), "autotune")
        return {f: getattr(r, f) for f, _ in A.TuneResult._fields_}

    def set_multimat(self, pairs: list, drivers: list) -> None:
        """dem_set_multimat: pairs is an ngroups x ngroups nested list of ContactParams
        (symmetric), drivers an ngroups x ndrivers nested list; pairs = [] returns
        to the single parameter sets."""
        ng = len(pairs)
        nd = len(drivers[0]) if ng and drivers else 0
        pp = (A.ContactParams * max(ng * ng, 1))()
        pd = (A.ContactParams * max(ng * nd, 1))()
        for a in range(ng):
            for b in range(ng):
                pp[a * ng + b] = pairs[a][b]
            for d in range(nd):
                pd[a * nd + d] = drivers[a][d]
        self._check(self.b.set_multimat(self.h, ng, pp, nd, pd), "set_multimat")

    def set_analysis(self, on: bool) -> None:
        """dem_set_analysis: contact passes write the per-interaction contact state."""
        self._check(self.b.set_analysis(self.h, int(bool(on))), "set_analysis")

    def contact_state(self) -> dict:
        """dem_get_contact_state, in the order of interactions()."""
        cnt = self.interaction_count()
        out = {"dn": np.zeros(cnt), "cp": np.zeros(3 * cnt), "fn": np.zeros(3 * cnt), "ft": np.zeros(3 * cnt)}
        st = A.ContactState(cnt, 0, A.ptr(out["dn"]), A.ptr(out["cp"]), A.ptr(out["fn"]), A.ptr(out["ft"]))
        self._check(self.b.get_contact_state(self.h, C.byref(st)), "get_contact_state")
        return out

    def stress_tensor(self) -> tuple:
        """dem_stress_tensor: (per particle 9-component stress in the particles()
        order of sort_by_id=False, total over the particles)."""
        stress, total = np.zeros(9 * self.n), np.zeros(9)
        self._check(self.b.stress_tensor(self.h, A.ptr(stress), A.ptr(total)), "stress_tensor")
        return stress.reshape(self.n, 9), total

    def set_mul_mode(self, mode: int) -> None:
        """dem_set_mul_mode: which integration multiplies run on the integer pipe (same bits)."""
        self._check(self.b.set_mul_mode(self.h, int(mode)), "set_mul_mode")

    def set_contact_int_share(self, eighths: int) -> None:
        self._check(self.b.set_contact_int_share(self.h, int(eighths)), "set_contact_int_share")

    def set_sphere_cell_broad_phase(self, on: int) -> None:
        """dem_set_sphere_cell_broad_phase: warp-per-cell staged sphere broad phase (same lists)."""
        self._check(self.b.set_sphere_cell_broad_phase(self.h, int(on)), "set_sphere_cell_broad_phase")

    def mul_mode(self) -> int:
        v = C.c_int()
        self._check(self.b.get_mul_mode(self.h, C.byref(v)), "get_mul_mode")
        return int(v.value)

    def set_graph_capacity(self, capacity: int) -> None:
        self._check(self.b.set_graph_capacity(self.h, int(capacity)), "set_graph_capacity")

    def system_count(self) -> int:
        v = C.c_int()
        self._check(self.b.system_count(self.h, C.byref(v)), "system_count")
        return int(v.value)

    def system_states(self) -> list:
        ns = self.system_count()
        arr = (A.State * ns)()
        self._check(self.b.simulation_state_systems(self.h, arr, ns), "simulation_state_systems")
        return [{"kinetic_energy": np.array(s.kinetic_energy[:]), "rotation_energy": np.array(s.rotation_energy[:]),
                 "mass": s.mass, "n_particles": s.n_particles, "n_interactions": s.n_interactions,
                 "n_active_interactions": s.n_active_interactions} for s in arr]

    def interaction_count(self) -> int:
        v = C.c_uint64()
        self._check(self.b.interaction_count(self.h, C.byref(v)), "interaction_count")
        return int(v.value)

    def interactions(self) -> dict:
        m = self.interaction_count()
        out = {"owner_id": np.zeros(m, np.uint64), "partner_id": np.zeros(m, np.uint64),
               "type": np.zeros(m, np.uint16), "swap": np.zeros(m, np.uint8), "owner_sub": np.zeros(m, np.uint32),
               "partner_sub": np.zeros(m, np.uint32), "friction": np.zeros(3 * m), "moment": np.zeros(3 * m)}
        lst = A.InteractionList(m, 0, A.ptr(out["owner_id"], A.PU64), A.ptr(out["partner_id"], A.PU64),
                                A.ptr(out["type"], A.PU16), A.ptr(out["swap"], A.PU8),
                                A.ptr(out["owner_sub"], A.PU32), A.ptr(out["partner_sub"], A.PU32),
                                A.ptr(out["friction"]), A.ptr(out["moment"]))
        self._check(self.b.get_interactions(self.h, C.byref(lst)), "get_interactions")
        out["friction"] = out["friction"].reshape(-1, 3)
        out["moment"] = out["moment"].reshape(-1, 3)
        return out

    def set_interactions(self, lst: dict) -> None:
        """read_dump_particle_interaction's restore: the history of a saved list
        (a dict as interactions() returns) for the next neighbour build."""
        m = len(lst["owner_id"])
        a = {"owner_id": np.ascontiguousarray(lst["owner_id"], dtype=np.uint64),
             "partner_id": np.ascontiguousarray(lst["partner_id"], dtype=np.uint64),
             "type": np.ascontiguousarray(lst["type"], dtype=np.uint16),
             "swap": np.ascontiguousarray(lst["swap"], dtype=np.uint8),
             "owner_sub": np.ascontiguousarray(lst["owner_sub"], dtype=np.uint32),
             "partner_sub": np.ascontiguousarray(lst["partner_sub"], dtype=np.uint32),
             "friction": np.ascontiguousarray(np.asarray(lst["friction"], dtype=np.float64).reshape(-1)),
             "moment": np.ascontiguousarray(np.asarray(lst["moment"], dtype=np.float64).reshape(-1))}
        st = A.InteractionList(m, m, A.ptr(a["owner_id"], A.PU64), A.ptr(a["partner_id"], A.PU64),
                               A.ptr(a["type"], A.PU16), A.ptr(a["swap"], A.PU8), A.ptr(a["owner_sub"], A.PU32),
                               A.ptr(a["partner_sub"], A.PU32), A.ptr(a["friction"]), A.ptr(a["moment"]))
        self._check(self.b.set_interactions(self.h, C.byref(st)), "set_interactions")

    # ------------------------------------------------------- inner bonds
    def set_inner_bond_params(self, params) -> None:
        """inner_bond_params: one dict (kn, kt, damp_rate and g, or gn + gt, or g +
        sigma) for every pair, or an ngroups x ngroups nested list of them."""
        def one(d):
            if isinstance(d, A.InnerBondParams):
                return d
            if "sigma" in d:
                mode, c1, c2 = A.RUPTURE_STRESS_ENERGY_SEPARATE, d["g"], d["sigma"]
            elif "g" in d:
                mode, c1, c2 = A.RUPTURE_ENERGY_MIXED, d["g"], 0.0
            else:
                mode, c1, c2 = A.RUPTURE_ENERGY_SEPARATE, d["gn"], d["gt"]
            return A.InnerBondParams(float(d["kn"]), float(d["kt"]), float(d["damp_rate"]), mode, 0, float(c1),
                                     float(c2))
        if isinstance(params, (dict, A.InnerBondParams)):
            arr = (A.InnerBondParams * 1)(one(params))
            ng = 0
        else:
            ng = len(params)
            arr = (A.InnerBondParams * (ng * ng))(*[one(params[i][j]) for i in range(ng) for j in range(ng)])
        self._check(self.b.set_inner_bond_params(self.h, ng, arr), "set_inner_bond_params")

    def stick_polyhedra(self, ids, cluster, sticking_threshold: float) -> int:
        """stick_polyhedra: bonds between the touching faces of particles of the same cluster."""
        ids = np.ascontiguousarray(ids, dtype=np.uint64)
        cl = np.ascontiguousarray(cluster, dtype=np.float64)
        nb = C.c_uint64()
        self._check(self.b.stick_polyhedra(self.h, A.ptr(ids, A.PU64), A.ptr(cl), len(ids),
                                           float(sticking_threshold), C.byref(nb)), "stick_polyhedra")
        return int(nb.value)

    def bond_count(self) -> int:
        v = C.c_uint64()
        self._check(self.b.bond_count(self.h, C.byref(v)), "bond_count")
        return int(v.value)

    def bonds(self) -> dict:
        m = self.bond_count()
        out = {k: np.zeros(m * w, dtype=dt) for k, (dt, w) in A.BOND_COLUMNS.items()}
        st = A.bond_struct(out, m)
        self._check(self.b.get_bonds(self.h, C.byref(st)), "get_bonds")
        out["tds"] = out["tds"].reshape(-1, 3)
        out["friction"] = out["friction"].reshape(-1, 3)
        return out

    def bond_state(self) -> dict:
        """dem_get_bond_state: dn, fn (= f_i - friction) and the friction of each bond
        after the last bond pass, in the rows of bonds()."""
        m = self.bond_count()
        out = {"dn": np.zeros(m), "fn": np.zeros(3 * m), "ft": np.zeros(3 * m)}
        cnt = C.c_uint64()
        self._check(self.b.get_bond_state(self.h, m, C.byref(cnt), A.ptr(out["dn"]), A.ptr(out["fn"]),
                                          A.ptr(out["ft"])), "get_bond_state")
        out["fn"] = out["fn"].reshape(-1, 3)
        out["ft"] = out["ft"].reshape(-1, 3)
        return out

    def set_bonds(self, bonds: dict) -> None:
        """read_dump_particle_fragmentation's restore (a dict as bonds() returns)."""
        m = len(bonds["id_i"])
        cols = {k: np.ascontiguousarray(np.asarray(bonds[k], dtype=dt).reshape(-1))
                for k, (dt, _w) in A.BOND_COLUMNS.items()}
        st = A.bond_struct(cols, m, m)
        self._check(self.b.set_bonds(self.h, C.byref(st)), "set_bonds")

    def inner_bond_polyhedron(self) -> None:
        self._check(self.b.inner_bond_polyhedron(self.h), "inner_bond_polyhedron")

    def apply_interface_fracture_criterion(self) -> int:
        v = C.c_uint64()
        self._check(self.b.apply_interface_fracture_criterion(self.h, C.byref(v)),
                    "apply_interface_fracture_criterion")
        return int(v.value)

    def broken_interface_count(self) -> int:
        v = C.c_uint64()
        self._check(self.b.broken_interface_count(self.h, C.byref(v)), "broken_interface_count")
        return int(v.value)

    # ---------------------------------------------------------- profiling
    def profile(self, enable: bool = True) -> None:
        self._check(self.b.profile(self.h, int(enable)), "profile")

    def kernel_stats(self) -> dict:
        arr = (A.KernelStat * 64)()
        cnt = C.c_int()
        self._check(self.b.kernel_stats(self.h, arr, 64, C.byref(cnt)), "kernel_stats")
        return {arr[i].name.decode(): {"launches": arr[i].launches, "timed": arr[i].timed,
                                       "total_ms": arr[i].total_ms} for i in range(cnt.value)}

    def reset_kernel_stats(self) -> None:
        self._check(self.b.reset_kernel_stats(self.h), "reset_kernel_stats")

    def stream_handle(self) -> int:
        v = C.c_void_p()
        self._check(self.b.ctx_stream(self.h, C.byref(v)), "ctx_stream")
        return int(v.value or 0)

    def packing_profile(self, nslabs: int, zlo: float, zhi: float) -> np.ndarray:
        out = np.zeros(nslabs)
        self._check(self.b.packing_profile(self.h, int(nslabs), float(zlo), float(zhi), A.ptr(out)),
                    "packing_profile")
        return out


# Reference operator names -> System methods (what an .msp deck names).
OPERATORS = {
    "update_particle_neighbors": System.update_particle_neighbors,
    "chunk_neighbors_contact": System.update_particle_neighbors,
    "nbh_sphere": System.update_particle_neighbors,
    "particle_displ_over": System.particle_displ_over,
    "reset_force_moment": System.reset_force_moment,
    "gravity_force": System.gravity_force,
    "contact_sphere": System.contact_sphere,
    "contact_singlemat_sphere_hooke": System.contact_sphere,
    "contact_singlemat_sphere_hooke_none": System.contact_sphere,
    "contact_singlemat_sphere_hooke_cohesive": System.contact_sphere,
    "nbh_polyhedron": System.update_particle_neighbors,
    "contact_polyhedron": System.contact_polyhedron,
    "contact_singlemat_polyhedron_hooke": System.contact_polyhedron,
    "contact_singlemat_polyhedron_hooke_none": System.contact_polyhedron,
    "compute_vertices": System.compute_vertices,
    "vertex_displ_over": System.vertex_displ_over,
    "force_to_accel": System.force_to_accel,
    "combined_compute_prolog": System.combined_compute_prolog,
    "combined_compute_epilog": System.combined_compute_epilog,
    "simulation_state": System.simulation_state,
}
