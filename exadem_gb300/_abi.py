"""ctypes mirror of ``include/dem_hotpath.h`` and ``include/dem_workloads.h``.

Loads the in-tree ``libexadem_gb300.so``.  There is no fallback: if the library
is missing the import of the compute path raises, so a GPU run can never
silently take another path.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libexadem_gb300.so"
# the seeded input generator (include/dem_workloads.h), host code in a library of its own
WORKLOADS_LIB_PATH = PKG / "libdem_workloads.so"

DEM_OK = 0
ERRORS = {1: "DEM_ERR_INVALID_ARG", 2: "DEM_ERR_CUDA", 3: "DEM_ERR_OOM", 4: "DEM_ERR_UNSUPPORTED",
          5: "DEM_ERR_OVERFLOW", 6: "DEM_ERR_TIMEOUT", 7: "DEM_ERR_STATE", 8: "DEM_ERR_NO_DEVICE"}

ITYPE_VERTEX_VERTEX = 0
ITYPE_VERTEX_EDGE = 1
ITYPE_VERTEX_FACE = 2
ITYPE_EDGE_EDGE = 3
ITYPE_VERTEX_CYLINDER = 4
ITYPE_VERTEX_SURFACE = 5
LAW_HOOKE_NONE = 0
LAW_HOOKE_COHESIVE = 1
LAW_HOOKE_DMT = 2

D = C.c_double
PD = C.POINTER(C.c_double)
PU64 = C.POINTER(C.c_uint64)
PU32 = C.POINTER(C.c_uint32)
PU16 = C.POINTER(C.c_uint16)
PU8 = C.POINTER(C.c_uint8)


class ContactParams(C.Structure):
    _fields_ = [("kn", D), ("kt", D), ("kr", D), ("mu", D), ("damp_rate", D), ("fc", D), ("dncut", D),
                ("gamma", D)]


class Params(C.Structure):
    _fields_ = [("bounds_lo", D * 3), ("bounds_hi", D * 3), ("periodic", C.c_int32 * 3),
                ("rcut_inc", D), ("cell_size", D), ("dt", D), ("gravity", D * 3),
                ("symetric", C.c_int32), ("law", C.c_int32),
                ("config", ContactParams), ("config_driver", ContactParams),
                ("fp32_broad_phase", C.c_int32), ("fp32_contact_screen", C.c_int32),
                ("fused_step", C.c_int32), ("graph_step", C.c_int32), ("learned_sizing", C.c_int32),
                ("reserved", C.c_int32 * 3)]


PARTICLE_FIELDS = ["rx", "ry", "rz", "vx", "vy", "vz", "fx", "fy", "fz",
                   "vrotx", "vroty", "vrotz", "arotx", "aroty", "arotz", "momx", "momy", "momz",
                   "qw", "qx", "qy", "qz", "inertiax", "inertiay", "inertiaz", "mass", "radius", "homothety"]


class Particles(C.Structure):
    _fields_ = [("n", C.c_uint64)] + [(f, PD) for f in PARTICLE_FIELDS] + [
        ("id", PU64), ("type", PU32), ("group", PU32)]


class Surface(C.Structure):
    _fields_ = [("offset", D), ("normal", D * 3), ("center", D * 3), ("vel", D * 3), ("vrot", D * 3)]


class Cylinder(C.Structure):
    _fields_ = [("radius", D), ("axis", D * 3), ("center", D * 3), ("vel", D * 3), ("vrot", D * 3)]


class Mesh(C.Structure):
    _fields_ = [("nv", C.c_int32), ("ne", C.c_int32), ("nf", C.c_int32), ("vertices", C.POINTER(D)),
                ("edges", C.POINTER(C.c_int32)), ("face_offsets", C.POINTER(C.c_int32)),
                ("face_vertices", C.POINTER(C.c_int32)), ("minkowski", D), ("center", D * 3), ("quat", D * 4)]


class State(C.Structure):
    _fields_ = [("kinetic_energy", D * 3), ("rotation_energy", D * 3), ("mass", D),
                ("n_particles", C.c_uint64), ("n_interactions", C.c_uint64),
                ("n_active_interactions", C.c_uint64)]


class SystemDesc(C.Structure):
    """dem_system: one independent system of a batched context."""
    _fields_ = [("first", C.c_uint64), ("count", C.c_uint64), ("bounds_lo", D * 3), ("bounds_hi", D * 3),
                ("periodic", C.c_int32 * 3), ("driver_first", C.c_int32), ("driver_count", C.c_int32)]


class TuneResult(C.Structure):
    _fields_ = [("rcut_inc", D), ("cell_size", D), ("block", C.c_int32), ("contact_blocks_per_sm", C.c_int32),
                ("ms_per_step", D), ("ms_per_step_before", D), ("trials", C.c_int32), ("vmax", C.c_float),
                ("mul_mode", C.c_int32), ("fused_contact", C.c_int32), ("contact_int_share", C.c_int32)]


class ContactState(C.Structure):
    _fields_ = [("capacity", C.c_uint64), ("count", C.c_uint64), ("dn", PD), ("cp", PD), ("fn", PD), ("ft", PD)]


class InteractionList(C.Structure):
    _fields_ = [("capacity", C.c_uint64), ("count", C.c_uint64), ("owner_id", PU64), ("partner_id", PU64),
                ("type", PU16), ("swap", PU8), ("owner_sub", PU32), ("partner_sub", PU32),
                ("friction", PD), ("moment", PD)]


class InnerBondParams(C.Structure):
    _fields_ = [("kn", D), ("kt", D), ("damp_rate", D), ("mode", C.c_int32), ("pad", C.c_int32), ("crit1", D),
                ("crit2", D)]


class BondList(C.Structure):
    _fields_ = [("capacity", C.c_uint64), ("count", C.c_uint64), ("id_i", PU64), ("id_j", PU64), ("sub_i", PU32),
                ("sub_j", PU32), ("dn0", PD), ("weight", PD), ("mode", C.POINTER(C.c_int32)), ("crit1", PD),
                ("crit2", PD), ("en", PD), ("et", PD), ("tds", PD), ("friction", PD), ("unbroken", PU8)]


RUPTURE_ENERGY_MIXED, RUPTURE_ENERGY_SEPARATE, RUPTURE_STRESS_ENERGY_SEPARATE = 0, 1, 2

# dem_bond_list columns: name -> (dtype, values per row)
BOND_COLUMNS = {"id_i": (np.uint64, 1), "id_j": (np.uint64, 1), "sub_i": (np.uint32, 1), "sub_j": (np.uint32, 1),
                "dn0": (np.float64, 1), "weight": (np.float64, 1), "mode": (np.int32, 1), "crit1": (np.float64, 1),
                "crit2": (np.float64, 1), "en": (np.float64, 1), "et": (np.float64, 1), "tds": (np.float64, 3),
                "friction": (np.float64, 3), "unbroken": (np.uint8, 1)}


def bond_struct(cols: dict, capacity: int, count: int = 0) -> BondList:
    """A dem_bond_list over the arrays of `cols` (BOND_COLUMNS names)."""
    types = {np.uint64: PU64, np.uint32: PU32, np.float64: PD, np.int32: C.POINTER(C.c_int32), np.uint8: PU8}
    st = BondList()
    st.capacity = capacity
    st.count = count
    for k, (dt, _w) in BOND_COLUMNS.items():
        setattr(st, k, ptr(cols[k], types[dt]))
    return st


class KernelStat(C.Structure):
    _fields_ = [("name", C.c_char * 24), ("launches", C.c_uint64), ("timed", C.c_uint64), ("total_ms", D)]


class RsaSpec(C.Structure):
    _fields_ = [("n", C.c_uint64), ("rmin", D), ("rmax", D), ("density", D), ("lo", D * 3), ("hi", D * 3),
                ("periodic", C.c_int32 * 3), ("grow_axis", C.c_int32), ("region", C.c_int32),
                ("cyl_center", D * 2), ("cyl_radius", D), ("vmin", D), ("vmax", D), ("seed", C.c_uint64),
                ("max_attempts", C.c_uint64), ("id_offset", C.c_uint64), ("radii", PD)]


class Shape(C.Structure):
    _fields_ = [("nv", C.c_int32), ("ne", C.c_int32), ("nf", C.c_int32), ("vertices", PD),
                ("edges", C.POINTER(C.c_int32)), ("face_sizes", C.POINTER(C.c_int32)),
                ("face_vertices", C.POINTER(C.c_int32)), ("radius", D), ("obb_center", D * 3), ("obb_e1", D * 3),
                ("obb_e2", D * 3), ("obb_e3", D * 3), ("obb_extent", D * 3)]


def ptr(a: np.ndarray | None, ctype=PD):
    if a is None:
        return C.cast(None, ctype)
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctype)


def particles_struct(arrays: dict, n: int) -> Particles:
    """Builds a Particles view over numpy arrays (kept alive by the caller)."""
    p = Particles()
    p.n = n
    for f in PARTICLE_FIELDS:
        setattr(p, f, ptr(arrays.get(f)))
    p.id = ptr(arrays.get("id"), PU64)
    p.type = ptr(arrays.get("type"), PU32)
    p.group = ptr(arrays.get("group"), PU32)
    return p


# ---- function signatures shared by the library and the oracle ---------------
_CTX = C.c_void_p


def _sig(lib, name, args, res=C.c_int):
    fn = getattr(lib, name)
    fn.argtypes = args
    fn.restype = res
    return fn


def declare_library(lib) -> None:
    _sig(lib, "dem_ctx_create", [C.POINTER(Params), C.POINTER(_CTX)])
    _sig(lib, "dem_ctx_destroy", [_CTX])
    _sig(lib, "dem_last_error", [_CTX], C.c_char_p)
    _sig(lib, "dem_ctx_stream", [_CTX, C.POINTER(C.c_void_p)])
    _sig(lib, "dem_set_params", [_CTX, C.POINTER(Params)])
    _sig(lib, "dem_set_particles", [_CTX, C.POINTER(Particles), C.c_int])
    _sig(lib, "dem_get_particles", [_CTX, C.POINTER(Particles), C.c_int])
    _sig(lib, "dem_register_surface", [_CTX, C.POINTER(Surface)])
    _sig(lib, "dem_register_cylinder", [_CTX, C.POINTER(Cylinder)])
    _sig(lib, "dem_register_mesh", [_CTX, C.POINTER(Mesh)])
    _sig(lib, "dem_particle_displ_over", [_CTX, C.POINTER(C.c_int)])
    for name in ["dem_update_particle_neighbors", "dem_reset_force_moment", "dem_gravity_force",
                 "dem_contact_sphere", "dem_force_to_accel", "dem_combined_compute_prolog",
                 "dem_combined_compute_epilog", "dem_first_iteration"]:
        _sig(lib, name, [_CTX])
    _sig(lib, "dem_step", [_CTX, C.c_int])
    _sig(lib, "dem_set_shapes", [_CTX, C.POINTER(Shape), C.c_int])
    _sig(lib, "dem_compute_vertices", [_CTX])
    _sig(lib, "dem_contact_polyhedron", [_CTX])
    _sig(lib, "dem_vertex_displ_over", [_CTX, C.POINTER(C.c_int)])
    _sig(lib, "dem_rebuild_count", [_CTX, PU64])
    _sig(lib, "dem_simulation_state", [_CTX, C.POINTER(State)])
    _sig(lib, "dem_set_systems", [_CTX, C.POINTER(SystemDesc), C.c_int])
    _sig(lib, "dem_set_graph_capacity", [_CTX, C.c_uint64])
    _sig(lib, "dem_autotune", [_CTX, C.c_int, C.c_int, C.POINTER(TuneResult)])
    _sig(lib, "dem_set_mul_mode", [_CTX, C.c_int])
    _sig(lib, "dem_set_contact_int_share", [_CTX, C.c_int])
    _sig(lib, "dem_set_sphere_cell_broad_phase", [_CTX, C.c_int])
    _sig(lib, "dem_set_multimat", [_CTX, C.c_int, C.POINTER(ContactParams), C.c_int, C.POINTER(ContactParams)])
    _sig(lib, "dem_set_analysis", [_CTX, C.c_int])
    _sig(lib, "dem_get_contact_state", [_CTX, C.POINTER(ContactState)])
    _sig(lib, "dem_stress_tensor", [_CTX, PD, PD])
    _sig(lib, "dem_get_mul_mode", [_CTX, C.POINTER(C.c_int)])
    VP = C.c_void_p
    _sig(lib, "dem_mlp_harvest", [_CTX, VP, VP, C.c_uint64, PU64, PU64])
    _sig(lib, "dem_mlp_init", [_CTX, C.c_uint64, C.POINTER(C.c_float)])
    _sig(lib, "dem_mlp_set_params", [_CTX, C.POINTER(C.c_float)])
    _sig(lib, "dem_mlp_get_params", [_CTX, C.POINTER(C.c_float)])
    _sig(lib, "dem_mlp_forward", [_CTX, VP, C.c_uint64, VP])
    _sig(lib, "dem_mlp_loss_grad", [_CTX, VP, VP, C.c_uint64, C.POINTER(C.c_float), PD])
    _sig(lib, "dem_mlp_train", [_CTX, VP, VP, C.c_uint64, C.c_int, C.c_uint64, C.c_float, C.c_uint64, PD])
    _sig(lib, "dem_learned_stats", [_CTX, PU64, PU64, PU64])
    _sig(lib, "dem_system_count", [_CTX, C.POINTER(C.c_int)])
    _sig(lib, "dem_simulation_state_systems", [_CTX, C.POINTER(State), C.c_int])
    _sig(lib, "dem_interaction_count", [_CTX, PU64])
    _sig(lib, "dem_get_interactions", [_CTX, C.POINTER(InteractionList)])
    _sig(lib, "dem_set_interactions", [_CTX, C.POINTER(InteractionList)])
    _sig(lib, "dem_packing_profile", [_CTX, C.c_int, D, D, PD])
    _sig(lib, "dem_set_inner_bond_params", [_CTX, C.c_int, C.POINTER(InnerBondParams)])
    _sig(lib, "dem_stick_polyhedra", [_CTX, PU64, PD, C.c_uint64, D, PU64])
    _sig(lib, "dem_bond_count", [_CTX, PU64])
    _sig(lib, "dem_get_bonds", [_CTX, C.POINTER(BondList)])
    _sig(lib, "dem_get_bond_state", [_CTX, C.c_uint64, PU64, PD, PD, PD])
    _sig(lib, "dem_set_bonds", [_CTX, C.POINTER(BondList)])
    _sig(lib, "dem_broken_interface_count", [_CTX, PU64])
    _sig(lib, "dem_inner_bond_polyhedron", [_CTX])
    _sig(lib, "dem_apply_interface_fracture_criterion", [_CTX, PU64])
    _sig(lib, "dem_profile", [_CTX, C.c_int])
    _sig(lib, "dem_kernel_stats", [_CTX, C.POINTER(KernelStat), C.c_int, C.POINTER(C.c_int)])
    _sig(lib, "dem_reset_kernel_stats", [_CTX])
    _sig(lib, "dem_simulation_state_noalloc", [C.POINTER(Particles), PD, C.c_void_p])
    _sig(lib, "dem_selftest_division", [C.c_uint64, C.c_uint64, PU64, PU64])
    _sig(lib, "dem_selftest_poly_decisions", [C.c_uint64, C.c_uint64, PU64])
    _sig(lib, "dem_selftest_emu_mul", [C.c_uint64, C.c_uint64, PU64])
    _sig(lib, "dem_selftest_rolling_clip", [C.c_uint64, C.c_uint64, PU64, PU64])


# Symbols declared in include/dem_hotpath.h, dem_selftest.h and dem_learned.h (the product library).
EXPORTED = ["dem_ctx_create", "dem_ctx_destroy", "dem_last_error", "dem_ctx_stream", "dem_set_params",
            "dem_set_particles", "dem_get_particles", "dem_register_surface", "dem_register_cylinder",
            "dem_register_mesh",
            "dem_particle_displ_over", "dem_update_particle_neighbors", "dem_reset_force_moment",
            "dem_gravity_force", "dem_contact_sphere", "dem_force_to_accel", "dem_combined_compute_prolog",
            "dem_combined_compute_epilog", "dem_simulation_state", "dem_first_iteration", "dem_step",
            "dem_rebuild_count", "dem_interaction_count", "dem_get_interactions", "dem_set_interactions", "dem_packing_profile",
            "dem_profile", "dem_kernel_stats", "dem_reset_kernel_stats",
            "dem_simulation_state_noalloc", "dem_selftest_division", "dem_selftest_poly_decisions", "dem_selftest_emu_mul", "dem_selftest_rolling_clip", "dem_set_shapes", "dem_compute_vertices",
            "dem_contact_polyhedron", "dem_vertex_displ_over", "dem_set_systems", "dem_system_count",
            "dem_simulation_state_systems", "dem_set_graph_capacity", "dem_autotune", "dem_set_mul_mode", "dem_get_mul_mode", "dem_set_multimat", "dem_set_analysis", "dem_get_contact_state", "dem_stress_tensor", "dem_mlp_harvest",
            "dem_mlp_init", "dem_mlp_set_params", "dem_mlp_get_params", "dem_mlp_forward", "dem_mlp_loss_grad",
            "dem_mlp_train", "dem_learned_stats", "dem_set_inner_bond_params", "dem_stick_polyhedra",
            "dem_bond_count", "dem_get_bonds", "dem_set_bonds", "dem_broken_interface_count",
            "dem_inner_bond_polyhedron", "dem_apply_interface_fracture_criterion", "dem_set_contact_int_share",
            "dem_set_sphere_cell_broad_phase", "dem_get_bond_state"]

_LIB = None


def load(path: Path | None = None):
    """Loads (once) and returns the native library; raises if it is not built."""
    global _LIB
    if _LIB is None:
        p = Path(path) if path else LIB_PATH
        if not p.exists():
            raise RuntimeError(f"native library missing: {p} (run exadem_gb300.build.build())")
        lib = C.CDLL(str(p))
        declare_library(lib)
        _LIB = lib
    return _LIB


WORKLOADS_EXPORTED = ["dem_generate_rsa_spheres"]
_WLIB = None


def load_workloads(path: Path | None = None):
    """Loads (once) the input generator library (host code, no CUDA)."""
    global _WLIB
    if _WLIB is None:
        p = Path(path) if path else WORKLOADS_LIB_PATH
        if not p.exists():
            raise RuntimeError(f"generator library missing: {p} (run exadem_gb300.build.build())")
        lib = C.CDLL(str(p))
        _sig(lib, "dem_generate_rsa_spheres", [C.POINTER(RsaSpec), C.POINTER(Particles), PD])
        _WLIB = lib
    return _WLIB


class DemError(RuntimeError):
    def __init__(self, code: int, where: str, msg: str = ""):
        super().__init__(f"{where}: {ERRORS.get(code, code)} {msg}".strip())
        self.code = code
