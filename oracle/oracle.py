"""Python loader of the CPU oracle (test infrastructure only).

Only tests, the smoke check and the CPU-baseline leg of the benchmark use it,
as the checker.  It exposes the oracle's C functions through the same method
table as the native library, so ``exadem_gb300.system.System`` drives either
one with identical calls.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from exadem_gb300 import _abi as A
from exadem_gb300.system import System

from . import build as _build

_LIB = None
_CTX = C.c_void_p


def load(rebuild: bool = True):
    global _LIB
    if _LIB is None:
        path = _build.build() if rebuild else _build.LIB
        lib = C.CDLL(str(path))
        sig = lambda n, a, r=C.c_int: (setattr(getattr(lib, n), "argtypes", a), setattr(getattr(lib, n), "restype", r))
        sig("oracle_create", [C.POINTER(A.Params), C.POINTER(_CTX)])
        sig("oracle_set_params", [_CTX, C.POINTER(A.Params)])
        sig("oracle_set_multimat", [_CTX, C.c_int, C.POINTER(A.ContactParams), C.c_int, C.POINTER(A.ContactParams)])
        sig("oracle_set_analysis", [_CTX, C.c_int])
        sig("oracle_get_contact_state", [_CTX, C.POINTER(A.ContactState)])
        sig("oracle_stress_tensor", [_CTX, C.POINTER(C.c_double), C.POINTER(C.c_double)])
        sig("oracle_destroy", [_CTX])
        sig("oracle_set_threads", [C.c_int])
        sig("oracle_set_mesh_brute_force", [C.c_int])
        sig("oracle_last_error", [_CTX], C.c_char_p)
        sig("oracle_set_particles", [_CTX, C.POINTER(A.Particles)])
        sig("oracle_get_particles", [_CTX, C.POINTER(A.Particles)])
        sig("oracle_register_surface", [_CTX, C.POINTER(A.Surface)])
        sig("oracle_register_cylinder", [_CTX, C.POINTER(A.Cylinder)])
        sig("oracle_register_mesh", [_CTX, C.POINTER(A.Mesh)])
        sig("oracle_displ_over", [_CTX, C.POINTER(C.c_int)])
        for n in ["oracle_update_neighbors", "oracle_reset_force_moment", "oracle_gravity_force",
                  "oracle_contact_sphere", "oracle_force_to_accel", "oracle_prolog", "oracle_epilog",
                  "oracle_first_iteration"]:
            sig(n, [_CTX])
        sig("oracle_step", [_CTX, C.c_int])
        sig("oracle_rebuild_count", [_CTX, A.PU64])
        sig("oracle_state", [_CTX, C.POINTER(A.State)])
        sig("oracle_interaction_count", [_CTX, A.PU64])
        sig("oracle_get_interactions", [_CTX, C.POINTER(A.InteractionList)])
        sig("oracle_set_interactions", [_CTX, C.POINTER(A.InteractionList)])
        sig("oracle_packing_profile", [_CTX, C.c_int, C.c_double, C.c_double, A.PD])
        sig("oracle_set_shapes", [_CTX, C.POINTER(A.Shape), C.c_int])
        sig("oracle_compute_vertices", [_CTX])
        sig("oracle_set_inner_bond_params", [_CTX, C.c_int, C.POINTER(A.InnerBondParams)])
        sig("oracle_stick_polyhedra", [_CTX, A.PU64, A.PD, C.c_uint64, C.c_double, A.PU64])
        sig("oracle_bond_count", [_CTX, A.PU64])
        sig("oracle_get_bonds", [_CTX, C.POINTER(A.BondList)])
        sig("oracle_get_bond_state", [_CTX, C.c_uint64, A.PU64, A.PD, A.PD, A.PD])
        sig("oracle_set_bonds", [_CTX, C.POINTER(A.BondList)])
        sig("oracle_broken_interface_count", [_CTX, A.PU64])
        sig("oracle_inner_bond_polyhedron", [_CTX])
        sig("oracle_apply_interface_fracture_criterion", [_CTX, A.PU64])
        _LIB = lib
    return _LIB


class OracleBackend:
    _MAP = {"ctx_create": "oracle_create", "ctx_destroy": "oracle_destroy", "last_error": "oracle_last_error",
            "register_surface": "oracle_register_surface", "register_cylinder": "oracle_register_cylinder",
            "register_mesh": "oracle_register_mesh",
            "update_particle_neighbors": "oracle_update_neighbors", "particle_displ_over": "oracle_displ_over",
            "reset_force_moment": "oracle_reset_force_moment", "gravity_force": "oracle_gravity_force",
            "contact_sphere": "oracle_contact_sphere", "force_to_accel": "oracle_force_to_accel",
            "combined_compute_prolog": "oracle_prolog", "combined_compute_epilog": "oracle_epilog",
            "first_iteration": "oracle_first_iteration", "step": "oracle_step",
            "rebuild_count": "oracle_rebuild_count", "simulation_state": "oracle_state",
            "interaction_count": "oracle_interaction_count", "get_interactions": "oracle_get_interactions",
            "set_interactions": "oracle_set_interactions",
            "packing_profile": "oracle_packing_profile", "set_shapes": "oracle_set_shapes",
            "contact_polyhedron": "oracle_contact_sphere", "compute_vertices": "oracle_compute_vertices",
            "vertex_displ_over": "oracle_displ_over", "set_multimat": "oracle_set_multimat",
            "set_analysis": "oracle_set_analysis", "get_contact_state": "oracle_get_contact_state",
            "stress_tensor": "oracle_stress_tensor", "set_inner_bond_params": "oracle_set_inner_bond_params",
            "stick_polyhedra": "oracle_stick_polyhedra", "bond_count": "oracle_bond_count",
            "get_bonds": "oracle_get_bonds", "set_bonds": "oracle_set_bonds",
            "get_bond_state": "oracle_get_bond_state",
            "broken_interface_count": "oracle_broken_interface_count",
            "inner_bond_polyhedron": "oracle_inner_bond_polyhedron",
            "apply_interface_fracture_criterion": "oracle_apply_interface_fracture_criterion"}

    def __init__(self):
        self.lib = load()

    def set_particles(self, h, st, on_device=0):
        return self.lib.oracle_set_particles(h, st)

    def get_particles(self, h, st, on_device=0):
        return self.lib.oracle_get_particles(h, st)

    def set_params(self, h, p):
        return self.lib.oracle_set_params(h, p)

    def __getattr__(self, name):
        return getattr(self.lib, self._MAP[name])


def set_threads(n: int) -> int:
    return load().oracle_set_threads(int(n))


def oracle_system(params: A.Params) -> System:
    return System(params, backend=OracleBackend())
