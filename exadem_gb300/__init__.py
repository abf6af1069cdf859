"""GB300-native (sm_103a) implementation of exaDEM's per-timestep DEM hot path.

The compute path is the native library ``libexadem_gb300.so`` (C ABI declared
in ``include/dem_hotpath.h``); ``System`` mirrors the reference operators.
"""
from ._abi import DemError, load  # noqa: F401
from .system import OPERATORS, System, contact_params, empty_particles, make_params  # noqa: F401

__all__ = ["System", "make_params", "contact_params", "empty_particles", "OPERATORS", "DemError", "load"]
