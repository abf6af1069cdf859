"""Shared helpers of the parity tests: run a workload on the native library and
on the oracle with identical calls, and compare the results."""
from __future__ import annotations

import numpy as np

KEY = ["owner_id", "partner_id", "type", "swap", "owner_sub", "partner_sub"]
FIELDS_STATE = ["rx", "ry", "rz", "vx", "vy", "vz", "fx", "fy", "fz", "vrotx", "vroty", "vrotz",
                "arotx", "aroty", "arotz", "momx", "momy", "momz", "qw", "qx", "qy", "qz"]

# Tolerances of the parity contract: forces 1e-12 relative after one step,
# energies and packing profile 1e-9 relative after 100 steps.
FORCE_RTOL = 1e-12
ENERGY_RTOL = 1e-9


def assert_same_list(a: dict, b: dict) -> None:
    """Interaction list (sorted pair ids plus feature types) must match bit-exactly."""
    assert len(a["owner_id"]) == len(b["owner_id"]), (len(a["owner_id"]), len(b["owner_id"]))
    for k in KEY:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def assert_close_rel(x: np.ndarray, y: np.ndarray, rtol: float, name: str) -> None:
    """|x - y| <= rtol * max(|y|, scale) element-wise, scale = max |y| * rtol guard for zeros."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    scale = max(float(np.max(np.abs(y))) if y.size else 0.0, 1e-300)
    err = np.abs(x - y)
    lim = rtol * np.maximum(np.abs(y), scale * 1e-3)
    bad = err > lim
    assert not bad.any(), f"{name}: {bad.sum()} / {bad.size} entries off, max err {err.max():.3e}"


def assert_forces(a: dict, b: dict, rtol: float = FORCE_RTOL) -> None:
    for f in ["fx", "fy", "fz", "momx", "momy", "momz"]:
        assert_close_rel(a[f], b[f], rtol, f)


def assert_state(a: dict, b: dict, rtol: float, fields=FIELDS_STATE) -> None:
    np.testing.assert_array_equal(a["id"], b["id"])
    for f in fields:
        assert_close_rel(a[f], b[f], rtol, f)


def bit_equal_fraction(a: dict, b: dict, fields=FIELDS_STATE) -> float:
    tot = eq = 0
    for f in fields:
        tot += a[f].size
        eq += int(np.sum(a[f] == b[f]))
    return eq / max(tot, 1)


def pair(workload):
    """(native System, oracle System) loaded with the same workload."""
    from oracle.oracle import oracle_system

    return workload.build(), workload.build(oracle_system)
