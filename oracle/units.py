"""Seeded cases for the per-function comparison of the oracle with exaDEM's own
functions (test infrastructure only).

``oracle/ref_harness.cpp`` (exaDEM's headers compiled on the host) and
``oracle/dem_oracle.cpp`` export the same batch entry points, ``ref_unit_<name>``
and ``oracle_unit_<name>``, over rows of doubles.  ``cases(name, n, seed)``
draws n input rows for one of them, mixing random draws with the edge cases the
functions branch on (thresholds met exactly, zeros, degenerate geometry);
``run(lib, prefix, name, rows)`` calls one library and returns its output rows.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

PD = C.POINTER(C.c_double)

# name -> (input width, output width, extra leading integer argument or None)
LAYOUT = {
    "contact_force_core": (45, 12, "law"),
    "damping": (5, 2, None),
    "detect_vv": (8, 8, None),
    "detect_ve": (11, 8, None),
    "detect_ee": (14, 8, None),
    "filter_vv": (9, 1, None),
    "filter_ve": (12, 1, None),
    "filter_ee": (15, 1, None),
    "world_vertex": (11, 3, None),
    "obb_intersect": (30, 1, None),
    "compute_obb": (24, 15, None),
    "push_quaternion": (11, 7, None),
    "angular": (15, 6, None),
    "surface": (11, 13, None),
    "cylinder": (11, 13, None),
    "bond_law": (35, 20, None),
}
FILTER_KIND = {"filter_vv": 0, "filter_ve": 1, "filter_ee": 2}


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(PD)


def run(lib, prefix: str, name: str, rows: np.ndarray, law: int = 0) -> np.ndarray:
    """Output rows of ``<prefix>_unit_<name>`` on the input rows."""
    kin, kout, extra = LAYOUT[name]
    rows = np.ascontiguousarray(rows, dtype=np.float64).reshape(-1, kin)
    n = rows.shape[0]
    out = np.zeros((n, kout), dtype=np.float64)
    if name in FILTER_KIND:
        fn = getattr(lib, f"{prefix}_unit_filter")
        fn.argtypes = [C.c_int, C.c_long, PD, PD]
        rc = fn(FILTER_KIND[name], n, _ptr(rows), _ptr(out))
    elif extra == "law":
        fn = getattr(lib, f"{prefix}_unit_{name}")
        fn.argtypes = [C.c_int, C.c_long, PD, PD]
        rc = fn(law, n, _ptr(rows), _ptr(out))
    else:
        fn = getattr(lib, f"{prefix}_unit_{name}")
        fn.argtypes = [C.c_long, PD, PD]
        rc = fn(n, _ptr(rows), _ptr(out))
    assert rc == 0, f"{prefix}_unit_{name} returned {rc}"
    return out


def run_pair_order(lib, prefix: str, keys: np.ndarray) -> np.ndarray:
    keys = np.ascontiguousarray(keys, dtype=np.uint64).reshape(-1, 12)
    out = np.zeros((keys.shape[0], 2), dtype=np.int32)
    fn = getattr(lib, f"{prefix}_unit_pair_order")
    fn.argtypes = [C.c_long, C.POINTER(C.c_uint64), C.POINTER(C.c_int32)]
    assert fn(keys.shape[0], keys.ctypes.data_as(C.POINTER(C.c_uint64)), out.ctypes.data_as(C.POINTER(C.c_int32))) == 0
    return out


# ----------------------------------------------------------------- generators
def _unit(rng, n):
    v = rng.standard_normal((n, 3))
    return v / np.linalg.norm(v, axis=1)[:, None]


def _quat(rng, n, off_unit=0.0):
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1)[:, None]
    if off_unit:
        q *= (1.0 + off_unit * rng.uniform(-1, 1, (n, 1)))
    return q


def _maybe_zero(rng, a, frac):
    a = a.copy()
    a[rng.random(a.shape[0]) < frac] = 0.0
    return a


def _rotmat(q):
    w, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
        np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
        np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1)], -2)


def cases(name: str, n: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return _GEN[name](rng, n)


def _contact_force_core(rng, n):
    r = np.zeros((n, 45))
    u = rng.random(n)
    # overlap: mostly small penetrations, with exact zeros, the cohesion distance and positives
    dn = -10.0 ** rng.uniform(-8, -1, n)
    dn = np.where(u < 0.08, 0.0, dn)
    dn = np.where((u >= 0.08) & (u < 0.16), 0.01, dn)
    dn = np.where((u >= 0.16) & (u < 0.30), rng.uniform(0, 0.02, n), dn)
    r[:, 0] = dn
    r[:, 1:4] = _unit(rng, n)
    r[:, 4] = 10.0 ** rng.uniform(-5, -3, n)                       # dt
    kn = 10.0 ** rng.uniform(3, 6, n)
    r[:, 5] = kn
    r[:, 6] = kn * rng.uniform(0.5, 1.0, n)                        # kt
    r[:, 7] = np.where(rng.random(n) < 0.5, 0.0, rng.uniform(0, 200, n))  # kr
    r[:, 8] = np.where(rng.random(n) < 0.05, 0.0, rng.uniform(0, 1, n))   # mu
    r[:, 9] = np.where(rng.random(n) < 0.05, 0.0, rng.uniform(0, 1, n))   # damp_rate
    r[:, 10] = np.where(rng.random(n) < 0.3, 0.0, rng.uniform(0, 20, n))  # fc
    r[:, 11] = np.where(rng.random(n) < 0.1, 0.0, 0.01)                   # dncut
    r[:, 12] = np.where(rng.random(n) < 0.3, 0.0, rng.uniform(0, 1, n))   # gamma
    r[:, 13] = 10.0 ** rng.uniform(-3, 1, n)                       # meff
    r[:, 14] = rng.uniform(0.05, 1.0, n)                           # reff
    r[:, 15:18] = _maybe_zero(rng, rng.standard_normal((n, 3)) * 10.0 ** rng.uniform(-6, 1, (n, 1)), 0.3)  # ft
    pos_i = rng.uniform(-5, 5, (n, 3))
    r[:, 21:24] = pos_i
    r[:, 18:21] = pos_i + rng.standard_normal((n, 3)) * 0.5        # contact point
    r[:, 24:27] = rng.standard_normal((n, 3))                      # vel_i
    r[:, 27:30] = _maybe_zero(rng, rng.standard_normal((n, 3)), 0.8)       # f_i (zero as the callers pass)
    r[:, 30:33] = _maybe_zero(rng, rng.standard_normal((n, 3)) * 10.0 ** rng.uniform(-8, 0, (n, 1)), 0.3)  # mom_i
    w_i = rng.standard_normal((n, 3)) * 10.0 ** rng.uniform(-6, 1, (n, 1))
    k = rng.random(n)
    w_i[k < 0.2] = 0.0                                             # spin exactly zero: the 0/0 quirk
    w_i[(k >= 0.2) & (k < 0.25), 1:] = 0.0
    r[:, 33:36] = w_i
    r[:, 36:39] = pos_i + rng.standard_normal((n, 3))              # pos_j
    r[:, 39:42] = rng.standard_normal((n, 3))
    r[:, 42:45] = _maybe_zero(rng, rng.standard_normal((n, 3)), 0.3)
    return r


def _bond_law(rng, n):
    """force_law_core inputs: dn around dn0 on both sides (tension and compression,
    delta exactly 0), weights 1/k, zero and nonzero cumulated displacements and spins."""
    r = np.zeros((n, 35))
    dn0 = np.where(rng.random(n) < 0.3, 0.0, rng.standard_normal(n) * 1e-6)
    u = rng.random(n)
    dn = dn0 + rng.standard_normal(n) * 10.0 ** rng.uniform(-9, -2, n)
    dn = np.where(u < 0.1, dn0, dn)                                 # delta exactly zero
    r[:, 0] = dn
    r[:, 1:4] = _unit(rng, n)
    r[:, 4] = dn0
    r[:, 5] = 1.0 / rng.integers(1, 9, n)                          # weight 1/(bonds of the interface)
    r[:, 6] = 10.0 ** rng.uniform(-5, -3, n)                       # dt
    kn = 10.0 ** rng.uniform(3, 7, n)
    r[:, 7] = kn
    r[:, 8] = kn * rng.uniform(0.5, 1.0, n)                        # kt
    r[:, 9] = np.where(rng.random(n) < 0.05, 0.0, rng.uniform(0, 1, n))  # damp_rate
    r[:, 10] = 10.0 ** rng.uniform(-3, 1, n)                       # meff
    r[:, 11:14] = _maybe_zero(rng, rng.standard_normal((n, 3)) * 10.0 ** rng.uniform(-9, -3, (n, 1)), 0.3)  # tds
    pos_i = rng.uniform(-5, 5, (n, 3))
    r[:, 17:20] = pos_i
    r[:, 14:17] = pos_i + rng.standard_normal((n, 3)) * 0.5        # contact point
    r[:, 20:23] = _maybe_zero(rng, rng.standard_normal((n, 3)), 0.2)
    r[:, 23:26] = _maybe_zero(rng, rng.standard_normal((n, 3)), 0.4)
    r[:, 26:29] = pos_i + rng.standard_normal((n, 3))              # pos_j
    r[:, 29:32] = _maybe_zero(rng, rng.standard_normal((n, 3)), 0.2)
    r[:, 32:35] = _maybe_zero(rng, rng.standard_normal((n, 3)), 0.4)
    return r


def _damping(rng, n):
    r = np.zeros((n, 5))
    r[:, 0] = rng.uniform(0, 1, n)
    r[:, 1] = 10.0 ** rng.uniform(2, 7, n)
    r[:, 2] = 10.0 ** rng.uniform(-4, 2, n)
    r[:, 3] = np.where(rng.random(n) < 0.2, r[:, 2], 10.0 ** rng.uniform(-4, 2, n))
    return r


def _pair_points(rng, n, scale=1.0):
    a = rng.uniform(-3, 3, (n, 3))
    return a, a + _unit(rng, n) * rng.uniform(0, 2 * scale, (n, 1))


def _detect_vv(rng, n):
    r = np.zeros((n, 8))
    a, b = _pair_points(rng, n)
    same = rng.random(n) < 0.005
    b[same] = a[same]                                                # coincident centres
    r[:, 0:3], r[:, 4:7] = a, b
    r[:, 3] = rng.uniform(0.01, 0.6, n)
    r[:, 7] = rng.uniform(0.01, 0.6, n)
    # exact touching distance along an axis: dn = 0
    t = rng.random(n) < 0.05
    r[t, 4:7] = r[t, 0:3]
    r[t, 4] = r[t, 0] + (r[t, 3] + r[t, 7])
    return r


def _segment(rng, n, center, length=1.0):
    d = _unit(rng, n) * rng.uniform(0.1, length, (n, 1))
    return center - 0.5 * d, center + 0.5 * d


def _detect_ve(rng, n):
    r = np.zeros((n, 11))
    c = rng.uniform(-2, 2, (n, 3))
    f, s = _segment(rng, n, c)
    t = rng.uniform(-0.3, 1.3, (n, 1))
    t[rng.random(n) < 0.05] = 0.0
    t[rng.random(n) < 0.05] = 1.0
    foot = f + t * (s - f)
    vi = foot + _unit(rng, n) * rng.uniform(0, 0.1, (n, 1))
    r[:, 0:3], r[:, 4:7], r[:, 7:10] = vi, f, s
    r[:, 3] = rng.uniform(0.001, 0.05, n)
    r[:, 10] = rng.uniform(0.001, 0.05, n)
    return r


def _detect_ee(rng, n):
    r = np.zeros((n, 14))
    c = rng.uniform(-2, 2, (n, 3))
    fi, si = _segment(rng, n, c)
    cj = c + _unit(rng, n) * rng.uniform(0, 0.1, (n, 1))
    fj, sj = _segment(rng, n, cj)
    par = rng.random(n) < 0.05                                       # parallel edges: |f| below 1e-12
    fj[par] = fi[par] + (cj - c)[par]
    sj[par] = si[par] + (cj - c)[par]
    r[:, 0:3], r[:, 3:6], r[:, 7:10], r[:, 10:13] = fi, si, fj, sj
    r[:, 6] = rng.uniform(0.001, 0.05, n)
    r[:, 13] = rng.uniform(0.001, 0.05, n)
    return r


def _filter_vv(rng, n):
    r = np.zeros((n, 9))
    d = _detect_vv(rng, n)
    r[:, 0] = np.where(rng.random(n) < 0.1, 0.0, rng.uniform(0, 0.2, n))
    r[:, 1:4], r[:, 4], r[:, 5:8], r[:, 8] = d[:, 0:3], d[:, 3], d[:, 4:7], d[:, 7]
    t = rng.random(n) < 0.05                                         # d exactly ri + rj + rV along x
    r[t, 5:8] = r[t, 1:4]
    r[t, 5] = r[t, 1] + (r[t, 4] + r[t, 8] + r[t, 0])
    return r


def _filter_ve(rng, n):
    r = np.zeros((n, 12))
    d = _detect_ve(rng, n)
    r[:, 0] = np.where(rng.random(n) < 0.1, 0.0, rng.uniform(0, 0.2, n))
    r[:, 1:4], r[:, 4], r[:, 5:8], r[:, 8:11], r[:, 11] = d[:, 0:3], d[:, 3], d[:, 4:7], d[:, 7:10], d[:, 10]
    # the line parameter exactly at -rV or 1 + rV, on an axis-aligned edge
    t = rng.random(n) < 0.05
    rv = r[t, 0]
    r[t, 5:8] = 0.0
    r[t, 8:11] = 0.0
    r[t, 8] = 1.0
    r[t, 1] = np.where(rng.random(t.sum()) < 0.5, -rv, 1.0 + rv)
    r[t, 2] = 0.01
    r[t, 3] = 0.0
    return r


def _filter_ee(rng, n):
    r = np.zeros((n, 15))
    d = _detect_ee(rng, n)
    r[:, 0] = np.where(rng.random(n) < 0.1, 0.0, rng.uniform(0, 0.2, n))
    r[:, 1:7], r[:, 7], r[:, 8:14], r[:, 14] = d[:, 0:6], d[:, 6], d[:, 7:13], d[:, 13]
    return r


def _world_vertex(rng, n):
    r = np.zeros((n, 11))
    r[:, 0:3] = rng.uniform(-100, 100, (n, 3))
    r[:, 3:7] = _quat(rng, n, off_unit=1e-3)
    r[:, 7] = np.where(rng.random(n) < 0.5, 1.0, rng.uniform(0.5, 2.0, n))
    r[:, 8:11] = rng.uniform(-1, 1, (n, 3))
    return r


def _obb_rows(rng, n, scale=1.0):
    q = _quat(rng, n)
    R = _rotmat(q)
    o = np.zeros((n, 15))
    o[:, 0:3] = rng.uniform(-2, 2, (n, 3))
    o[:, 3:6], o[:, 6:9], o[:, 9:12] = R[:, :, 0], R[:, :, 1], R[:, :, 2]
    o[:, 12:15] = rng.uniform(0.05, 1.0, (n, 3)) * scale
    axis = rng.random(n) < 0.1                                       # identity axes, as the vertex gates use
    o[axis, 3:12] = np.array([1, 0, 0, 0, 1, 0, 0, 0, 1], dtype=np.float64)
    return o


def _obb_intersect(rng, n):
    r = np.zeros((n, 30))
    r[:, 0:15] = _obb_rows(rng, n)
    r[:, 15:30] = _obb_rows(rng, n)
    r[:, 15:18] = r[:, 0:3] + _unit(rng, n) * rng.uniform(0, 3, (n, 1))
    return r


def _compute_obb(rng, n):
    r = np.zeros((n, 24))
    r[:, 0:15] = _obb_rows(rng, n)
    r[:, 15:18] = rng.uniform(-50, 50, (n, 3))
    r[:, 18:22] = _quat(rng, n, off_unit=1e-4)
    r[:, 22] = np.where(rng.random(n) < 0.5, 1.0, rng.uniform(0.5, 2.0, n))
    r[:, 23] = np.where(rng.random(n) < 0.2, 0.0, rng.uniform(0, 0.05, n))
    return r


def _push_quaternion(rng, n):
    r = np.zeros((n, 11))
    r[:, 0:4] = _quat(rng, n, off_unit=1e-6)
    r[np.arange(n) < n // 20, 0:4] = np.array([1.0, 0.0, 0.0, 0.0])
    r[:, 4:7] = _maybe_zero(rng, rng.standard_normal((n, 3)) * 10.0 ** rng.uniform(-4, 2, (n, 1)), 0.2)
    r[:, 7:10] = _maybe_zero(rng, rng.standard_normal((n, 3)) * 10.0 ** rng.uniform(-4, 3, (n, 1)), 0.2)
    r[:, 10] = 10.0 ** rng.uniform(-5, -2, n)
    tiny = rng.random(n) < 0.01                                      # norm below 1e-9: reset to identity
    r[tiny, 0:4] = 1e-6 * rng.standard_normal((tiny.sum(), 4))
    r[tiny, 4:7] = 0.0
    return r


def _angular(rng, n):
    r = np.zeros((n, 15))
    r[:, 0:4] = _quat(rng, n, off_unit=1e-6)
    r[:, 4:7] = _maybe_zero(rng, rng.standard_normal((n, 3)) * 10.0 ** rng.uniform(-6, 2, (n, 1)), 0.2)
    r[:, 7:10] = _maybe_zero(rng, rng.standard_normal((n, 3)) * 10.0 ** rng.uniform(-4, 2, (n, 1)), 0.2)
    I = 10.0 ** rng.uniform(-4, 1, (n, 3))
    iso = rng.random(n) < 0.5
    I[iso] = I[iso, :1]
    r[:, 10:13] = I
    r[:, 13] = 10.0 ** rng.uniform(-5, -2, n)
    return r


def _surface(rng, n):
    r = np.zeros((n, 11))
    nrm = _unit(rng, n)
    ax = rng.random(n) < 0.5                                         # axis-aligned walls, as the decks use
    k = rng.integers(0, 3, n)
    nrm[ax] = 0.0
    nrm[ax, k[ax]] = np.where(rng.random(ax.sum()) < 0.5, 1.0, -1.0)
    off = rng.uniform(-20, 20, n)
    r[:, 0] = off
    r[:, 1:4] = nrm
    c = rng.random(n)
    r[:, 4:7] = off[:, None] * nrm                                   # centre on the plane ...
    r[c < 0.3, 4:7] = 0.0                                            # ... defaulted ...
    moved = (c >= 0.3) & (c < 0.5)                                   # ... or moved along the plane
    r[moved, 4:7] += np.cross(nrm[moved], _unit(rng, moved.sum())) * 3.0
    r[:, 7] = rng.uniform(0.05, 1.0, n)
    r[:, 8:11] = off[:, None] * nrm + rng.standard_normal((n, 3)) * 1.5
    return r


def _cylinder(rng, n):
    r = np.zeros((n, 11))
    k = rng.integers(0, 3, n)
    axis = np.ones((n, 3))
    axis[np.arange(n), k] = 0.0                                      # component mask, e.g. (1, 0, 1)
    r[:, 0] = rng.uniform(1, 50, n)
    r[:, 1:4] = axis
    r[:, 4:7] = rng.uniform(-50, 50, (n, 3))
    r[:, 7] = rng.uniform(0.05, 1.0, n)
    proj_c = axis * r[:, 4:7]
    d = _unit(rng, n) * axis
    d /= np.maximum(np.linalg.norm(d, axis=1), 1e-300)[:, None]
    p = proj_c + d * (r[:, 0] - r[:, 7] * rng.uniform(0, 2, n))[:, None]
    p += (1.0 - axis) * rng.uniform(-30, 30, (n, 3))
    r[:, 8:11] = p
    return r


def pair_keys(n: int, seed: int) -> np.ndarray:
    """Rows of two keys (owner id, partner id, type, swap, owner sub, partner sub) with many ties."""
    rng = np.random.default_rng(seed)
    k = np.zeros((n, 12), dtype=np.uint64)
    hi = [4, 4, 13, 2, 5, 5]
    for h in (0, 6):
        for j, m in enumerate(hi):
            k[:, h + j] = rng.integers(0, m, n)
    big = rng.random(n) < 0.1
    k[big, 0] = rng.integers(0, 2 ** 63, big.sum(), dtype=np.uint64)
    eq = rng.random(n) < 0.2
    k[eq, 6:12] = k[eq, 0:6]
    return k


_GEN = {
    "bond_law": _bond_law,
    "contact_force_core": _contact_force_core, "damping": _damping, "detect_vv": _detect_vv,
    "detect_ve": _detect_ve, "detect_ee": _detect_ee, "filter_vv": _filter_vv, "filter_ve": _filter_ve,
    "filter_ee": _filter_ee, "world_vertex": _world_vertex, "obb_intersect": _obb_intersect,
    "compute_obb": _compute_obb, "push_quaternion": _push_quaternion, "angular": _angular,
    "surface": _surface, "cylinder": _cylinder,
}


# --------------------------------------------------------------- vertex-face
def vertex_face_cases(shape: dict, face: int, n: int, seed: int) -> np.ndarray:
    """Rows rV, vi[3], ri, hj, then the world vertices of ``shape`` in a random pose,
    with vi near face ``face`` (inside, on the boundary, above and below)."""
    rng = np.random.default_rng(seed)
    v0 = np.asarray(shape["vertices"], dtype=np.float64)
    nv = len(v0)
    q = _quat(rng, n)
    R = _rotmat(q)
    h = np.where(rng.random(n) < 0.5, 1.0, rng.uniform(0.8, 1.2, n))
    p = rng.uniform(-5, 5, (n, 3))
    world = p[:, None, :] + np.einsum("nij,nvj->nvi", R, h[:, None, None] * v0[None])
    f = shape["faces"][face]
    fv = world[:, f, :]
    w = rng.dirichlet(np.ones(len(f)), n)
    inside = np.einsum("nk,nki->ni", w, fv)
    c = rng.random(n)
    a = fv[:, 0, :]
    b = fv[:, 1 % len(f), :]
    edge_pt = a + rng.uniform(0, 1, (n, 1)) * (b - a)
    base = np.where((c < 0.15)[:, None], edge_pt, inside)
    base = np.where(((c >= 0.15) & (c < 0.25))[:, None], fv[:, 0, :], base)  # at a face vertex
    nrm = np.cross(fv[:, 1, :] - fv[:, 0, :], fv[:, -1, :] - fv[:, 0, :])
    nrm /= np.linalg.norm(nrm, axis=1)[:, None]
    off = rng.uniform(-0.1, 0.1, (n, 1))
    off[rng.random(n) < 0.05] = 0.0
    vi = base + nrm * off + rng.standard_normal((n, 3)) * 0.05 * (rng.random((n, 1)) < 0.5)
    r = np.zeros((n, 6 + 3 * nv))
    r[:, 0] = np.where(rng.random(n) < 0.1, 0.0, rng.uniform(0, 0.1, n))
    r[:, 1:4] = vi
    r[:, 4] = rng.uniform(0.001, 0.05, n)
    r[:, 5] = h
    r[:, 6:] = world.reshape(n, 3 * nv)
    return r


def run_vertex_face_ref(lib, shape_index: int, face: int, nv: int, rows: np.ndarray) -> np.ndarray:
    rows = np.ascontiguousarray(rows, dtype=np.float64)
    out = np.zeros((rows.shape[0], 9))
    lib.ref_unit_vertex_face.argtypes = [C.c_int, C.c_int, C.c_long, PD, PD]
    assert lib.ref_unit_vertex_face(shape_index, face, rows.shape[0], _ptr(rows), _ptr(out)) == 0
    return out


def run_vertex_face_oracle(lib, shape: dict, face: int, rows: np.ndarray) -> np.ndarray:
    rows = np.ascontiguousarray(rows, dtype=np.float64)
    out = np.zeros((rows.shape[0], 9))
    f = np.asarray(shape["faces"][face], dtype=np.int32)
    nv = len(shape["vertices"])
    fn = lib.oracle_unit_vertex_face
    fn.argtypes = [C.POINTER(C.c_int32), C.c_int, C.c_int, C.c_double, C.c_long, PD, PD]
    assert fn(f.ctypes.data_as(C.POINTER(C.c_int32)), len(f), nv, float(shape["radius"]), rows.shape[0],
              _ptr(rows), _ptr(out)) == 0
    return out


FACE_AREA_H = (1.0, 0.8, 1.3)


def face_areas_ref(lib, shape_index: int, nf: int) -> np.ndarray:
    """get_face_area(f, h) of every face for the homotheties FACE_AREA_H (rows)."""
    lib.ref_shape_face_areas.argtypes = [C.c_int, C.c_double, PD]
    out = np.zeros((len(FACE_AREA_H), nf))
    for k, h in enumerate(FACE_AREA_H):
        row = np.zeros(nf)
        assert lib.ref_shape_face_areas(shape_index, h, _ptr(row)) == 0
        out[k] = row
    return out


def face_areas_oracle(lib, shape: dict) -> np.ndarray:
    v = np.ascontiguousarray(shape["vertices"], dtype=np.float64).reshape(-1)
    sizes = np.asarray([len(f) for f in shape["faces"]], dtype=np.int32)
    fv = np.asarray([x for f in shape["faces"] for x in f], dtype=np.int32)
    P32 = C.POINTER(C.c_int32)
    fn = lib.oracle_unit_face_areas
    fn.argtypes = [PD, C.c_int, P32, P32, C.c_int, C.c_double, PD]
    out = np.zeros((len(FACE_AREA_H), len(sizes)))
    for k, h in enumerate(FACE_AREA_H):
        row = np.zeros(len(sizes))
        assert fn(_ptr(v), len(v) // 3, sizes.ctypes.data_as(P32), fv.ctypes.data_as(P32), len(sizes), h,
                  _ptr(row)) == 0
        out[k] = row
    return out


def read_shps_ref(lib, path) -> list[dict]:
    """exaDEM's read_shp over every shape of a file, as dicts of the shapes' arrays."""
    lib.ref_read_shps.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    first, count = C.c_int(), C.c_int()
    assert lib.ref_read_shps(str(path).encode(), C.byref(first), C.byref(count)) == 0, f"cannot open {path}"
    return [_ref_shape(lib, first.value + k) for k in range(count.value)]


def _ref_shape(lib, s: int) -> dict:
    counts = np.zeros(4, dtype=np.int64)
    lib.ref_shape_info.argtypes = [C.c_int, C.POINTER(C.c_int64)]
    lib.ref_shape_info(s, counts.ctypes.data_as(C.POINTER(C.c_int64)))
    nv, ne, nf, nfa = (int(x) for x in counts)
    v = np.zeros((nv, 3))
    e = np.zeros(2 * ne, dtype=np.int32)
    fa = np.zeros(nfa, dtype=np.int32)
    sc = np.zeros(5)
    ob = np.zeros(15)
    name = C.create_string_buffer(64)
    lib.ref_shape_arrays.argtypes = [C.c_int, PD, C.POINTER(C.c_int32), C.POINTER(C.c_int32), PD, PD, C.c_char_p]
    lib.ref_shape_arrays(s, _ptr(v), e.ctypes.data_as(C.POINTER(C.c_int32)), fa.ctypes.data_as(C.POINTER(C.c_int32)),
                         _ptr(sc), _ptr(ob), name)
    faces, k = [], 1
    for _ in range(nf):
        c = int(fa[k])
        faces.append([int(x) for x in fa[k + 1:k + 1 + c]])
        k += c + 1
    return {"index": s, "name": name.value.decode(), "vertices": v, "edges": e.reshape(-1, 2), "faces": faces,
            "radius": sc[0], "volume": sc[1], "i_over_m": tuple(sc[2:5]),
            "obb": {"center": ob[0:3], "e1": ob[3:6], "e2": ob[6:9], "e3": ob[9:12], "extent": ob[12:15]}}
