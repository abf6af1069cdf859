"""CPU tests of the seeded input generator: determinism and no initial overlap
(including across periodic boundaries)."""
import numpy as np

from exadem_gb300 import workloads as W


def _min_gap(w, per):
    from scipy.spatial import cKDTree

    P = np.stack([w.particles["rx"], w.particles["ry"], w.particles["rz"]], 1)
    hi = np.array(w.params.bounds_hi[:])
    box = np.where(per, hi, 1e12) if any(per) else None
    t = cKDTree(P, boxsize=box)
    pairs = t.query_pairs(2 * float(w.particles["radius"].max()) + 0.01, output_type="ndarray")
    d = P[pairs[:, 0]] - P[pairs[:, 1]]
    for k in range(3):
        if per[k]:
            d[:, k] -= hi[k] * np.round(d[:, k] / hi[k])
    r = w.particles["radius"]
    return float((np.sqrt((d ** 2).sum(1)) - r[pairs[:, 0]] - r[pairs[:, 1]]).min())


def test_box_deterministic_and_disjoint(native_lib):
    a, b = W.spheres_box(n=2000, box=20.0, seed=7), W.spheres_box(n=2000, box=20.0, seed=7)
    for k in ("rx", "ry", "rz", "vx", "radius", "mass"):
        np.testing.assert_array_equal(a.particles[k], b.particles[k])
    assert _min_gap(a, (0, 0, 0)) >= 0.0
    p = a.particles
    assert p["rx"].min() >= 0.5 and p["rx"].max() <= 19.5
    np.testing.assert_allclose(p["mass"], 2500 * 4.0 / 3.0 * np.pi * 0.125)
    np.testing.assert_allclose(p["inertiax"], 0.4 * p["mass"] * 0.25)


def test_periodic_floor_disjoint_across_boundary(native_lib):
    w = W.spheres_floor(n=20_000, side=30.0)
    assert _min_gap(w, (1, 1, 0)) >= 0.0
    assert w.info["phi_achieved"] > 0.2
    assert w.particles["rz"].min() >= 0.4


def test_drum_inside_cylinder(native_lib):
    w = W.spheres_drum(n=3000)
    c = w.cylinders[0]
    R = c["radius"]
    cx, cz = c["center"][0], c["center"][2]
    p = w.particles
    dist = np.sqrt((p["rx"] - cx) ** 2 + (p["rz"] - cz) ** 2) + p["radius"]
    assert dist.max() <= R
    assert _min_gap(w, (0, 1, 0)) >= 0.0
