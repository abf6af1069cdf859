"""Analytic known-answer tests of the CPU oracle (no GPU).

The reference ships no golden values for this path, so the oracle's
restatement is pinned by physics with closed-form answers:
  * elastic head-on impact (damp_rate = 0): restitution 1 and contact time
    pi * sqrt(m_eff / kn) (linear spring);
  * a sphere sliding on a wall: |f_t| clipped to mu * kn * |dn| (common_kernels.hpp:116-135);
  * torque-free rotation: |q| stays 1, omega stays constant;
  * first_iteration leaves forces (not accelerations) in f, so the first
    prolog uses f as acceleration (main-config.msp:55-65);
  * a cube resting face-down on a floor: 4 vertex-wall contacts, net upward
    force 4 * kn * overlap, no torque.
"""
import math

import numpy as np
import pytest

from exadem_gb300 import make_params
from exadem_gb300 import workloads as W


def oracle(params):
    from oracle.oracle import oracle_system

    return oracle_system(params)


def two_spheres(gap, v, damp=0.0, kn=1e4, m=1.0, r=0.5, dt=1e-5):
    p = make_params((-5, -5, -5), (5, 5, 5), rcut_inc=0.05, dt=dt, gravity=(0, 0, 0),
                    config=dict(kn=kn, kt=0.0, kr=0.0, mu=0.0, damp_rate=damp))
    s = oracle(p)
    x = r + 0.5 * gap
    s.set_particles({"rx": np.array([-x, x]), "ry": np.zeros(2), "rz": np.zeros(2), "vx": np.array([v, -v]),
                     "radius": np.array([r, r]), "mass": np.array([m, m]), "inertiax": np.full(2, 0.4 * m * r * r),
                     "inertiay": np.full(2, 0.4 * m * r * r), "inertiaz": np.full(2, 0.4 * m * r * r)})
    return s


def test_elastic_impact_restitution_and_duration():
    v, kn, m, dt = 0.1, 1e4, 1.0, 1e-5
    s = two_spheres(gap=0.0, v=v, kn=kn, m=m, dt=dt)
    s.first_iteration()
    t_contact = 0
    for k in range(4000):
        s.step(1)
        st = s.simulation_state()
        if st["n_active_interactions"]:
            t_contact += 1
        p = s.particles()
        if p["vx"][0] < 0 and st["n_active_interactions"] == 0 and k > 10:
            break
    p = s.particles()
    e = -p["vx"][0] / v
    assert abs(e - 1.0) < 2e-3
    meff = m * m / (m + m)
    assert abs(t_contact * dt - math.pi * math.sqrt(meff / kn)) < 3 * dt


def test_damped_impact_loses_energy():
    v = 0.1
    s = two_spheres(gap=0.0, v=v, damp=0.3)
    s.first_iteration()
    s.step(4000)
    p = s.particles()
    e = -p["vx"][0] / v
    zeta = 0.3
    e_lin = math.exp(-math.pi * zeta / math.sqrt(1 - zeta * zeta))
    assert 0.0 < e < 1.0
    assert abs(e - e_lin) < 0.15  # the no-tension clamp ends the contact a little early


def test_coulomb_clip_on_wall():
    kn, mu, dn = 1e4, 0.3, 1e-3
    p = make_params((-5, -5, -5), (5, 5, 5), rcut_inc=0.05, dt=1e-3, gravity=(0, 0, 0),
                    config=dict(kn=kn, kt=1e6, kr=0.0, mu=mu, damp_rate=0.0))
    s = oracle(p)
    s.set_particles({"rx": np.zeros(1), "ry": np.zeros(1), "rz": np.array([0.5 - dn]), "vx": np.array([2.0]),
                     "radius": np.array([0.5]), "mass": np.array([1.0])})
    s.register_surface(offset=0.0, normal=(0.0, 0.0, 1.0))
    s.first_iteration()
    f = s.particles()
    assert abs(f["fz"][0] - kn * dn) < 1e-9 * kn * dn
    assert abs(abs(f["fx"][0]) - mu * kn * dn) < 1e-12 * kn
    assert f["fx"][0] < 0  # opposes sliding


def test_torque_free_rotation_keeps_unit_quaternion():
    p = make_params((-5, -5, -5), (5, 5, 5), rcut_inc=0.05, dt=1e-3, gravity=(0, 0, 0))
    s = oracle(p)
    w = np.array([0.3, -1.1, 2.0])
    s.set_particles({"rx": np.zeros(1), "ry": np.zeros(1), "rz": np.zeros(1), "radius": np.array([0.5]),
                     "vrotx": w[:1], "vroty": w[1:2], "vrotz": w[2:]})
    s.first_iteration()
    s.step(500)
    p = s.particles()
    q = np.array([p["qw"][0], p["qx"][0], p["qy"][0], p["qz"][0]])
    assert abs(np.linalg.norm(q) - 1.0) < 1e-14
    np.testing.assert_array_equal([p["vrotx"][0], p["vroty"][0], p["vrotz"][0]], w)
    angle = 2 * math.acos(min(1.0, q[0]))
    assert abs(angle - np.linalg.norm(w) * 0.5) < 2e-3


def test_first_step_uses_force_as_acceleration():
    dt, g, m = 1e-3, -9.81, 3.0
    p = make_params((-5, -5, -5), (5, 5, 5), rcut_inc=0.05, dt=dt, gravity=(0, 0, g))
    s = oracle(p)
    s.set_particles({"rx": np.zeros(1), "ry": np.zeros(1), "rz": np.zeros(1), "radius": np.array([0.5]),
                     "mass": np.array([m])})
    s.first_iteration()
    assert s.particles()["fz"][0] == g * m
    s.step(1)
    vz = s.particles()["vz"][0]
    assert abs(vz - (0.5 * dt * g * m + 0.5 * dt * g)) < 1e-15


def test_cube_resting_on_floor():
    cube = W.shape_cube(1.0, 0.01)
    kn, dn, m = 1e5, 1e-4, 0.02
    p = make_params((-5, -5, -5), (5, 5, 5), rcut_inc=0.05, dt=1e-4, gravity=(0, 0, -9.81),
                    config=dict(kn=kn, kt=8e4, kr=0.0, mu=0.5, damp_rate=0.9))
    s = oracle(p)
    s.set_shapes([cube])
    z = 0.5 + 0.01 - dn
    s.set_particles({"rx": np.zeros(1), "ry": np.zeros(1), "rz": np.array([z]), "radius": np.array([cube["max_rcut"]]),
                     "mass": np.array([m]), "inertiax": np.array([m / 6]), "inertiay": np.array([m / 6]),
                     "inertiaz": np.array([m / 6]), "type": np.zeros(1, np.uint32)})
    s.register_surface(offset=0.0, normal=(0.0, 0.0, 1.0))
    s.first_iteration()
    it = s.interactions()
    assert np.all(it["type"] == 5) and len(it["type"]) == 4
    assert s.simulation_state()["n_active_interactions"] == 4
    f = s.particles()
    assert abs(f["fz"][0] - (-9.81 * m + 4 * kn * dn)) < 1e-9
    assert abs(f["momx"][0]) < 1e-12 and abs(f["momy"][0]) < 1e-12
