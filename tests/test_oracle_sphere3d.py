"""CPU checks of the RigidBody3D sphere oracle (no GPU).

* sphere mass / inertia: the reference's known answer (rigidbody3dtests/rigidbody3d_inertia_tests.cpp:17-47),
  and the host mirror's formula bit-identical to the oracle's;
* 3D broad phase: grid set == all-pairs set (the criterion of the reference's 2D test,
  ball2dtests/collision_detection_tests.cpp:34-40; the 3D fixture is not in the reference mount);
* frictionless head-on pair: the closed-form impulse of SphereSphereConstraint::resolveImpact
  (rigidbody3d/Constraints/SphereSphereConstraint.cpp:43-70);
* momentum and angular momentum conserved by sphere-sphere contacts
  (GeometricImpactFrictionMap.cpp:396-424 asserts);
* a sphere rolling down an incline: acceleration (5/7) g sin(theta).
"""
import json
import math
import os

import numpy as np
import pytest

from scisim_gb300 import scenes
from scisim_gb300.rigidbody3d import RigidBodySphere

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_sphere_inertia_known_answer(oracle):
    for case in json.load(open(os.path.join(GOLDEN, "sphere_inertia.json"))):
        M, I = oracle.sphere_mass_inertia(case["r"], case["density"])
        assert abs(M - case["M"]) <= case["tol_M"]
        assert abs(I - case["I"]) <= case["tol_I"]
        M2, CM, I2, R = RigidBodySphere(case["r"]).computeMassAndInertia(case["density"])
        assert M2 == M and np.all(I2 == I) and np.all(CM == 0.0) and np.all(R == np.eye(3))
        m3, i3 = scenes.sphere_mass_inertia(np.array([case["r"]]), case["density"])
        assert m3[0] == M and i3[0] == I


@pytest.mark.parametrize("seed,n,spread", [(0, 2000, 10.0), (1, 3000, 4.0), (2, 500, 1.0)])
def test_grid3d_equals_allpairs(oracle, seed, n, spread):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-spread, spread, (n, 3))
    e = rng.uniform(0.01, 0.4, (n, 3))
    boxes = np.concatenate([c - e, c + e], 1)
    boxes[5] = boxes[6]                                   # identical boxes
    boxes[7] = np.concatenate([c[7] - 2.0, c[7] + 2.0])   # one large box
    b9 = boxes[9]
    boxes[8] = [b9[3], b9[1], b9[2], b9[3] + 0.3, b9[4], b9[5]]   # touching faces overlap
    g = oracle.grid_overlaps_3d(boxes)
    a = oracle.allpairs_overlaps_3d(boxes)
    assert g.shape == a.shape and np.array_equal(g, a)
    assert [8, 9] in g.tolist()


def two_spheres(v_a, v_b, w_a=(0, 0, 0), w_b=(0, 0, 0), r=(0.5, 0.3), gap=-1e-3):
    x = np.array([[0.0, 0.0, 0.0], [r[0] + r[1] + gap, 0.0, 0.0]])
    m, i0 = scenes.sphere_mass_inertia(np.array(r))
    q = np.concatenate([x.reshape(-1), np.tile(np.eye(3).reshape(-1), 2)])
    v = np.concatenate([np.array([v_a, v_b], float).reshape(-1), np.array([w_a, w_b], float).reshape(-1)])
    return q, v, np.array(r), m, np.repeat(i0, 3)


def test_head_on_frictionless_closed_form(oracle):
    q, v, r, m, I0 = two_spheres((1.0, 0, 0), (-0.5, 0, 0))
    CoR = 0.4
    sim = oracle.Sphere3D(q, v, r, m, I0, np.zeros((0, 3)), np.zeros((0, 3)), dt=0.01, gravity=(0, 0, 0), mu=0.0,
                          CoR=CoR, tol=1e-14, max_iters=100)
    st = sim.step()
    assert st["n_contacts"] == 1 and st["succeeded"]
    c = sim.last_contacts()
    # n = normalize(x_a - x_b) = -e_x, ndotv = n.(v_a - v_b) = -1.5
    ndotv = -1.5
    alpha = -(1 + CoR) * ndotv * m[0] * m[1] / (m[0] + m[1])
    assert abs(c["alpha"][0] - alpha) <= 1e-12 * alpha
    assert np.all(c["beta"] == 0.0)


def test_momentum_conserved_by_sphere_contacts(oracle):
    s = scenes.sphere_pile(n=400, seed=3, width=2.0, depth=2.0)
    n = s["r"].shape[0]
    # squeeze the lattice so that spheres touch, no gravity, no planes
    q = s["q"].copy()
    x = q[:3 * n].reshape(-1, 3)
    q[:3 * n] = (x * 0.92).reshape(-1)
    v = s["v"].copy()
    v[:3 * n] *= 10.0
    sim = oracle.Sphere3D(q, v, s["r"], s["m"], s["I0"], np.zeros((0, 3)), np.zeros((0, 3)), dt=0.004,
                          gravity=(0, 0, 0), mu=0.6, CoR=0.2, tol=1e-12, max_iters=2000)

    def moments(q, v):
        x, vl, w = q[:3 * n].reshape(-1, 3), v[:3 * n].reshape(-1, 3), v[3 * n:].reshape(-1, 3)
        p = (s["m"][:, None] * vl).sum(0)
        Iw, _ = sim.world_inertia()
        L = (s["m"][:, None] * np.cross(x, vl)).sum(0) + np.einsum("bij,bj->i", Iw.reshape(-1, 3, 3), w)
        return p, L

    p0, L0 = moments(*sim.state())
    st = sim.step()
    assert st["n_sphere_sphere"] > 50 and st["n_sphere_plane"] == 0
    p1, L1 = moments(*sim.state())
    scale_p = np.abs(s["m"][:, None] * v[:3 * n].reshape(-1, 3)).sum()
    assert np.abs(p1 - p0).max() <= 1e-12 * scale_p
    assert np.abs(L1 - L0).max() <= 1e-11 * max(1.0, np.abs(L0).max(), scale_p)


def test_sphere_rolls_down_incline(oracle):
    """No slip on an incline with enough friction: a = 5/7 g sin(theta) along the slope."""
    th = math.radians(20.0)
    r = 0.25
    nrm = np.array([-math.sin(th), math.cos(th), 0.0])
    down = np.array([-math.cos(th), -math.sin(th), 0.0])
    x0 = r * nrm
    m, i0 = scenes.sphere_mass_inertia(np.array([r]))
    q = np.concatenate([x0, np.eye(3).reshape(-1)])
    v = np.zeros(6)
    dt, T, g = 0.001, 0.5, 9.81
    sim = oracle.Sphere3D(q, v, np.array([r]), m, np.repeat(i0, 3), np.zeros((1, 3)), nrm[None, :], dt=dt,
                          gravity=(0.0, -g, 0.0), mu=0.8, CoR=0.0, tol=1e-13, max_iters=500)
    for _ in range(int(round(T / dt))):
        sim.step()
    q1, v1 = sim.state()
    speed = float(v1[:3] @ down)
    a_expected = 5.0 / 7.0 * g * math.sin(th)
    assert abs(speed - a_expected * T) <= 0.02 * a_expected * T
    # rolling without slipping: contact point velocity ~ 0 along the slope
    w = v1[3:]
    vc = v1[:3] + np.cross(w, -r * nrm)
    assert abs(vc @ down) <= 0.02 * a_expected * T
