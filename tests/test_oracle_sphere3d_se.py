"""The oracle's SymplecticEulerImpactFrictionMap for spheres (oracle/sphere3d_oracle.cpp, se_step):
the force first, the solve with the extra relative velocities N^T vdelta and D^T vdelta,
exponential-Euler configuration updates, and the 3D impulse cache whose cached forces are turned
from the cached normal onto the new one (SymplecticEulerImpactFrictionMap.cpp:48-199, 201-407).

The reference registers its 3D symplectic-Euler scenes as serialization tests only
(rigidbody3dcli/CMakeLists.txt:39-43), so the restatement is checked by what those scenes are
built to show and by closed forms: a sphere dropped on a plane comes to rest on it and stays
there without sinking (unlike the geometric map's drift); stacks of spheres between planes
settle and stay; a sphere rolls down an incline at (5/7) g sin theta; the warm start from the
transported cache converges at once on a resting contact.
"""
import os

import numpy as np
import pytest

ASSETS = "/root/reference/assets/rigidbody3d/tests_symplectic_euler"


def _sim(O, sc, **over):
    kw = dict(dt=sc["dt"], gravity=sc["gravity"], mu=sc["mu"], CoR=sc["CoR"], tol=sc["tol"],
              max_iters=sc["max_iters"], eval_every=sc["eval_every"], staggering=O.STAGGER_SYMPLECTIC_EULER,
              cache_mode=sc["cache_mode"], stabilize=sc["stabilization"],
              penetration_threshold=sc["penetration_threshold"])
    kw.update(over)
    return O.Sphere3D(sc["q"], sc["v"], sc["r"], sc["m"], sc["I0"], sc["plane_x"], sc["plane_n"], **kw)


@pytest.mark.skipif(not os.path.isdir(ASSETS), reason="reference assets not present")
def test_reference_sphere_falling_on_plane(oracle):
    from scisim_gb300 import scene_io
    sc = scene_io.load_rigidbody3d_scene(os.path.join(ASSETS, "sphere_falling_on_plane.xml"))
    assert sc["staggering"] == "symplectic_euler" and sc["integrator"] == "dmv"
    sim = _sim(oracle, sc)
    st, tot, bad = sim.run(1000)
    q_rest, _ = sim.state()
    st, tot, bad = sim.run(500)
    q, v = sim.state()
    r = sc["r"][0]
    assert bad == 0 and st["iterations"] == 1                 # the transported cache starts at the answer
    assert r <= q[1] <= r + 1e-3 and np.abs(v).max() <= 1e-12
    assert np.abs(q - q_rest).max() <= 1e-12                  # no drift into the plane


@pytest.mark.skipif(not os.path.isdir(ASSETS), reason="reference assets not present")
@pytest.mark.parametrize("name", ["spheres_in_planes_0.xml", "spheres_in_planes_1.xml"])
def test_reference_spheres_in_planes_settle(oracle, name):
    from scisim_gb300 import scene_io
    sc = scene_io.load_rigidbody3d_scene(os.path.join(ASSETS, name))
    sim = _sim(oracle, sc)
    sim.run(1000)
    q_rest, _ = sim.state()
    st, tot, bad = sim.run(500)
    q, v = sim.state()
    assert bad == 0 and np.abs(v).max() <= 1e-12 and np.abs(q - q_rest).max() <= 1e-12
    n = sc["r"].shape[0]
    x = q[:3 * n].reshape(n, 3)
    # no sphere sinks into a plane (the penetration of the first impacts stays: these scenes do
    # not stabilise, and the map never pushes an overlap back out)
    for pl in range(sc["plane_x"].shape[0]):
        d = (x - sc["plane_x"][pl]) @ sc["plane_n"][pl] / np.linalg.norm(sc["plane_n"][pl])
        assert np.all(d >= sc["r"] - 1e-3)


def test_sphere_rolls_down_incline(oracle):
    th = np.deg2rad(20.0)
    g, r, dt, T = 9.81, 0.5, 1e-3, 1.0
    n = np.array([np.sin(th), np.cos(th), 0.0])
    d = np.array([np.cos(th), -np.sin(th), 0.0])
    m, I0 = oracle.sphere_mass_inertia(r, 1.0)
    q = np.concatenate([n * r, np.eye(3).reshape(-1)])
    sim = oracle.Sphere3D(q, np.zeros(6), [r], [m], [I0] * 3, [[0.0, 0.0, 0.0]], [n], dt=dt, gravity=(0.0, -g, 0.0),
                          mu=0.5, CoR=0.0, tol=1e-12, max_iters=1000, staggering=oracle.STAGGER_SYMPLECTIC_EULER,
                          cache_mode=oracle.CACHE_NORMAL_AND_FRICTION)
    st, tot, bad = sim.run(int(T / dt))
    q1, v1 = sim.state()
    a = 5.0 / 7.0 * g * np.sin(th)
    assert bad == 0
    assert abs((q1[:3] - n * r) @ d - 0.5 * a * T * T) <= 0.01 * 0.5 * a * T * T
    assert abs(v1[:3] @ d - a * T) <= 0.005 * a * T
    assert abs(v1[:3] @ n) <= 1e-9                            # no drift off or into the incline
    # no slip: v + omega x (-r n) has no component along the slope
    slip = v1[:3] + np.cross(v1[3:], -r * n)
    assert abs(slip @ d) <= 0.01 * a * T


def test_geometric_map_drifts_symplectic_euler_does_not(oracle):
    r, dt, g = 0.5, 1e-3, 9.81
    m, I0 = oracle.sphere_mass_inertia(r, 1.0)
    q = np.concatenate([[0.0, r, 0.0], np.eye(3).reshape(-1)])
    out = {}
    for stag in (oracle.STAGGER_GEOMETRIC, oracle.STAGGER_SYMPLECTIC_EULER):
        sim = oracle.Sphere3D(q, np.zeros(6), [r], [m], [I0] * 3, [[0.0, 0.0, 0.0]], [[0.0, 1.0, 0.0]], dt=dt,
                              gravity=(0.0, -g, 0.0), mu=0.5, CoR=0.0, tol=1e-12, max_iters=100, staggering=stag)
        sim.run(100)
        out[stag] = sim.state()[0][1]
    # the geometric map (SplitHam's half kicks) sinks g dt^2 / 2 a step; symplectic Euler not at all
    assert out[oracle.STAGGER_GEOMETRIC] < r - 40 * g * dt * dt
    assert abs(out[oracle.STAGGER_SYMPLECTIC_EULER] - r) <= 1e-12
