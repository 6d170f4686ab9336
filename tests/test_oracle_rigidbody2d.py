"""The oracle's restatement of the reference's RigidBody2D circle path (oracle/rigidbody2d_oracle.cpp):
rigid discs with rotation stepped by GeometricImpactFrictionMap and Sobogus(RigidBody2D).

The reference registers only serialization tests for rigidbody2d (rigidbody2dcli/CMakeLists.txt:18-49:
a resumed run equals an uninterrupted one), so the restatement is checked against closed forms and
the invariants the reference asserts: a disc rolls without slipping down an incline at (2/3) g sin
theta when mu >= tan theta / 3 and slides at g (sin theta - mu cos theta) otherwise, its spin then
growing at 2 mu g cos theta / r; a frictionless head-on elastic collision exchanges velocities and
leaves the spins alone; an oblique frictional collision conserves linear and angular momentum
(CircleCircleConstraint::conservesAngularMomentumUnderImpactAndFriction); a resting disc is held
by the impulse m g dt and drifts as the geometric map makes it; and a run restarted from its
state continues identically.
"""
import os

import numpy as np
import pytest

G, R, DT = 9.81, 0.5, 1e-3


def incline(O, mu, theta_deg=20.0, steps=1000, **kw):
    th = np.deg2rad(theta_deg)
    n = np.array([np.sin(th), np.cos(th)])
    d = np.array([np.cos(th), -np.sin(th)])
    m, I = O.circle_mass_inertia([R], 1.0)
    sim = O.RigidBody2D(np.r_[n * R, 0.0], np.zeros(3), [R], m, I, [[0.0, 0.0]], [n], dt=DT, gravity=(0.0, -G),
                        mu=mu, CoR=0.0, tol=1e-12, max_iters=1000, **kw)
    st, tot, bad = sim.run(steps)
    q, v = sim.state()
    return th, n, d, q, v, st, bad


@pytest.mark.parametrize("integrator", [0, 1])
def test_disc_rolls_down_incline(oracle, integrator):
    th, n, d, q, v, st, bad = incline(oracle, 0.5, integrator=integrator)
    T = 1.0
    a = 2.0 / 3.0 * G * np.sin(th)
    assert bad == 0 and st["succeeded"]
    assert abs((q[:2] - n * R) @ d - 0.5 * a * T * T) <= 0.01 * 0.5 * a * T * T
    assert abs(v[:2] @ d - a * T) <= 0.005 * a * T
    assert abs(v[:2] @ d + R * v[2]) <= 0.01 * a * T          # no slip at the contact
    # The geometric map applies gravity in its final map after the impulse: every step ends with
    # the normal velocity -g cos(theta) dt (and the position sinks g cos(theta) dt^2 per step).
    assert abs(v[:2] @ n + G * np.cos(th) * DT) <= 1e-9


def test_disc_slides_down_incline(oracle):
    mu = 0.05
    th, n, d, q, v, st, bad = incline(oracle, mu)
    T = 1.0
    a = G * (np.sin(th) - mu * np.cos(th))
    spin = -2.0 * mu * G * np.cos(th) / R * T
    assert bad == 0
    assert abs((q[:2] - n * R) @ d - 0.5 * a * T * T) <= 0.01 * 0.5 * a * T * T
    assert abs(v[:2] @ d - a * T) <= 0.005 * a * T
    assert abs(v[2] - spin) <= 0.005 * abs(spin)


def test_head_on_elastic_collision_exchanges_velocities(oracle):
    m, I = oracle.circle_mass_inertia([R, R], 1.0)
    q = np.array([-0.5005, 0.0, 0.3, 0.5005, 0.0, -0.2])
    v = np.array([1.0, 0.0, 2.0, -1.0, 0.0, -3.0])
    sim = oracle.RigidBody2D(q, v, [R, R], m, I, np.zeros((0, 2)), np.zeros((0, 2)), dt=DT, gravity=(0.0, 0.0),
                             mu=0.0, CoR=1.0, tol=1e-12, max_iters=100)
    st = sim.step()
    q1, v1 = sim.state()
    assert st["n_contacts"] == 1 and st["succeeded"]
    assert np.allclose(v1[[0, 1, 3, 4]], [-1.0, 0.0, 1.0, 0.0], atol=1e-12)
    assert v1[2] == 2.0 and v1[5] == -3.0


def test_oblique_frictional_collision_conserves_momentum(oracle):
    r = np.array([0.4, 0.6])
    m, I = oracle.circle_mass_inertia(r, 1.3)
    q = np.array([0.0, 0.0, 0.0, 0.999, 0.05, 0.0])
    v = np.array([2.0, 0.7, 1.5, -0.5, -0.4, -2.0])
    sim = oracle.RigidBody2D(q, v, r, m, I, np.zeros((0, 2)), np.zeros((0, 2)), dt=DT, gravity=(0.0, 0.0),
                             mu=0.8, CoR=0.5, tol=1e-13, max_iters=500)

    def momenta(qq, vv):
        x, w = qq.reshape(2, 3), vv.reshape(2, 3)
        p = (m[:, None] * w[:, :2]).sum(0)
        L = (m * (x[:, 0] * w[:, 1] - x[:, 1] * w[:, 0]) + I * w[:, 2]).sum()
        return p, L

    p0, L0 = momenta(q, v)
    st = sim.step()
    q1, v1 = sim.state()
    c = sim.last_contacts()
    assert st["n_contacts"] == 1 and st["succeeded"]
    assert c["alpha"][0] > 0.0 and c["beta"][0] != 0.0       # an impulse with friction was applied
    p1, L1 = momenta(q1, v1)
    assert np.allclose(p1, p0, rtol=0, atol=1e-12 * np.abs(p0).max())
    assert abs(L1 - L0) <= 1e-12 * max(1.0, abs(L0))
    assert np.any(v1[[2, 5]] != v[[2, 5]])                  # friction changed the spins


def test_resting_disc_warm_start(oracle):
    m, I = oracle.circle_mass_inertia([R], 1.0)
    kw = dict(dt=DT, gravity=(0.0, -G), mu=0.5, CoR=0.0, tol=1e-12, max_iters=1000)
    cold = oracle.RigidBody2D([0.0, R, 0.0], np.zeros(3), [R], m, I, [[0.0, 0.0]], [[0.0, 1.0]], **kw)
    warm = oracle.RigidBody2D([0.0, R, 0.0], np.zeros(3), [R], m, I, [[0.0, 0.0]], [[0.0, 1.0]],
                              cache_mode=oracle.CACHE_NORMAL_AND_FRICTION, **kw)
    for _ in range(20):
        sc, sw = cold.step(), warm.step()
    c = warm.last_contacts()
    assert abs(c["alpha"][0] - m[0] * G * DT) <= 1e-12 * m[0] * G * DT   # the impulse holds the disc up
    assert sw["iterations"] <= sc["iterations"] and sw["succeeded"]
    q, v = warm.state()
    # the geometric map's drift: 20 steps of g dt^2, and the final map's gravity kick -g dt
    assert abs(q[1] - (R - 20 * G * DT * DT)) <= 1e-12 and abs(v[1] + G * DT) <= 1e-15
    assert q[0] == 0.0 and v[0] == 0.0 and v[2] == 0.0


def test_split_run_equals_whole_run(oracle):
    rng = np.random.default_rng(3)
    n = 24
    r = rng.uniform(0.1, 0.2, n)
    m, I = oracle.circle_mass_inertia(r, 1.0)
    xy = np.stack([np.tile(np.arange(6) * 0.45 - 1.1, 4), np.repeat(np.arange(4) * 0.45 + 0.25, 6)], 1)
    q = np.concatenate([xy, rng.uniform(-1, 1, (n, 1))], 1).reshape(-1)
    v = np.concatenate([rng.normal(0, 0.5, (n, 2)), rng.normal(0, 1, (n, 1))], 1).reshape(-1)
    planes = dict(plane_x=[[0.0, 0.0], [-1.5, 0.0], [1.5, 0.0]], plane_n=[[0.0, 1.0], [1.0, 0.0], [-1.0, 0.0]])
    kw = dict(dt=0.005, gravity=(0.0, -G), mu=0.4, CoR=0.2, tol=1e-10, max_iters=2000)
    whole = oracle.RigidBody2D(q, v, r, m, I, planes["plane_x"], planes["plane_n"], **kw)
    whole.run(200)
    first = oracle.RigidBody2D(q, v, r, m, I, planes["plane_x"], planes["plane_n"], **kw)
    first.run(100)
    qh, vh = first.state()
    second = oracle.RigidBody2D(qh, vh, r, m, I, planes["plane_x"], planes["plane_n"], **kw)
    second.iteration = 100
    second.run(100)
    qa, va = whole.state()
    qb, vb = second.state()
    assert np.array_equal(qa, qb) and np.array_equal(va, vb)
    assert np.all(qa.reshape(-1, 3)[:, 1] >= 0.0)           # nothing fell through the floor


ASSETS = "/root/reference/assets/rigidbody2d"


def _sim(O, sc):
    integ = O.SYMPLECTIC_EULER if sc["integrator"] == "symplectic_euler" else O.VERLET
    stag = O.STAGGER_STABILIZED if sc["staggering"] == "stabilized" else O.STAGGER_GEOMETRIC
    return O.RigidBody2D(sc["q"], sc["v"], sc["r"], sc["m"], sc["I"], sc["plane_x"], sc["plane_n"], dt=sc["dt"],
                         gravity=sc["gravity"], mu=sc["mu"], CoR=sc["CoR"], tol=sc["tol"], max_iters=sc["max_iters"],
                         eval_every=sc["eval_every"], integrator=integ, cache_mode=sc["cache_mode"], staggering=stag)


@pytest.mark.skipif(not os.path.isdir(ASSETS), reason="reference assets not present")
def test_reference_ball_rolling_down_hill(oracle):
    """The reference's own scene (tests_serialization/ball_rolling_down_hill.xml): "a ball rolling
    down a valley that should come to rest at the bottom of the valley" (the valley's planes meet at
    x = 2)."""
    from scisim_gb300 import scene_io
    sc = scene_io.load_rigidbody2d_scene(os.path.join(ASSETS, "tests_serialization", "ball_rolling_down_hill.xml"))
    sim = _sim(oracle, sc)
    st, tot, bad = sim.run(4000)
    q, v = sim.state()
    assert bad == 0 and tot >= 4000
    assert abs(q[0] - 2.0) <= 1e-3 and abs(v[0]) <= 1e-12 and abs(v[2]) <= 1e-12
    assert abs(v[1] - sc["gravity"][1] * sc["dt"]) <= 1e-12      # at rest but for the final map's kick


@pytest.mark.skipif(not os.path.isdir(ASSETS), reason="reference assets not present")
def test_reference_circle_scenes_step(oracle):
    """Every circle-only rigidbody2d scene of the reference's assets loads and steps 200 times with
    finite states and solves that stay within their iteration caps."""
    import glob

    from scisim_gb300 import scene_io
    ran = 0
    for f in sorted(glob.glob(os.path.join(ASSETS, "**", "*.xml"), recursive=True)):
        try:
            sc = scene_io.load_rigidbody2d_scene(f)
        except scene_io.SceneError:
            continue
        sim = _sim(oracle, sc)
        st, tot, bad = sim.run(200)
        q, v = sim.state()
        assert np.all(np.isfinite(q)) and np.all(np.isfinite(v)), f
        assert st["iterations"] <= sc["max_iters"], f
        ran += 1
    assert ran >= 22


@pytest.mark.skipif(not os.path.isdir(ASSETS), reason="reference assets not present")
def test_reference_drift_safe_ball_on_plane(oracle):
    """tests_serialization/drift_safe_ball_on_plane.xml with its StabilizedImpactFrictionMap: the
    ball falls onto the plane and then stays exactly where it stopped, at rest, above the plane
    (the geometric map would sink it by g dt^2 every step)."""
    from scisim_gb300 import scene_io
    sc = scene_io.load_rigidbody2d_scene(os.path.join(ASSETS, "tests_serialization", "drift_safe_ball_on_plane.xml"))
    assert sc["staggering"] == "stabilized"
    sim = _sim(oracle, sc)
    sim.run(200)
    q_rest, _ = sim.state()
    st, tot, bad = sim.run(1800)
    q, v = sim.state()
    assert bad == 0 and np.array_equal(q, q_rest) and np.all(v == 0.0)
    assert 0.0 <= q[1] - sc["r"][0] <= 0.01
