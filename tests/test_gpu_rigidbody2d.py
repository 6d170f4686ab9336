"""GPU parity tests for RigidBody2D circles (sg_rigidbody2d_upload): libscisim_gb300.so against the CPU
oracle's restatement of the reference's circle path (oracle/rigidbody2d_oracle.cpp).

Bars:
* every step of a frictional pile of spinning circles, geometric map with symplectic Euler and with
  Verlet, impulse cache on: the contact set (ia, ib), normals, the tangent rows' angular entries,
  the impulses, sweeps, residual, positions, angles and velocities bit-exact with the oracle stepping
  the same state under the GPU's colour order;
* the stabilized map (no cache) the same way;
* a disc rolling down a 20 degree incline at (2/3) g sin(theta) within 1 %, without slip, as the
  oracle does; the reference's own circle scenes (a fixture made from its assets) step on the GPU
  bit for bit as on the oracle.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

G = 9.81


def pile(seed=3, n=144):
    rng = np.random.default_rng(seed)
    side = int(np.sqrt(n))
    r = rng.uniform(0.1, 0.2, n)
    xy = np.stack([np.tile(np.arange(side) * 0.45 - 0.45 * (side - 1) / 2, side),
                   np.repeat(np.arange(side) * 0.45 + 0.25, side)], 1)
    xy += rng.uniform(-0.02, 0.02, xy.shape)
    q = np.concatenate([xy, rng.uniform(-1, 1, (n, 1))], 1).reshape(-1)
    v = np.concatenate([rng.normal(0, 0.5, (n, 2)), rng.normal(0, 2, (n, 1))], 1).reshape(-1)
    half = 0.45 * side / 2 + 0.3
    planes = dict(plane_x=[[0.0, 0.0], [-half, 0.0], [half, 0.0]], plane_n=[[0.0, 1.0], [1.0, 0.0], [-1.0, 0.0]])
    return q, v, r, planes


def run_pair(gpulib, oracle, steps, integrator, cache, staggering, CoR, mu=0.4, seed=3):
    q, v, r, pl = pile(seed)
    m, I = oracle.circle_mass_inertia(r, 1.0)
    kw = dict(dt=0.005, gravity=(0.0, -G), mu=mu, CoR=CoR, tol=1e-10, max_iters=2000, eval_every=1,
              integrator=integrator, cache_mode=cache)
    ctx = gpulib.Context(**kw)
    ctx.upload_rigidbody2d(q, v, r, m, I, pl["plane_x"], pl["plane_n"])
    if staggering != gpulib.STAGGER_GEOMETRIC:
        ctx.set_staggering(staggering)
    sim = oracle.RigidBody2D(q, v, r, m, I, pl["plane_x"], pl["plane_n"], staggering=staggering, **kw)
    seen = 0
    for it in range(1, steps + 1):
        st = ctx.step(1, first_iteration=it)
        if st["n_contacts"] > 0:
            order, _ = ctx.last_solve_order()
            sim.set_next_order(order)
            seen += 1
        so = sim.step()
        assert st["n_contacts"] == so["n_contacts"], it
        g = ctx.rigidbody2d_last_contacts()
        c = sim.last_contacts()
        for k in ("ia", "ib", "n", "ta", "tb", "alpha", "beta"):
            assert np.array_equal(g[k], c[k]), (it, k)
        assert st["iterations"] == so["iterations"] and st["error"] == so["error"], it
        gq, gv = ctx.state()
        oq, ov = sim.state()
        assert np.array_equal(gq, oq) and np.array_equal(gv, ov), it
    ctx.close()
    return seen


def test_rigidbody2d_geometric_symplectic_euler_bit_exact(gpulib, oracle):
    seen = run_pair(gpulib, oracle, 120, gpulib.SYMPLECTIC_EULER, gpulib.CACHE_NORMAL_AND_FRICTION,
                    gpulib.STAGGER_GEOMETRIC, 0.2)
    assert seen > 60


def test_rigidbody2d_geometric_verlet_bit_exact(gpulib, oracle):
    seen = run_pair(gpulib, oracle, 80, gpulib.VERLET, gpulib.CACHE_NORMAL_AND_FRICTION, gpulib.STAGGER_GEOMETRIC,
                    0.3, mu=0.8, seed=5)
    assert seen > 30


def test_rigidbody2d_stabilized_bit_exact(gpulib, oracle):
    seen = run_pair(gpulib, oracle, 80, gpulib.SYMPLECTIC_EULER, gpulib.CACHE_NONE, gpulib.STAGGER_STABILIZED, 0.0)
    assert seen > 30


def test_rigidbody2d_disc_rolls_down_incline(gpulib, oracle):
    R, DT = 0.5, 1e-3
    th = np.deg2rad(20.0)
    n = np.array([np.sin(th), np.cos(th)])
    d = np.array([np.cos(th), -np.sin(th)])
    m, I = oracle.circle_mass_inertia([R], 1.0)
    ctx = gpulib.Context(dt=DT, gravity=(0.0, -G), mu=0.5, CoR=0.0, tol=1e-12, max_iters=1000)
    ctx.upload_rigidbody2d(np.r_[n * R, 0.0], np.zeros(3), [R], m, I, [[0.0, 0.0]], [n])
    st = ctx.step(1000)
    q, v = ctx.state()
    ctx.close()
    a = 2.0 / 3.0 * G * np.sin(th)
    assert st["status"] == gpulib.SG_OK
    assert abs((q[:2] - n * R) @ d - 0.5 * a) <= 0.01 * 0.5 * a
    assert abs(v[:2] @ d - a) <= 0.005 * a
    assert abs(v[:2] @ d + R * v[2]) <= 0.01 * a          # no slip at the contact


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "rigidbody2d_scenes.json")


def test_rigidbody2d_reference_scenes(gpulib, oracle):
    """The reference's 22 circle scenes (assets/rigidbody2d, read by scene_io into
    tests/golden/rigidbody2d_scenes.json) stepped 200 times on the GPU and on the oracle under the
    GPU's colour order: the same states bit for bit."""
    import json
    scenes_ = json.load(open(GOLDEN))
    assert len(scenes_) >= 22
    for sc in scenes_:
        integ = gpulib.SYMPLECTIC_EULER if sc["integrator"] == "symplectic_euler" else gpulib.VERLET
        stag = gpulib.STAGGER_STABILIZED if sc["staggering"] == "stabilized" else gpulib.STAGGER_GEOMETRIC
        kw = dict(dt=sc["dt"], gravity=tuple(sc["gravity"]), mu=sc["mu"], CoR=sc["CoR"], tol=sc["tol"],
                  max_iters=sc["max_iters"], eval_every=sc["eval_every"], integrator=integ,
                  cache_mode=sc["cache_mode"])
        arr = {k: np.asarray(sc[k], np.float64) for k in ("q", "v", "r", "m", "I", "plane_x", "plane_n")}
        ctx = gpulib.Context(**kw)
        ctx.upload_rigidbody2d(arr["q"], arr["v"], arr["r"], arr["m"], arr["I"], arr["plane_x"], arr["plane_n"])
        if stag != gpulib.STAGGER_GEOMETRIC:
            ctx.set_staggering(stag)
        sim = oracle.RigidBody2D(arr["q"], arr["v"], arr["r"], arr["m"], arr["I"], arr["plane_x"], arr["plane_n"],
                                 staggering=stag, **kw)
        for it in range(1, 201):
            st = ctx.step(1, first_iteration=it)
            if st["n_contacts"] > 0:
                sim.set_next_order(ctx.last_solve_order()[0])
            sim.step()
        gq, gv = ctx.state()
        oq, ov = sim.state()
        ctx.close()
        assert np.array_equal(gq, oq) and np.array_equal(gv, ov), sc["xml"]
