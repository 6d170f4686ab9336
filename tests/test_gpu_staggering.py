"""SymplecticEulerImpactFrictionMap and StabilizedImpactFrictionMap on the GPU (sg_set_staggering)
against the oracle's restatements, which the reference's 18 registered symplectic-Euler slope tests and
its drift-safe scene pin (tests/test_oracle_golden.py).

Bars: a registered slope scene bit-exact over 2,000 steps; a frictional box drop with the impulse
cache and pose stabilisation bit-exact every step (positions, velocities, impulses, sweeps and
residual) when the oracle replays the GPU's colour order; restitution rejected as in the reference.
The stabilized map: the drift-safe scene bit-exact and at rest, a box drop bit-exact every step.
"""
import json
import os

import numpy as np
import pytest

from scisim_gb300 import scenes

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
CACHE = {"none": 0, "normal": 1, "normal_and_friction": 2}


def test_registered_slope_scene_bitexact(gpulib, oracle):
    sc = [x for x in json.load(open(os.path.join(GOLDEN, "slope_scenes.json")))
          if x["staggering"] == "symplectic_euler" and x["kind"] == "sliding"][0]
    b = sc["ball"]
    kw = dict(dt=sc["dt"], gravity=sc["gravity"], mu=sc["mu"], CoR=sc["CoR"], tol=sc["tol"],
              max_iters=sc["max_iters"], eval_every=sc["eval_every"], cache_mode=CACHE[sc["cache_impulses"]])
    ctx = gpulib.Context(integrator=gpulib.VERLET, **kw)
    ctx.upload_ball2d([b["x"], b["y"]], [b["vx"], b["vy"]], [b["r"]], [b["m"]], sc["plane_x"], sc["plane_n"])
    ctx.set_staggering(gpulib.STAGGER_SYMPLECTIC_EULER, bool(sc["stabilization"]), sc["penetration_threshold"])
    ctx.step(2000)
    ora = oracle.Ball2D([b["x"], b["y"]], [b["vx"], b["vy"]], [b["r"]], [b["m"]], sc["plane_x"], sc["plane_n"],
                        integrator=oracle.VERLET, staggering=oracle.STAGGER_SYMPLECTIC_EULER,
                        stabilize=bool(sc["stabilization"]), penetration_threshold=sc["penetration_threshold"], **kw)
    ora.run(2000)
    gq, gv = ctx.state()
    oq, ov = ora.state()
    assert np.array_equal(gq, oq) and np.array_equal(gv, ov)
    ctx.close()


@pytest.mark.parametrize("stabilize", [False, True])
def test_box_drop_replayed_order_bitexact(gpulib, oracle, stabilize):
    s = scenes.box_drop_1024(seed=4, n_side=14)
    kw = dict(dt=s["dt"], gravity=s["gravity"], mu=0.5, CoR=0.0, tol=1e-9, max_iters=500, cache_mode=2)
    ctx = gpulib.Context(**kw)
    ctx.upload_ball2d(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"])
    ctx.set_staggering(gpulib.STAGGER_SYMPLECTIC_EULER, stabilize, 1e-4)
    ora = oracle.Ball2D(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"],
                        staggering=oracle.STAGGER_SYMPLECTIC_EULER, stabilize=stabilize, penetration_threshold=1e-4,
                        **kw)
    contacts = 0
    for step in range(60):
        st = ctx.step(1)
        order, _ = ctx.last_solve_order()
        if st["n_contacts"]:
            ora.set_next_order(order)
        ost = ora.step()
        assert st["n_contacts"] == ost["n_contacts"], step
        contacts += st["n_contacts"]
        gq, gv = ctx.state()
        oq, ov = ora.state()
        assert np.array_equal(gq, oq) and np.array_equal(gv, ov), step
        if st["n_contacts"]:
            gc, oc = ctx.last_contacts(), ora.last_contacts()
            assert np.array_equal(gc["alpha"], oc["alpha"]) and np.array_equal(gc["beta"], oc["beta"]), step
            assert st["iterations"] == ost["iterations"] and st["error"] == ost["error"], step
    assert contacts > 500
    ctx.close()


def test_restitution_is_rejected(gpulib):
    ctx = gpulib.Context(CoR=0.3)
    with pytest.raises(gpulib.SgError):
        ctx.set_staggering(gpulib.STAGGER_SYMPLECTIC_EULER)
    ctx.close()


def test_stabilized_drift_safe_scene_bitexact(gpulib, oracle):
    kw = dict(dt=0.01, gravity=(0.0, -10.0), mu=0.5, CoR=0.0, tol=1e-12, max_iters=5000, eval_every=1, cache_mode=0)
    ctx = gpulib.Context(integrator=gpulib.VERLET, **kw)
    ctx.upload_ball2d([0.0, 1.0], [0.0, 0.0], [0.5], [8.0], [[0.0, 0.0]], [[0.0, 1.0]])
    ctx.set_staggering(gpulib.STAGGER_STABILIZED)
    ctx.step(450)
    ora = oracle.Ball2D([0.0, 1.0], [0.0, 0.0], [0.5], [8.0], [[0.0, 0.0]], [[0.0, 1.0]], integrator=oracle.VERLET,
                        staggering=oracle.STAGGER_STABILIZED, **kw)
    ora.run(450)
    gq, gv = ctx.state()
    oq, ov = ora.state()
    assert np.array_equal(gq, oq) and np.array_equal(gv, ov) and np.all(gv == 0.0)
    ctx.close()


def test_stabilized_box_drop_replayed_order_bitexact(gpulib, oracle):
    s = scenes.box_drop_1024(seed=4, n_side=14)
    kw = dict(dt=s["dt"], gravity=s["gravity"], mu=0.5, CoR=0.3, tol=1e-9, max_iters=500, cache_mode=0)
    ctx = gpulib.Context(**kw)
    ctx.upload_ball2d(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"])
    ctx.set_staggering(gpulib.STAGGER_STABILIZED)
    ora = oracle.Ball2D(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"],
                        staggering=oracle.STAGGER_STABILIZED, **kw)
    for step in range(60):
        st = ctx.step(1)
        order, _ = ctx.last_solve_order()
        if st["n_contacts"]:
            ora.set_next_order(order)
        ost = ora.step()
        assert st["n_contacts"] == ost["n_contacts"], step
        gq, gv = ctx.state()
        oq, ov = ora.state()
        assert np.array_equal(gq, oq) and np.array_equal(gv, ov), step
    with pytest.raises(gpulib.SgError):
        gpulib.Context(cache_mode=2).set_staggering(gpulib.STAGGER_STABILIZED)
    ctx.close()
