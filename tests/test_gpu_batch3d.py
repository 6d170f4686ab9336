"""Batched sphere scenes (sg_sphere3d_batch_upload) against the oracle stepping each scene alone.

Bars, per scene and per step, with the oracle replaying the scene's part of the GPU's colour order
from the GPU's state: the same contact count, the same Gauss-Seidel sweep count and convergence,
positions and linear velocities bit-exact, orientations and angular velocities within 1e-13 (as
for single sphere scenes: CUDA's sin/cos and the host's may differ in the last bit).
"""
import numpy as np
import pytest

from scisim_gb300 import scenes

pytestmark = pytest.mark.gpu


def _split(b, q, v, s):
    x = scenes.batch_scene3(b, s, q, v)
    return x["q"], x["v"]


def test_sphere_batch_matches_scenes_alone(gpulib, oracle):
    b = scenes.sphere_batch(n_scenes=6, seed=11, nmin=40, nmax=300)
    S = len(b["mu"])
    kw = dict(dt=b["dt"], gravity=b["gravity"], tol=1e-9, max_iters=300)
    ctx = gpulib.Context(integrator=gpulib.SPLIT_HAM, mu=0.5, CoR=0.0, **kw)
    ctx.upload_sphere3d_batch(b["body_off"], b["q"], b["v"], b["r"], b["m"], b["I0"], b["plane_off"], b["plane_x"],
                              b["plane_n"], b["mu"], b["CoR"])
    sims = []
    for s in range(S):
        x = scenes.batch_scene3(b, s)
        sims.append(oracle.Sphere3D(x["q"], x["v"], x["r"], x["m"], x["I0"], x["plane_x"], x["plane_n"],
                                    mu=x["mu"], CoR=x["CoR"], **kw))
    checked_contacts = 0
    for step in range(40):
        q0, v0 = ctx.state()
        ctx.step(1, first_iteration=step + 1)
        stats = ctx.batch_scene_stats()
        order, _ = ctx.last_solve_order()
        coff = np.concatenate([[0], np.cumsum(stats["n_contacts"])])
        q1, v1 = ctx.state()
        for s in range(S):
            o = sims[s]
            if step > 0:
                o.set_state(*_split(b, q0, v0, s))
            c0, c1 = int(coff[s]), int(coff[s + 1])
            if c1 > c0:
                o.set_next_order(order[(order >= c0) & (order < c1)] - c0)
            ost = o.step()
            assert ost["n_contacts"] == c1 - c0, (step, s)
            checked_contacts += c1 - c0
            if c1 > c0:
                assert stats["iterations"][s] == ost["iterations"], (step, s)
                assert bool(stats["succeeded"][s]) == bool(ost["succeeded"]), (step, s)
            gq, gv = _split(b, q1, v1, s)
            oq, ov = o.state()
            n = int(b["body_off"][s + 1] - b["body_off"][s])
            assert np.array_equal(gq[:3 * n], oq[:3 * n]), ("positions", step, s)
            assert np.array_equal(gv[:3 * n], ov[:3 * n]), ("velocities", step, s)
            assert np.abs(gq[3 * n:] - oq[3 * n:]).max() <= 1e-13, ("orientations", step, s)
            assert np.abs(gv[3 * n:] - ov[3 * n:]).max() <= 1e-13, ("angular velocities", step, s)
    assert checked_contacts > 1000
    ctx.close()


def test_sphere_batch_c5_shape(gpulib):
    """256 scenes of 64-1,024 spheres: every scene that reports convergence meets the tolerance,
    and the per-scene contact counts add up to the step's."""
    b = scenes.sphere_batch(n_scenes=256, seed=4)
    ctx = gpulib.Context(integrator=gpulib.SPLIT_HAM, dt=b["dt"], gravity=b["gravity"], tol=1e-6, max_iters=500)
    ctx.upload_sphere3d_batch(b["body_off"], b["q"], b["v"], b["r"], b["m"], b["I0"], b["plane_off"], b["plane_x"],
                              b["plane_n"], b["mu"], b["CoR"])
    for step in range(30):
        st = ctx.step(1, first_iteration=step + 1)
    stats = ctx.batch_scene_stats()
    assert int(np.sum(stats["n_contacts"])) == st["n_contacts"] > 0
    conv = stats["succeeded"].astype(bool)
    assert conv.sum() > 0
    assert np.all(stats["error"][conv] < 1e-6)
    ctx.close()


def test_sphere_batch_fp32_refine(gpulib, oracle):
    """FP32 sweeps + FP64 refinement, scene by scene: every scene that reports convergence meets the
    tolerance under the oracle's FP64 residual of its own contacts (with the GPU's impulses), the
    reported residual is that residual, and positions stay within 1e-3 of the FP64 batch."""
    b = scenes.sphere_batch(n_scenes=8, seed=13, nmin=60, nmax=500)
    S = len(b["mu"])
    tol = 1e-7
    kw = dict(integrator=gpulib.SPLIT_HAM, dt=b["dt"], gravity=b["gravity"], tol=tol, max_iters=3000)

    def make(**extra):
        ctx = gpulib.Context(**kw, **extra)
        ctx.upload_sphere3d_batch(b["body_off"], b["q"], b["v"], b["r"], b["m"], b["I0"], b["plane_off"],
                                  b["plane_x"], b["plane_n"], b["mu"], b["CoR"])
        return ctx

    f64, f32 = make(), make(precision=gpulib.PRECISION_FP32_REFINE)
    for step in range(40):
        f64.step(1, first_iteration=step + 1)
    for step in range(39):
        f32.step(1, first_iteration=step + 1)
    q0, v0 = f32.state()
    f32.step(1, first_iteration=40)
    stats = f32.batch_scene_stats()
    g = f32.sphere3d_last_contacts()
    order, _ = f32.last_solve_order()
    coff = np.concatenate([[0], np.cumsum(stats["n_contacts"])])
    checked = 0
    for s in range(S):
        c0, c1 = int(coff[s]), int(coff[s + 1])
        if c1 == c0:
            continue
        b0 = int(b["body_off"][s])
        x = scenes.batch_scene3(b, s, q0, v0)
        sim = oracle.Sphere3D(x["q"], x["v"], x["r"], x["m"], x["I0"], x["plane_x"], x["plane_n"], mu=x["mu"],
                              CoR=x["CoR"], dt=b["dt"], gravity=b["gravity"], tol=tol, max_iters=3000)
        sim.set_state(x["q"], x["v"])
        Iw, Iinv = sim.world_inertia()
        sim.set_next_order(order[(order >= c0) & (order < c1)] - c0)
        sim.step()
        c = sim.last_contacts()
        ia = g["ia"][c0:c1] - b0
        ib = np.where(g["ib"][c0:c1] >= 0, g["ib"][c0:c1] - b0, -1).astype(np.int32)
        assert np.array_equal(ia, c["ia"]) and np.array_equal(ib, np.where(c["ib"] >= 0, c["ib"], -1)), s
        res = oracle.residual_3d(x["m"], Iinv, Iw, x["v"], ia.astype(np.int32), ib, g["bases"][c0:c1].reshape(-1),
                                 c["arm_a"].reshape(-1), c["arm_b"].reshape(-1), float(x["CoR"]), float(x["mu"]),
                                 g["alpha"][c0:c1], g["beta"][c0:c1].reshape(-1))
        err = float(stats["error"][s])
        assert abs(res - err) <= 1e-12 + 1e-6 * err, s
        if stats["succeeded"][s]:
            assert res <= tol * 1.001, s
            checked += 1
    assert checked >= 4
    nb = int(b["body_off"][-1])
    qa, _ = f64.state()
    qb, _ = f32.state()
    assert np.abs(qa[:3 * nb] - qb[:3 * nb]).max() <= 1e-3
    prof = f32.profile_read()
    assert prof["contact_sweeps32"] > 0
    f64.close()
    f32.close()
