"""Autotuner (sg_autotune) and tuning knobs (sg_get_tuning / sg_set_tuning).

Bars: the autotuner leaves the scene exactly as it found it (same checkpoint bytes) and keeps
the fastest of the candidates it timed (a later candidate replaces an earlier one only when 3 %
faster); the step after tuning is the step a fresh context gives
from the same checkpoint with the chosen tuning (bit-identical); candidates that do not apply
(two-level sweeps for spheres, everything in the FP64 form) are reported as NaN.
"""
import numpy as np
import pytest

from scisim_gb300 import scenes

pytestmark = pytest.mark.gpu


def kept(ms):
    """The autotuner's rule: candidates in order (NaN: not applicable), a later one replaces the
    kept one only when 3 % faster."""
    i = None
    for j, x in enumerate(ms):
        if np.isnan(x):
            continue
        if i is None or x < 0.97 * ms[i]:
            i = j
    return i


def test_autotune_dense_pile(gpulib):
    s = scenes.dense_pile(n=32768, seed=2, width=20.0, height=15.0)
    kw = dict(dt=s["dt"], gravity=s["gravity"], mu=s["mu"], CoR=s["CoR"], tol=1e-6, max_iters=80,
              cache_mode=gpulib.CACHE_NORMAL_AND_FRICTION, precision=gpulib.PRECISION_FP32_REFINE)
    ctx = gpulib.Context(**kw)
    ctx.upload_ball2d(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"])
    ctx.step(420, first_iteration=1)
    before = ctx.checkpoint()
    best, ms = ctx.autotune(trial_steps=2, first_iteration=421)
    assert ctx.checkpoint() == before, "the autotuner must restore the state it started from"
    assert np.all(np.isfinite(ms)) and np.all(ms > 0.0)
    i = kept(ms)
    assert best["two_level"] == (1 if i < 3 else 0) and best["check_interval"] == (8, 16, 32)[i % 3]
    assert ctx.tuning() == best
    ctx.step(1, first_iteration=421)
    qa, va = ctx.state()
    other = gpulib.Context(dt=1e-3, gravity=(0.0, 0.0), tol=1e-3, max_iters=3)
    other.restore(before)
    other.set_tuning(**best)
    other.step(1, first_iteration=421)
    qb, vb = other.state()
    assert np.array_equal(qa, qb) and np.array_equal(va, vb)
    ctx.close()
    other.close()


def test_autotune_candidates_that_do_not_apply(gpulib):
    s = scenes.box_drop_1024(seed=7, n_side=8)
    ctx = gpulib.Context(dt=s["dt"], gravity=s["gravity"], tol=1e-9, max_iters=100)
    ctx.upload_ball2d(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"])
    ctx.step(5)
    tuning = ctx.tuning()
    best, ms = ctx.autotune(trial_steps=1, first_iteration=6)
    assert np.isfinite(ms[0]) and np.all(np.isnan(ms[1:])), "FP64 form: one timing, nothing to choose"
    assert best == tuning
    ctx.close()
    sp = scenes.sphere_pile(n=200, seed=3, width=1.0, depth=1.0)
    c3 = gpulib.Context(dt=sp["dt"], gravity=sp["gravity"], mu=sp["mu"], CoR=sp["CoR"], tol=1e-9, max_iters=100,
                        integrator=gpulib.SPLIT_HAM, precision=gpulib.PRECISION_FP32_REFINE)
    c3.upload_sphere3d(sp["q"], sp["v"], sp["r"], sp["m"], sp["I0"], sp["plane_x"], sp["plane_n"])
    c3.step(10)
    best, ms = c3.autotune(trial_steps=1, first_iteration=11)
    assert np.all(np.isfinite(ms[:3])) and np.all(np.isnan(ms[3:])), "spheres: no two-level candidates"
    assert best["check_interval"] == (8, 16, 32)[kept(ms)]
    with pytest.raises(gpulib.SgError):
        c3.set_tuning(check_interval=0)
    c3.close()
