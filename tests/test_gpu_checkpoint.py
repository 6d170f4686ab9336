"""Checkpoint / resume (sg_checkpoint_save / sg_checkpoint_load) against an uninterrupted run.

The reference's serialisation (ball2dcli/ball2d_cli.cpp:199-316, Ball2DSim.cpp:810-822) exists so
that a resumed simulation continues exactly; the bar here is the same: a run resumed from a
checkpoint in a fresh context (created with other settings) gives bit-identical positions,
velocities and impulses to the run that never stopped.  Covered: a frictional Ball2D scene with
the impulse cache (FP64), a dense pile on the two-level FP32 path, and a sphere pile.
"""
import numpy as np
import pytest

from scisim_gb300 import scenes

pytestmark = pytest.mark.gpu


def _resume_matches(gpulib, make_ctx, upload, first, n_before, n_after, last_contacts=True):
    a = make_ctx()
    upload(a)
    a.step(n_before, first_iteration=first)
    ck = a.checkpoint()
    a.step(n_after, first_iteration=first + n_before)
    qa, va = a.state()
    ca = a.last_contacts() if last_contacts else None
    # A fresh context with other settings: the checkpoint brings back the original ones.
    b = gpulib.Context(dt=1e-4, gravity=(0.0, 0.0, 0.0), mu=0.0, CoR=1.0, tol=1e-3, max_iters=3,
                       integrator=a_integrator(gpulib, upload))
    b.restore(ck)
    assert b.checkpoint() == ck, "a restored context must save the same checkpoint"
    b.step(n_after, first_iteration=first + n_before)
    qb, vb = b.state()
    assert np.array_equal(qa, qb) and np.array_equal(va, vb), "resumed state differs"
    if last_contacts:
        cb = b.last_contacts()
        for k in ("ia", "ib", "n", "alpha", "beta"):
            assert np.array_equal(ca[k], cb[k]), k
    a.close()
    b.close()
    return ck


def a_integrator(gpulib, upload):
    return gpulib.SPLIT_HAM if getattr(upload, "spheres", False) else gpulib.SYMPLECTIC_EULER


def test_ball2d_resume_is_bit_identical(gpulib):
    s = scenes.box_drop_1024(seed=7, n_side=16)
    kw = dict(dt=s["dt"], gravity=s["gravity"], mu=0.5, CoR=0.3, tol=1e-9, max_iters=500,
              cache_mode=gpulib.CACHE_NORMAL_AND_FRICTION)

    def upload(ctx):
        ctx.upload_ball2d(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"])

    ck = _resume_matches(gpulib, lambda: gpulib.Context(**kw), upload, 1, 60, 25)
    assert len(ck) > 8 * 4 * s["r"].shape[0]


def test_two_level_pile_resume_is_bit_identical(gpulib):
    s = scenes.dense_pile(n=32768, seed=2, width=20.0, height=15.0)
    kw = dict(dt=s["dt"], gravity=s["gravity"], mu=s["mu"], CoR=s["CoR"], tol=1e-6, max_iters=60,
              cache_mode=gpulib.CACHE_NORMAL_AND_FRICTION, precision=gpulib.PRECISION_FP32_REFINE)

    def make():
        ctx = gpulib.Context(**kw)
        ctx.profile_enable(True)
        return ctx

    def upload(ctx):
        ctx.upload_ball2d(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"])

    a = make()
    upload(a)
    a.step(420, first_iteration=1)
    ck = a.checkpoint()
    a.profile_read(reset=True)
    a.step(3, first_iteration=421)
    assert a.profile_read()["two_level_solves"] == 3
    qa, va = a.state()
    b = gpulib.Context(dt=1e-4, gravity=(0.0, 0.0, 0.0), mu=0.0, CoR=1.0, tol=1e-3, max_iters=3)
    b.restore(ck)
    b.step(3, first_iteration=421)
    qb, vb = b.state()
    assert np.array_equal(qa, qb) and np.array_equal(va, vb), "two-level resume differs"


def test_sphere_resume_is_bit_identical(gpulib):
    s = scenes.sphere_pile(n=600, seed=3, width=1.5, depth=1.5)
    kw = dict(dt=s["dt"], gravity=s["gravity"], mu=s["mu"], CoR=s["CoR"], tol=1e-9, max_iters=300,
              integrator=gpulib.SPLIT_HAM)

    def upload(ctx):
        ctx.upload_sphere3d(s["q"], s["v"], s["r"], s["m"], s["I0"], s["plane_x"], s["plane_n"])

    upload.spheres = True
    a = gpulib.Context(**kw)
    upload(a)
    a.step(40, first_iteration=1)
    ck = a.checkpoint()
    a.step(15, first_iteration=41)
    qa, va = a.state()
    ga = a.sphere3d_last_contacts()
    b = gpulib.Context(dt=1e-4, gravity=(0.0, 0.0, 0.0), mu=0.0, CoR=1.0, tol=1e-3, max_iters=3,
                       integrator=gpulib.SPLIT_HAM)
    b.restore(ck)
    assert b.checkpoint() == ck
    b.step(15, first_iteration=41)
    qb, vb = b.state()
    gb = b.sphere3d_last_contacts()
    assert np.array_equal(qa, qb) and np.array_equal(va, vb), "sphere resume differs"
    assert np.array_equal(ga["bases"], gb["bases"]) and np.array_equal(ga["alpha"], gb["alpha"])


def test_bad_checkpoint_is_rejected(gpulib):
    s = scenes.box_drop_1024(seed=7, n_side=8)
    ctx = gpulib.Context(dt=s["dt"], gravity=s["gravity"], tol=1e-9, max_iters=100)
    ctx.upload_ball2d(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"])
    ck = bytearray(ctx.checkpoint())
    with pytest.raises(gpulib.SgError):
        ctx.restore(bytes(ck[: len(ck) // 2]))  # truncated
    ck[0] ^= 0xFF
    with pytest.raises(gpulib.SgError):
        ctx.restore(bytes(ck))  # wrong magic
    ctx.close()
