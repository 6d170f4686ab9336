"""GPU parity tests of the FrictionSolver-level entry points with all of FrictionSolver::solve's inputs
(scisim/ConstrainedMaps/FrictionSolver.h:28): the map's extra relative velocities nrel_extra and
drel_extra (Sobogus::solve adds them to the kinematic relative velocities, Sobogus.cpp:892-904), for
Ball2D (sg_sobogus_solve_2d_ex) and RigidBody3D spheres (sg_sobogus_solve_3d).

Bars: under the GPU's colour order replayed on the oracle, impulses, post-impact velocities,
friction impulses (and torques), residual and iteration count are bit-exact; in the FP32 form the
oracle's residual of the GPU's impulses meets the tolerance; invalid inputs are rejected before any
solve work.
"""
import numpy as np
import pytest

from scisim_gb300 import scenes

pytestmark = pytest.mark.gpu


def ball2d_problem(gpulib, steps=30, seed=7):
    """Contacts of a frictional box drop after `steps` steps, as a FrictionSolver sees them."""
    s = scenes.box_drop_1024(seed=seed, n_side=12)
    ctx = gpulib.Context(dt=s["dt"], gravity=s["gravity"], mu=0.5, CoR=0.3, tol=1e-9, max_iters=500)
    ctx.upload_ball2d(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"])
    ctx.step(steps)
    q0, v0 = ctx.state()
    ctx.step(1)
    c = ctx.last_contacts()
    ctx.close()
    n = c["n"].reshape(-1, 2)
    bases = np.stack([n[:, 0], n[:, 1], -n[:, 1], n[:, 0]], axis=1).reshape(-1)
    # A FrictionSolver sees a static plane as body -1 (Constraint::getSimulatedBodyIndices).
    return s, v0, c["ia"], np.where(c["ib"] >= 0, c["ib"], -1).astype(np.int32), bases


def sphere_problem(gpulib, steps=60):
    """Contacts of a sphere pile after `steps` steps with their arms, as a FrictionSolver sees them."""
    s = scenes.sphere_pile(n=900, seed=7, width=2.0, depth=2.0)
    nb = s["r"].shape[0]
    ctx = gpulib.Context(dt=s["dt"], gravity=s["gravity"], mu=s["mu"], CoR=s["CoR"], tol=1e-10, max_iters=300,
                         integrator=gpulib.SPLIT_HAM)
    ctx.upload_sphere3d(s["q"], s["v"], s["r"], s["m"], s["I0"], s["plane_x"], s["plane_n"])
    ctx.step(steps)
    q0, v0 = ctx.state()
    Iw, Iinv = ctx.sphere3d_world_inertia()
    ctx.step(1)
    c = ctx.sphere3d_last_contacts()
    ctx.close()
    x = q0[: 3 * nb].reshape(-1, 3)
    ia = c["ia"]
    ib = np.where(c["ib"] >= 0, c["ib"], -1).astype(np.int32)  # static planes are body -1 to a FrictionSolver
    E = c["bases"].reshape(-1, 9)
    n = E[:, 0:3]
    arm_a = np.zeros((ia.shape[0], 3))
    arm_b = np.zeros((ia.shape[0], 3))
    for k in range(ia.shape[0]):
        a, b = ia[k], ib[k]
        if b >= 0:
            p = x[a] + s["r"][a] / (s["r"][a] + s["r"][b]) * (x[b] - x[a])
            arm_a[k] = p - x[a]
            arm_b[k] = p - x[b]
        else:
            arm_a[k] = -s["r"][a] * n[k]
    return s, v0, Iw.reshape(-1), Iinv.reshape(-1), ia, ib, E.reshape(-1), arm_a.reshape(-1), arm_b.reshape(-1)


def test_solve_2d_extras_bit_exact(gpulib, oracle):
    s, v0, ia, ib, bases = ball2d_problem(gpulib)
    nc = ia.shape[0]
    assert nc > 50
    rng = np.random.default_rng(3)
    nrel = rng.normal(0.0, 0.05, nc)
    drel = rng.normal(0.0, 0.05, nc)
    alpha0 = np.abs(rng.normal(0.0, 1e-3, nc))
    beta0 = rng.normal(0.0, 1e-4, nc)
    CoR = rng.uniform(0.0, 0.5, nc)
    ctx = gpulib.Context(dt=s["dt"], gravity=s["gravity"], mu=0.5, CoR=0.3, tol=1e-9, max_iters=500)
    g = ctx.sobogus_solve_2d(s["m"], v0, ia, ib, bases, CoR, 0.5, 1e-9, 500, alpha=alpha0, beta=beta0,
                             nrel_extra=nrel, drel_extra=drel)
    order, _ = ctx.last_solve_order()
    o = oracle.sobogus_solve_2d(s["m"], v0, ia, ib, bases, CoR, 0.5, 1e-9, 500, alpha=alpha0, beta=beta0,
                                order=order, nrel_extra=nrel, drel_extra=drel)
    for k in ("alpha", "beta", "v2", "f"):
        assert np.array_equal(g[k], o[k]), k
    assert g["iterations"] == o["iterations"] and g["error"] == o["error"]
    # The extras change the problem: the solution without them differs.
    z = ctx.sobogus_solve_2d(s["m"], v0, ia, ib, bases, CoR, 0.5, 1e-9, 500, alpha=alpha0, beta=beta0)
    assert not np.array_equal(z["v2"], g["v2"])
    # Zero extras through the extended entry equal the plain entry bit for bit.
    zz = ctx.sobogus_solve_2d(s["m"], v0, ia, ib, bases, CoR, 0.5, 1e-9, 500, alpha=alpha0, beta=beta0,
                              nrel_extra=np.zeros(nc), drel_extra=np.zeros(nc))
    for k in ("alpha", "beta", "v2", "f"):
        assert np.array_equal(z[k], zz[k]), k
    ctx.close()


def test_solve_3d_bit_exact_with_extras(gpulib, oracle):
    s, v0, Iw, Iinv, ia, ib, bases, arm_a, arm_b = sphere_problem(gpulib)
    nc = ia.shape[0]
    assert nc > 50 and (ib >= 0).any() and (ib < 0).any()
    rng = np.random.default_rng(5)
    CoR = np.full(nc, s["CoR"])
    ctx = gpulib.Context(dt=s["dt"], gravity=s["gravity"], mu=s["mu"], CoR=s["CoR"], tol=1e-10, max_iters=300,
                         integrator=gpulib.SPLIT_HAM)
    for extras in (False, True):
        nrel = rng.normal(0.0, 0.02, nc) if extras else None
        drel = rng.normal(0.0, 0.02, 2 * nc) if extras else None
        alpha0 = np.abs(rng.normal(0.0, 1e-4, nc))
        beta0 = rng.normal(0.0, 1e-5, 2 * nc)
        g = ctx.sobogus_solve_3d(s["m"], Iw, Iinv, v0, ia, ib, bases, arm_a, arm_b, CoR, s["mu"], 1e-10, 300,
                                 alpha=alpha0, beta=beta0, nrel_extra=nrel, drel_extra=drel)
        order, _ = ctx.last_solve_order()
        o = oracle.sobogus_solve_3d(s["m"], Iinv, Iw, v0, ia, ib, bases, arm_a, arm_b, CoR, s["mu"], 1e-10, 300,
                                    alpha=alpha0, beta=beta0, order=order, nrel_extra=nrel, drel_extra=drel)
        for k in ("alpha", "beta", "v2", "f"):
            assert np.array_equal(g[k], o[k]), (extras, k, np.abs(g[k] - o[k]).max())
        assert g["iterations"] == o["iterations"] and g["error"] == o["error"]
    ctx.close()


def test_solve_3d_fp32_meets_tol(gpulib, oracle):
    s, v0, Iw, Iinv, ia, ib, bases, arm_a, arm_b = sphere_problem(gpulib)
    nc = ia.shape[0]
    rng = np.random.default_rng(6)
    nrel = rng.normal(0.0, 0.02, nc)
    drel = rng.normal(0.0, 0.02, 2 * nc)
    CoR = np.full(nc, s["CoR"])
    ctx = gpulib.Context(dt=s["dt"], gravity=s["gravity"], mu=s["mu"], CoR=s["CoR"], tol=1e-8, max_iters=2000,
                         integrator=gpulib.SPLIT_HAM, precision=gpulib.PRECISION_FP32_REFINE)
    g = ctx.sobogus_solve_3d(s["m"], Iw, Iinv, v0, ia, ib, bases, arm_a, arm_b, CoR, s["mu"], 1e-8, 2000,
                             nrel_extra=nrel, drel_extra=drel)
    ctx.close()
    assert g["succeeded"]
    # The oracle's residual of the GPU's impulses, with the same extras folded into the forcing terms.
    err = oracle.residual_3d(s["m"], Iinv, Iw, v0, ia, ib, bases, arm_a, arm_b, CoR, s["mu"], g["alpha"], g["beta"],
                             nrel_extra=nrel, drel_extra=drel)
    assert err <= 1e-8, err


def test_solve_3d_rejects_invalid_input(gpulib):
    s, v0, Iw, Iinv, ia, ib, bases, arm_a, arm_b = sphere_problem(gpulib, steps=40)
    nc = ia.shape[0]
    ctx = gpulib.Context(dt=s["dt"], gravity=s["gravity"], integrator=gpulib.SPLIT_HAM)
    CoR = np.zeros(nc)
    bad = bases.copy()
    bad[3:6] *= 2.0  # tangent of contact 0 no longer unit length
    with pytest.raises(gpulib.SgError, match="SG_BAD_INPUT"):
        ctx.sobogus_solve_3d(s["m"], Iw, Iinv, v0, ia, ib, bad, arm_a, arm_b, CoR, 0.5, 1e-8, 100)
    arm = arm_a.copy()
    arm[0:3] += bases[3:6] * 1e-3  # arm of contact 0 off the normal's line
    with pytest.raises(gpulib.SgError, match="SG_BAD_INPUT"):
        ctx.sobogus_solve_3d(s["m"], Iw, Iinv, v0, ia, ib, bases, arm, arm_b, CoR, 0.5, 1e-8, 100)
    ia2 = ia.copy()
    ia2[0] = s["r"].shape[0]
    with pytest.raises(gpulib.SgError, match="SG_BAD_INPUT"):
        ctx.sobogus_solve_3d(s["m"], Iw, Iinv, v0, ia2, ib, bases, arm_a, arm_b, CoR, 0.5, 1e-8, 100)
    # No contacts: v2 = v0, no friction impulse.
    g = ctx.sobogus_solve_3d(s["m"], Iw, Iinv, v0, ia[:0], ib[:0], bases[:0], arm_a[:0], arm_b[:0], CoR[:0], 0.5,
                             1e-8, 100)
    assert np.array_equal(g["v2"], v0) and not g["f"].any() and g["succeeded"]
    ctx.close()
