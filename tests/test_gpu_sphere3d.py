"""GPU parity tests for RigidBody3D spheres: libscisim_gb300.so (C ABI) against the CPU oracle.

Bars:
* contact sets (ia, ib), bases, forcing, Delassus blocks, Gauss-Seidel iterates under the
  GPU's colour order replayed on the oracle, impulses, positions and linear velocities:
  bit-exact, given the same state;
* orientations and angular velocities: within 1e-13 (CUDA's sin/cos and the host's may
  differ in the last bit);
* the rolling-sphere analytic check: within 2 % of (5/7) g sin(theta), as on the oracle.
"""
import math

import numpy as np
import pytest

from scisim_gb300 import scenes

pytestmark = pytest.mark.gpu


def make_scene(n=1200, seed=7, width=2.0, depth=2.0):
    return scenes.sphere_pile(n=n, seed=seed, width=width, depth=depth)


def gpu_ctx(gpulib, s, **kw):
    cfg = dict(dt=s["dt"], gravity=s["gravity"], mu=s["mu"], CoR=s["CoR"], tol=1e-10, max_iters=400,
               integrator=gpulib.SPLIT_HAM)
    cfg.update(kw)
    ctx = gpulib.Context(**cfg)
    ctx.upload_sphere3d(s["q"], s["v"], s["r"], s["m"], s["I0"], s["plane_x"], s["plane_n"])
    return ctx


def oracle_sim(oracle, s, q=None, v=None, **kw):
    cfg = dict(dt=s["dt"], gravity=s["gravity"], mu=s["mu"], CoR=s["CoR"], tol=1e-10, max_iters=400)
    cfg.update(kw)
    return oracle.Sphere3D(s["q"] if q is None else q, s["v"] if v is None else v, s["r"], s["m"], s["I0"],
                           s["plane_x"], s["plane_n"], **cfg)


def split(x, nb, dim):
    return x[: 3 * nb], x[3 * nb:]


def compare_step(ctx, sim, nb):
    """Steps both from the GPU's current state, replaying the GPU's colour order on the oracle."""
    q0, v0 = ctx.state()
    st = ctx.step(1)
    order, _ = ctx.last_solve_order()
    g = ctx.sphere3d_last_contacts()
    q1, v1 = ctx.state()
    sim.set_state(q0, v0)
    if st["n_contacts"] > 0:
        sim.set_next_order(order)
    so = sim.step()
    c = sim.last_contacts()
    assert st["n_contacts"] == so["n_contacts"]
    assert np.array_equal(g["ia"], c["ia"]) and np.array_equal(g["ib"], c["ib"])
    assert np.array_equal(g["bases"], c["bases"])
    assert st["iterations"] == so["iterations"]
    assert np.array_equal(g["alpha"], c["alpha"]) and np.array_equal(g["beta"], c["beta"])
    qo, vo = sim.state()
    assert np.array_equal(q1[: 3 * nb], qo[: 3 * nb])        # positions
    assert np.array_equal(v1[: 3 * nb], vo[: 3 * nb])        # linear velocities
    assert np.abs(q1[3 * nb:] - qo[3 * nb:]).max() <= 1e-13  # orientations
    w_scale = max(1.0, np.abs(vo[3 * nb:]).max())
    assert np.abs(v1[3 * nb:] - vo[3 * nb:]).max() <= 1e-13 * w_scale
    return st


def test_sphere3d_steps_match_oracle(gpulib, oracle):
    s = make_scene()
    nb = s["r"].shape[0]
    ctx = gpu_ctx(gpulib, s)
    sim = oracle_sim(oracle, s)
    # let the pile fall for a while (fast, no comparison), then compare step by step
    ctx.step(60)
    seen = 0
    for _ in range(12):
        st = compare_step(ctx, sim, nb)
        seen += st["n_contacts"]
    assert seen > 12 * 200


def test_sphere3d_frictionless_and_restitution(gpulib, oracle):
    s = make_scene(n=600, seed=11)
    nb = s["r"].shape[0]
    ctx = gpu_ctx(gpulib, s, mu=0.0, CoR=0.7)
    sim = oracle_sim(oracle, s, mu=0.0, CoR=0.7)
    ctx.step(80)
    for _ in range(6):
        compare_step(ctx, sim, nb)


def test_sphere3d_free_flight(gpulib, oracle):
    # one layer of 8 x 8 spheres on a 0.5 lattice (gaps >= 0.3), far above the floor: no contacts
    s = scenes.sphere_pile(n=64, seed=2, width=4.0, depth=4.0, spacing=0.5)
    q = s["q"].copy()
    nb = s["r"].shape[0]
    q[1: 3 * nb: 3] += 5.0
    s2 = dict(s, q=q, plane_x=s["plane_x"][:1], plane_n=s["plane_n"][:1])  # floor only
    ctx = gpu_ctx(gpulib, s2)
    sim = oracle_sim(oracle, s2)
    for _ in range(5):
        st = compare_step(ctx, sim, nb)
        assert st["n_contacts"] == 0


def test_sphere3d_world_inertia(gpulib, oracle):
    s = make_scene(n=300, seed=4)
    ctx = gpu_ctx(gpulib, s)
    sim = oracle_sim(oracle, s)
    Iw, Iinv = ctx.sphere3d_world_inertia()
    Ow, Oinv = sim.world_inertia()
    assert np.array_equal(Iw, Ow) and np.array_equal(Iinv, Oinv)  # construction form
    ctx.step(20)
    q, v = ctx.state()
    sim.set_state(q, v)
    Iw, Iinv = ctx.sphere3d_world_inertia()
    Ow, Oinv = sim.world_inertia()
    assert np.array_equal(Iw, Ow) and np.array_equal(Iinv, Oinv)  # updateMandMinv form


def test_sphere3d_residual_is_oracle_residual(gpulib, oracle):
    s = make_scene(n=800, seed=5)
    nb = s["r"].shape[0]
    ctx = gpu_ctx(gpulib, s, tol=1e-9, max_iters=3000)
    ctx.step(70)
    q0, v0 = ctx.state()
    st = ctx.step(1)
    g = ctx.sphere3d_last_contacts()
    sim = oracle_sim(oracle, s, q=q0, v=v0, tol=1e-9, max_iters=3000)
    sim.set_state(q0, v0)
    Iw, Iinv = sim.world_inertia()
    # arms from the oracle's active set on the same state (contact point at q0)
    sim.set_next_order(ctx.last_solve_order()[0])
    sim.step()
    c = sim.last_contacts()
    ib = np.where(g["ib"] >= 0, g["ib"], -1)
    res = oracle.residual_3d(s["m"], Iinv, Iw, v0, g["ia"], ib, g["bases"].reshape(-1), c["arm_a"].reshape(-1),
                             c["arm_b"].reshape(-1), s["CoR"], s["mu"], g["alpha"], g["beta"].reshape(-1))
    assert st["error"] <= 1e-9 or not st["succeeded"]
    assert abs(res - st["error"]) <= 1e-12 + 1e-6 * st["error"]


def test_sphere3d_flow_equals_step(gpulib):
    s = make_scene(n=500, seed=8)
    a = gpu_ctx(gpulib, s)
    b = gpu_ctx(gpulib, s)
    a.step(30)
    q, v = s["q"], s["v"]
    for it in range(1, 31):
        q, v, _ = b.flow(it, q, v)
    qa, va = a.state()
    assert np.array_equal(qa, q) and np.array_equal(va, v)


def test_sphere3d_deterministic(gpulib):
    s = make_scene(n=900, seed=9)
    a = gpu_ctx(gpulib, s)
    b = gpu_ctx(gpulib, s)
    a.step(50)
    b.step(50)
    qa, va = a.state()
    qb, vb = b.state()
    assert np.array_equal(qa, qb) and np.array_equal(va, vb)


def test_sphere3d_rolls_down_incline(gpulib):
    th = math.radians(20.0)
    r = 0.25
    nrm = np.array([-math.sin(th), math.cos(th), 0.0])
    down = np.array([-math.cos(th), -math.sin(th), 0.0])
    m, i0 = scenes.sphere_mass_inertia(np.array([r]))
    s = dict(q=np.concatenate([r * nrm, np.eye(3).reshape(-1)]), v=np.zeros(6), r=np.array([r]), m=m,
             I0=np.repeat(i0, 3), plane_x=np.zeros((1, 3)), plane_n=nrm[None, :], dt=0.001,
             gravity=(0.0, -9.81, 0.0), mu=0.8, CoR=0.0)
    ctx = gpu_ctx(gpulib, s, tol=1e-13, max_iters=500)
    T = 0.5
    ctx.step(int(round(T / s["dt"])))
    q1, v1 = ctx.state()
    a = 5.0 / 7.0 * 9.81 * math.sin(th)
    assert abs(float(v1[:3] @ down) - a * T) <= 0.02 * a * T


def test_sphere3d_bad_inputs(gpulib):
    s = make_scene(n=64, seed=1)
    ctx = gpulib.Context(dt=0.004, gravity=(0, -9.81, 0), integrator=gpulib.SYMPLECTIC_EULER)
    ctx.upload_sphere3d(s["q"], s["v"], s["r"], s["m"], s["I0"], s["plane_x"], s["plane_n"])
    with pytest.raises(gpulib.SgError):
        ctx.step(1)  # sphere scenes step with SPLIT_HAM
    ctx2 = gpulib.Context(integrator=gpulib.SPLIT_HAM)
    bad_r = s["r"].copy()
    bad_r[3] = -1.0
    with pytest.raises(gpulib.SgError):
        ctx2.upload_sphere3d(s["q"], s["v"], bad_r, s["m"], s["I0"], s["plane_x"], s["plane_n"])
    with pytest.raises(gpulib.SgError):
        ctx2.upload_sphere3d(s["q"], s["v"], s["r"], s["m"], s["I0"], s["plane_x"], np.zeros((5, 3)))
    assert gpulib.lib().sg_last_contacts(ctx.handle, 0, None, None, None, None, None) == -(2 ** 63)


def test_sphere3d_fp32_refine(gpulib, oracle):
    """FP32 sweeps + FP64 checks and refinement for spheres: a converged step meets the
    tolerance under the oracle's FP64 residual of the GPU's impulses, and positions stay within
    1e-3 of the FP64 solve after 60 steps."""
    s = make_scene(n=900, seed=12)
    f64 = gpu_ctx(gpulib, s, tol=1e-7, max_iters=3000)
    f32 = gpu_ctx(gpulib, s, tol=1e-7, max_iters=3000, precision=gpulib.PRECISION_FP32_REFINE)
    f64.step(60)
    f32.step(59)
    q0, v0 = f32.state()
    st = f32.step(1)
    g = f32.sphere3d_last_contacts()
    sim = oracle_sim(oracle, s, q=q0, v=v0, tol=1e-7, max_iters=3000)
    sim.set_state(q0, v0)
    Iw, Iinv = sim.world_inertia()
    sim.set_next_order(f32.last_solve_order()[0])
    sim.step()
    c = sim.last_contacts()
    assert np.array_equal(g["ia"], c["ia"]) and np.array_equal(g["ib"], c["ib"])
    ib = np.where(g["ib"] >= 0, g["ib"], -1)
    res = oracle.residual_3d(s["m"], Iinv, Iw, v0, g["ia"], ib, g["bases"].reshape(-1), c["arm_a"].reshape(-1),
                             c["arm_b"].reshape(-1), s["CoR"], s["mu"], g["alpha"], g["beta"].reshape(-1))
    assert st["n_contacts"] > 100
    if st["succeeded"]:
        assert res <= 1e-7 * 1.001
    assert abs(res - st["error"]) <= 1e-12 + 1e-6 * st["error"]
    nb = s["r"].shape[0]
    qa, _ = f64.state()
    qb, _ = f32.state()
    assert np.abs(qa[:3 * nb] - qb[:3 * nb]).max() <= 1e-3
