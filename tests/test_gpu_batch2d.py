"""Batched Ball2D scenes on the GPU against one CPU oracle per scene.

Bars: every scene, every step, bit-exact with the oracle stepping that scene alone (contact
set, impulses, per-scene Gauss-Seidel sweeps, positions and velocities), given the GPU's
colour order replayed per scene; the graph-replayed step loop and the capacity-overflow
retry give the same bits as step-by-step stepping.
"""
import numpy as np
import pytest

from scisim_gb300 import scenes

pytestmark = pytest.mark.gpu


def small_batch(seed=1, n_scenes=10, nmax=300):
    b = scenes.ball2d_batch(n_scenes=n_scenes, nmax=nmax, seed=seed)
    return b


def gpu_batch(gpulib, b, cache=None, **kw):
    cfg = dict(dt=b["dt"], gravity=b["gravity"], tol=1e-9, max_iters=2000, integrator=gpulib.SYMPLECTIC_EULER,
               cache_mode=gpulib.CACHE_NORMAL_AND_FRICTION if cache is None else cache)
    cfg.update(kw)
    ctx = gpulib.Context(**cfg)
    ctx.upload_batch2d(b["body_off"], b["q"], b["v"], b["r"], b["m"], b["plane_off"], b["plane_x"], b["plane_n"],
                       b["mu"], b["CoR"])
    return ctx


def oracle_scenes(oracle, b, cache, **kw):
    sims = []
    for s in range(len(b["mu"])):
        sc = scenes.batch_scene(b, s)
        cfg = dict(dt=sc["dt"], gravity=sc["gravity"], mu=sc["mu"], CoR=sc["CoR"], tol=1e-9, max_iters=2000,
                   cache_mode=cache)
        cfg.update(kw)
        sims.append(oracle.Ball2D(sc["q"], sc["v"], sc["r"], sc["m"], sc["plane_x"], sc["plane_n"], **cfg))
    return sims


def local_contacts(g, c0, c1, b0, p0):
    ia = g["ia"][c0:c1] - b0
    ib = g["ib"][c0:c1].copy()
    ball = ib >= 0
    ib[ball] -= b0
    ib[~ball] = -1 - ((-1 - ib[~ball]) - p0)
    return ia, ib


@pytest.mark.parametrize("cache", ["none", "normal_and_friction"])
def test_batch_matches_per_scene_oracle(gpulib, oracle, cache):
    b = small_batch()
    mode = {"none": gpulib.CACHE_NONE, "normal_and_friction": gpulib.CACHE_NORMAL_AND_FRICTION}[cache]
    ctx = gpu_batch(gpulib, b, cache=mode)
    sims = oracle_scenes(oracle, b, mode)
    S = len(sims)
    seen = 0
    for step in range(30):
        st = ctx.step(1, first_iteration=step + 1)
        stats = ctx.batch_scene_stats()
        order, _ = ctx.last_solve_order()
        g = ctx.last_contacts()
        q, v = ctx.state()
        coff = np.concatenate([[0], np.cumsum(stats["n_contacts"])])
        assert coff[-1] == st["n_contacts"]
        for s in range(S):
            c0, c1 = int(coff[s]), int(coff[s + 1])
            b0, b1 = int(b["body_off"][s]), int(b["body_off"][s + 1])
            if c1 > c0:
                sel = order[(order >= c0) & (order < c1)] - c0
                sims[s].set_next_order(sel)
            so = sims[s].step()
            assert so["n_contacts"] == c1 - c0
            if c1 > c0:
                assert so["iterations"] == stats["iterations"][s]
                oc = sims[s].last_contacts()
                ia, ib = local_contacts(g, c0, c1, b0, int(b["plane_off"][s]))
                assert np.array_equal(ia, oc["ia"]) and np.array_equal(ib, oc["ib"])
                assert np.array_equal(g["alpha"][c0:c1], oc["alpha"])
                assert np.array_equal(g["beta"][c0:c1], oc["beta"])
            qo, vo = sims[s].state()
            assert np.array_equal(q[2 * b0:2 * b1], qo) and np.array_equal(v[2 * b0:2 * b1], vo)
        seen += st["n_contacts"]
    assert seen > 1000


def test_batch_graph_and_overflow_retry_are_bit_exact(gpulib):
    b = small_batch(seed=2, n_scenes=24, nmax=500)
    a = gpu_batch(gpulib, b)
    a.step(16)                        # two replays of the 8-step graph
    c = gpu_batch(gpulib, b)
    for it in range(16):              # step by step, no graph
        c.step(1, first_iteration=it + 1)
    d = gpu_batch(gpulib, b)
    d.batch_set_capacity(40)          # overflows on the first chunk, restored and re-run
    st = d.step(16)
    qa, va = a.state()
    for other in (c, d):
        qo, vo = other.state()
        assert np.array_equal(qa, qo) and np.array_equal(va, vo)
    assert st["n_contacts"] > 40
    sa, sd = a.batch_scene_stats(), d.batch_scene_stats()
    assert np.array_equal(sa["iterations"], sd["iterations"])
    assert np.array_equal(sa["n_contacts"], sd["n_contacts"])


def test_batch_flow_and_stats(gpulib):
    b = small_batch(seed=3, n_scenes=6, nmax=200)
    a = gpu_batch(gpulib, b, tol=1e-6)
    c = gpu_batch(gpulib, b, tol=1e-6)
    tot = 0
    for it in range(1, 9):
        st = a.step(1, first_iteration=it)
        tot += st["n_contacts"]
    q, v = b["q"], b["v"]
    for it in range(1, 9):
        q, v, _ = c.flow(it, q, v)
    qa, va = a.state()
    assert np.array_equal(qa, q) and np.array_equal(va, v)
    stats = a.batch_scene_stats()
    assert stats["n_contacts"].sum() == st["n_contacts"]
    assert np.all(stats["error"][stats["succeeded"]] < 1e-6)
    assert tot > 0


def test_batch_fp32_refine(gpulib, oracle):
    """FP32 sweeps + FP64 refinement per scene: every scene that reports convergence meets the
    tolerance under the oracle's FP64 residual of its own contacts, and the trajectories stay
    within 1e-3 of the FP64 batch."""
    b = small_batch(seed=5, n_scenes=12, nmax=400)
    f64 = gpu_batch(gpulib, b, tol=1e-6, max_iters=3000)
    f32 = gpu_batch(gpulib, b, tol=1e-6, max_iters=3000, precision=gpulib.PRECISION_FP32_REFINE)
    f64.step(24)
    f32.step(23)
    q0, v0 = f32.state()
    f32.step(1)
    stats = f32.batch_scene_stats()
    g = f32.last_contacts()
    coff = np.concatenate([[0], np.cumsum(stats["n_contacts"])])
    checked = 0
    for s in range(len(b["mu"])):
        c0, c1 = int(coff[s]), int(coff[s + 1])
        if c1 == c0 or not stats["succeeded"][s]:
            continue
        b0, b1 = int(b["body_off"][s]), int(b["body_off"][s + 1])
        ia, ib = local_contacts(g, c0, c1, b0, int(b["plane_off"][s]))
        n = g["n"][c0:c1]
        bases = np.concatenate([n, np.stack([-n[:, 1], n[:, 0]], 1)], 1).reshape(-1)
        res = oracle.residual_2d(b["m"][b0:b1], v0[2 * b0:2 * b1], ia, np.where(ib >= 0, ib, -1), bases,
                                 float(b["CoR"][s]), float(b["mu"][s]), g["alpha"][c0:c1], g["beta"][c0:c1])
        assert res <= 1e-6 * 1.001
        checked += 1
    assert checked >= 3
    qa, _ = f64.state()
    qb, _ = f32.state()
    assert np.abs(qa - qb).max() <= 1e-3
