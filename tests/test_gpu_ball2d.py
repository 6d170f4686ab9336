"""GPU parity tests: libscisim_gb300.so (through the C ABI) against the CPU oracle.

Bars (stated per test):
* broad phase, CCD, contact sets, normals, forcing terms: bit-exact;
* Gauss-Seidel with the GPU's own colour order replayed on the oracle: bit-exact;
* frictionless restitution (unique impulses): 1e-6 relative to the largest impulse;
* frictional solves: both residuals <= tol; trajectories within the bound the tolerance implies.
"""
import gzip
import hashlib
import json
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def load_fixture(tag):
    with gzip.open(os.path.join(GOLDEN, "aabb2d_fixture_%s.txt.gz" % tag), "rt") as fh:
        return np.array([float(t) for t in fh.read().split()]).reshape(-1, 4)


def digest(pairs):
    return hashlib.sha256(np.ascontiguousarray(pairs, dtype=np.int32).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def ctx(gpulib):
    c = gpulib.Context()
    yield c
    c.close()


# ---------------------------------------------------------------- broad phase
@pytest.mark.parametrize("tag", ["00", "01", "02"])
def test_broadphase_reference_fixtures(ctx, tag):
    expected = json.load(open(os.path.join(GOLDEN, "aabb2d_expected.json")))[tag]
    pairs = ctx.broadphase_2d(load_fixture(tag))
    assert pairs.shape[0] == expected["n_pairs"]
    assert digest(pairs) == expected["sha256"]


def test_broadphase_edge_cases(ctx, oracle):
    # empty, single, touching (touching boxes overlap), identical, nested, one huge box
    assert ctx.broadphase_2d(np.zeros((0, 4))).shape == (0, 2)
    assert ctx.broadphase_2d(np.array([[0, 0, 1, 1.0]])).shape == (0, 2)
    touch = np.array([[0, 0, 1, 1.0], [1, 0, 2, 1.0], [2.0000001, 0, 3, 1.0]])
    assert ctx.broadphase_2d(touch).tolist() == [[0, 1]]
    same = np.tile([[0.5, 0.5, 1.5, 1.5]], (7, 1))
    assert ctx.broadphase_2d(same).shape[0] == 21
    rng = np.random.default_rng(0)
    c = rng.uniform(-50, 50, (3000, 2))
    e = rng.uniform(0.01, 0.5, (3000, 2))
    boxes = np.concatenate([c - e, c + e], 1)
    boxes[17] = [-100, -100, 100, 100]  # one giant box overlaps everything
    got = ctx.broadphase_2d(boxes)
    assert np.array_equal(got, oracle.allpairs_overlaps_2d(boxes))


# ---------------------------------------------------------------- narrow phase
def test_ccd_reference_cases(ctx, oracle):
    cases = json.load(open(os.path.join(GOLDEN, "ccd_cases.json")))
    q0a = np.array([c["q0a"] for c in cases])
    q1a = np.array([c["q1a"] for c in cases])
    q0b = np.array([c["q0b"] for c in cases])
    q1b = np.array([c["q1b"] for c in cases])
    ra = np.array([c["ra"] for c in cases])
    rb = np.array([c["rb"] for c in cases])
    coeffs, hit, t = ctx.ccd_2d(q0a, q1a, ra, q0b, q1b, rb)
    for k, c in enumerate(cases):
        oc = oracle.ccd_coeffs_2d(c["q0a"], c["q1a"], c["ra"], c["q0b"], c["q1b"], c["rb"])
        assert np.array_equal(coeffs[k], oc)  # bit-exact
        if c["cexpected"] is not None:
            assert np.abs(coeffs[k] - np.array(c["cexpected"])).max() <= 1e-9
        assert bool(hit[k]) == c["hit"]
        if c["time_expr"] is not None:
            assert abs(t[k] - float(eval(c["time_expr"], {"sqrt": math.sqrt}))) <= c["time_tol"]


def test_ccd_random_bitexact(ctx, oracle):
    rng = np.random.default_rng(4)
    n = 20000
    q0a, q1a, q0b, q1b = (rng.uniform(-1, 1, (n, 2)) for _ in range(4))
    ra, rb = rng.uniform(0.05, 0.4, n), rng.uniform(0.05, 0.4, n)
    coeffs, hit, t = ctx.ccd_2d(q0a, q1a, ra, q0b, q1b, rb)
    for k in range(0, n, 97):
        oc = oracle.ccd_coeffs_2d(q0a[k], q1a[k], ra[k], q0b[k], q1b[k], rb[k])
        assert np.array_equal(coeffs[k], oc)
        h, tt = oracle.ccd_happens(oc)
        assert h == bool(hit[k])
        if h:
            assert t[k] == tt


# ---------------------------------------------------------------- friction solve
def cluster_problem(seed, n=300, spread=3.0, static_floor=True):
    rng = np.random.default_rng(seed)
    q = rng.uniform(-spread, spread, (n, 2))
    r = np.full(n, 0.2)
    m = rng.uniform(0.5, 2.0, n)
    v = rng.normal(0, 1, (n, 2))
    ia, ib, bases = [], [], []
    for i in range(n):
        for j in range(i + 1, n):
            d = q[i] - q[j]
            if np.linalg.norm(d) <= r[i] + r[j]:
                nn = d / np.linalg.norm(d)
                ia.append(i)
                ib.append(j)
                bases += [nn[0], nn[1], -nn[1], nn[0]]
    if static_floor:
        for i in range(n):
            if q[i, 1] - r[i] <= -spread + 0.6:
                ia.append(i)
                ib.append(-1)
                bases += [0.0, 1.0, -1.0, 0.0]
    return m, v.reshape(-1), np.array(ia, np.int32), np.array(ib, np.int32), np.array(bases)


@pytest.mark.parametrize("mu,CoR", [(0.0, 0.3), (0.5, 0.0), (0.8, 0.2)])
def test_sobogus_solve_replayed_order_bitexact(ctx, oracle, mu, CoR):
    m, v0, ia, ib, bases = cluster_problem(1)
    assert ia.size > 100
    g = ctx.sobogus_solve_2d(m, v0, ia, ib, bases, CoR, mu, 1e-10, 400)
    order, offs = ctx.last_solve_order()
    assert sorted(order.tolist()) == list(range(ia.size))
    # colours are independent sets: no two contacts of a colour share a body
    for c in range(len(offs) - 1):
        ks = order[offs[c]:offs[c + 1]]
        bodies = np.concatenate([ia[ks], ib[ks][ib[ks] >= 0]])
        assert np.unique(bodies).size == bodies.size
    o = oracle.sobogus_solve_2d(m, v0, ia, ib, bases, CoR, mu, 1e-10, 400, order=order)
    assert g["iterations"] == o["iterations"]
    assert g["error"] == o["error"]
    assert np.array_equal(g["alpha"], o["alpha"]) and np.array_equal(g["beta"], o["beta"])
    assert np.array_equal(g["v2"], o["v2"]) and np.array_equal(g["f"], o["f"])


def test_sobogus_frictionless_matches_sequential_reference_order(ctx, oracle):
    """Frictionless restitution: the post-impact velocity is unique (strictly convex
    problem in v), so the GPU's coloured order and the reference's sequential order agree
    on v2 to 1e-6 relative even where degenerate contact loops leave impulses non-unique."""
    m, v0, ia, ib, bases = cluster_problem(2, n=200, spread=3.5)
    g = ctx.sobogus_solve_2d(m, v0, ia, ib, bases, 0.3, 0.0, 1e-13, 20000)
    o = oracle.sobogus_solve_2d(m, v0, ia, ib, bases, 0.3, 0.0, 1e-13, 20000)
    assert g["succeeded"] and o["succeeded"]
    scale = np.abs(o["v2"]).max()
    assert np.abs(g["v2"] - o["v2"]).max() <= 1e-6 * scale
    assert (g["beta"] == 0.0).all()


def test_sobogus_frictionless_isolated_pairs_unique_impulses(ctx, oracle):
    """Isolated pairs have unique impulses: GPU alpha within 1e-6 relative of the oracle's
    and of BallBallConstraint::resolveImpact (BallBallConstraint.cpp:45-63)."""
    rng = np.random.default_rng(8)
    npair = 500
    m = rng.uniform(0.5, 3.0, 2 * npair)
    v0 = rng.normal(0, 1, 4 * npair)
    ang = rng.uniform(0, 2 * np.pi, npair)
    n = np.stack([np.cos(ang), np.sin(ang)], 1)
    ia = np.arange(0, 2 * npair, 2, dtype=np.int32)
    ib = ia + 1
    bases = np.concatenate([n, np.stack([-n[:, 1], n[:, 0]], 1)], 1).reshape(-1)
    g = ctx.sobogus_solve_2d(m, v0, ia, ib, bases, 0.4, 0.0, 1e-14, 100)
    o = oracle.sobogus_solve_2d(m, v0, ia, ib, bases, 0.4, 0.0, 1e-14, 100)
    vr = v0.reshape(-1, 2)[ia] - v0.reshape(-1, 2)[ib]
    ndotv = (n * vr).sum(1)
    closed = np.where(ndotv < 0, -(1.4) * ndotv / (1 / m[ia] + 1 / m[ib]), 0.0)
    scale = np.abs(closed).max()
    assert np.abs(g["alpha"] - o["alpha"]).max() <= 1e-6 * scale
    assert np.abs(g["alpha"] - closed).max() <= 1e-6 * scale


def test_sobogus_friction_residual_and_momentum(ctx, oracle):
    """Friction: the GPU solution meets tol under the oracle's own residual function."""
    m, v0, ia, ib, bases = cluster_problem(3, n=250, spread=4.5, static_floor=False)
    g = ctx.sobogus_solve_2d(m, v0, ia, ib, bases, 0.0, 0.5, 1e-9, 20000)
    assert g["succeeded"] and g["error"] <= 1e-9
    res = oracle.residual_2d(m, v0, ia, ib, bases, 0.0, 0.5, g["alpha"], g["beta"])
    assert res <= 2e-9
    p0 = (m[:, None] * v0.reshape(-1, 2)).sum(0)
    p1 = (m[:, None] * g["v2"].reshape(-1, 2)).sum(0)
    assert np.abs(p0 - p1).max() <= 1e-6


def test_sobogus_edge_cases(ctx, gpulib):
    # no contacts: v2 = v0
    r = ctx.sobogus_solve_2d(np.ones(3), np.arange(6.0), np.zeros(0, np.int32), np.zeros(0, np.int32),
                             np.zeros(0), 0.0, 0.5, 1e-9, 10)
    assert np.array_equal(r["v2"], np.arange(6.0)) and r["error"] == 0.0
    # bad body index is rejected on the host
    with pytest.raises(gpulib.SgError):
        ctx.sobogus_solve_2d(np.ones(2), np.zeros(4), [0], [5], [1.0, 0.0, 0.0, 1.0], 0.0, 0.5, 1e-9, 10)
    # max_iters reached: best iterate, SG_NOT_CONVERGED reported as succeeded = False
    m, v0, ia, ib, bases = cluster_problem(5)
    g = ctx.sobogus_solve_2d(m, v0, ia, ib, bases, 0.0, 0.5, 1e-30, 3)
    assert not g["succeeded"] and g["iterations"] == 3 and np.isfinite(g["error"])


# ---------------------------------------------------------------- full step
def box_scene(n_side=16, seed=3):
    from scisim_gb300 import scenes
    return scenes.box_drop_1024(seed=seed, n_side=n_side)


def run_both(gpulib, oracle, s, steps, **over):
    kw = dict(dt=s["dt"], gravity=s["gravity"], mu=s["mu"], CoR=s["CoR"], tol=s["tol"], max_iters=s["max_iters"])
    kw.update(over)
    ctx = gpulib.Context(**kw)
    ctx.upload_ball2d(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"])
    ora = oracle.Ball2D(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"], **kw)
    return ctx, ora


def test_step_contact_sets_bitexact_from_same_state(gpulib, oracle):
    """Every step: the GPU's active set equals the oracle's active set for the same (q0, q1)."""
    s = box_scene(16)
    ctx, ora = run_both(gpulib, oracle, s, 0)
    for step in range(60):
        q0, v0 = ctx.state()
        st = ctx.step(1)
        c = ctx.last_contacts()
        q1_pred, _ = ora.umap(q0, v0)
        ia, ib = ora.active_set(q0, q1_pred)
        assert st["n_contacts"] == ia.size
        assert np.array_equal(c["ia"], ia) and np.array_equal(c["ib"], ib), step
    ctx.close()


def test_step_trajectory_frictionless_restitution(gpulib, oracle):
    """mu = 0: unique impulses; GPU and oracle trajectories agree over 50 steps."""
    s = box_scene(12)
    ctx, ora = run_both(gpulib, oracle, s, 50, mu=0.0, tol=1e-12, max_iters=20000)
    worst_a = 0.0
    for step in range(50):
        st = ctx.step(1)
        ost = ora.step()
        assert st["n_contacts"] == ost["n_contacts"], step
        gc, oc = ctx.last_contacts(), ora.last_contacts()
        assert np.array_equal(gc["ia"], oc["ia"]) and np.array_equal(gc["ib"], oc["ib"])
        if oc["alpha"].size:
            worst_a = max(worst_a, np.abs(gc["alpha"] - oc["alpha"]).max() / max(np.abs(oc["alpha"]).max(), 1e-300))
    assert worst_a <= 1e-6
    gq, gv = ctx.state()
    oq, ov = ora.state()
    assert np.abs(gq - oq).max() <= 1e-8
    ctx.close()


def test_step_friction_replayed_order_bitexact(gpulib, oracle):
    """Friction (mu 0.5, CoR 0.3, tol 1e-9): when the oracle replays the GPU's colour order,
    every step of the box drop is bit-identical (positions, velocities, impulses)."""
    s = box_scene(14, seed=4)
    ctx, ora = run_both(gpulib, oracle, s, 0)
    for step in range(50):
        st = ctx.step(1)
        order, _ = ctx.last_solve_order()
        if st["n_contacts"]:
            ora.set_next_order(order)
        ost = ora.step()
        assert st["n_contacts"] == ost["n_contacts"], step
        gq, gv = ctx.state()
        oq, ov = ora.state()
        assert np.array_equal(gq, oq) and np.array_equal(gv, ov), step
        if st["n_contacts"]:
            gc, oc = ctx.last_contacts(), ora.last_contacts()
            assert np.array_equal(gc["alpha"], oc["alpha"]) and np.array_equal(gc["beta"], oc["beta"])
            assert st["iterations"] == ost["iterations"] and st["error"] == ost["error"]
    ctx.close()


def test_step_friction_residual_against_sequential_oracle(gpulib, oracle):
    """Friction against the reference's own (sequential) sweep order: contact sets equal
    from the same state, and every GPU solution meets tol under the oracle's residual."""
    s = box_scene(12)
    ctx, ora = run_both(gpulib, oracle, s, 0)
    for step in range(50):
        q0, v0 = ctx.state()
        st = ctx.step(1)
        if not st["n_contacts"]:
            continue
        gc = ctx.last_contacts()
        q1p, _ = ora.umap(q0, v0)
        ia, ib = ora.active_set(q0, q1p)
        assert np.array_equal(gc["ia"], ia) and np.array_equal(gc["ib"], ib)
        n = gc["n"]
        bases = np.concatenate([n, np.stack([-n[:, 1], n[:, 0]], 1)], 1).reshape(-1)
        ibs = np.where(gc["ib"] >= 0, gc["ib"], -1).astype(np.int32)
        res = oracle.residual_2d(s["m"], v0, gc["ia"], ibs, bases, s["CoR"], s["mu"], gc["alpha"], gc["beta"])
        assert st["error"] <= s["tol"] or st["iterations"] == s["max_iters"]
        if st["error"] <= s["tol"]:
            assert res <= 2 * s["tol"], (step, res)
    ctx.close()


def test_step_with_warm_start_cache(gpulib, oracle):
    s = box_scene(12, seed=9)
    ctx, ora = run_both(gpulib, oracle, s, 0, cache_mode=2, mu=0.0, tol=1e-12, max_iters=20000)
    for step in range(40):
        st = ctx.step(1)
        ost = ora.step()
        assert st["n_contacts"] == ost["n_contacts"]
    gq, _ = ctx.state()
    oq, _ = ora.state()
    assert np.abs(gq - oq).max() <= 1e-8
    ctx.close()


def test_step_determinism(gpulib):
    s = box_scene(16, seed=5)
    outs = []
    for _ in range(2):
        ctx = gpulib.Context(dt=s["dt"], mu=s["mu"], CoR=s["CoR"], tol=s["tol"], max_iters=300)
        ctx.upload_ball2d(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"])
        ctx.step(40)
        outs.append(ctx.state())
        ctx.close()
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


def test_flow_host_buffers_matches_device_steps(gpulib):
    s = box_scene(10, seed=6)
    kw = dict(dt=s["dt"], mu=s["mu"], CoR=s["CoR"], tol=s["tol"], max_iters=500)
    a = gpulib.Context(**kw)
    a.upload_ball2d(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"])
    a.step(20)
    b = gpulib.Context(**kw)
    b.upload_ball2d(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"])
    q, v = s["q"].copy(), s["v"].copy()
    for it in range(1, 21):
        q, v, _ = b.flow(it, q, v)
    qa, va = a.state()
    assert np.array_equal(qa, q) and np.array_equal(va, v)
    a.close()
    b.close()


def test_slope_scene_gpu_matches_oracle(gpulib, oracle):
    """Reference analytic slope scene (Verlet, dt 1e-5): GPU equals oracle after 2,000 steps."""
    scenes = json.load(open(os.path.join(GOLDEN, "slope_scenes.json")))
    sc = [x for x in scenes if x["name"] == "ball2d_sliding_friction_posx_01"][0]
    b = sc["ball"]
    kw = dict(dt=sc["dt"], gravity=sc["gravity"], mu=sc["mu"], CoR=sc["CoR"], tol=sc["tol"],
              max_iters=sc["max_iters"], integrator=1)
    ctx = gpulib.Context(**kw)
    ctx.upload_ball2d([b["x"], b["y"]], [b["vx"], b["vy"]], [b["r"]], [b["m"]], sc["plane_x"], sc["plane_n"])
    ctx.step(2000)
    ora = oracle.Ball2D([b["x"], b["y"]], [b["vx"], b["vy"]], [b["r"]], [b["m"]], sc["plane_x"], sc["plane_n"],
                        integrator=oracle.VERLET, **{k: v for k, v in kw.items() if k != "integrator"})
    ora.run(2000)
    gq, gv = ctx.state()
    oq, ov = ora.state()
    assert np.array_equal(gq, oq) and np.array_equal(gv, ov)
    ctx.close()


# ---------------------------------------------------------------- FP32 sweeps + FP64 refinement
@pytest.mark.parametrize("mu,CoR", [(0.5, 0.0), (0.0, 0.3)])
def test_fp32_refine_solve_meets_fp64_residual(gpulib, oracle, mu, CoR):
    """Mixed precision: the returned impulses meet tol under the oracle's FP64 residual;
    frictionless post-impact velocities agree with the FP64 solve to 1e-6 relative."""
    m, v0, ia, ib, bases = cluster_problem(21, n=260, spread=4.0)
    c32 = gpulib.Context(precision=gpulib.PRECISION_FP32_REFINE)
    c64 = gpulib.Context(precision=gpulib.PRECISION_FP64)
    g = c32.sobogus_solve_2d(m, v0, ia, ib, bases, CoR, mu, 1e-9, 20000)
    ref = c64.sobogus_solve_2d(m, v0, ia, ib, bases, CoR, mu, 1e-9, 20000)
    assert g["succeeded"] and g["error"] <= 1e-9
    res = oracle.residual_2d(m, v0, ia, ib, bases, CoR, mu, g["alpha"], g["beta"])
    assert res <= 2e-9
    if mu == 0.0:
        assert np.abs(g["v2"] - ref["v2"]).max() <= 1e-6 * np.abs(ref["v2"]).max()
    c32.close()
    c64.close()


@pytest.mark.parametrize("mu,bound", [(0.0, 1e-7), (0.5, 1e-3)])
def test_fp32_refine_steps(gpulib, oracle, mu, bound):
    """Box drop with FP32 sweeps: exact contact sets, residual <= tol (FP64-evaluated) or the
    iteration cap, and positions close to the FP64 GPU path after 40 steps: 1e-7 without
    friction (unique velocities), 1e-3 with friction (non-unique impulses: FP32 and FP64
    sweeps reach different valid solutions; measured drift ~5e-5)."""
    s = box_scene(12, seed=2)
    kw = dict(dt=s["dt"], gravity=s["gravity"], mu=mu, CoR=s["CoR"], tol=1e-9, max_iters=5000)
    a = gpulib.Context(precision=gpulib.PRECISION_FP32_REFINE, **kw)
    b = gpulib.Context(precision=gpulib.PRECISION_FP64, **kw)
    for c in (a, b):
        c.upload_ball2d(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"])
    ora = oracle.Ball2D(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"], **kw)
    for step in range(40):
        q0, v0 = a.state()
        st = a.step(1)
        b.step(1)
        if st["n_contacts"]:
            q1p, _ = ora.umap(q0, v0)
            ia, ib = ora.active_set(q0, q1p)
            gc = a.last_contacts()
            assert np.array_equal(gc["ia"], ia) and np.array_equal(gc["ib"], ib)
            assert st["error"] <= kw["tol"] or st["iterations"] == kw["max_iters"]
    qa, _ = a.state()
    qb, _ = b.state()
    assert np.abs(qa - qb).max() <= bound
    a.close()
    b.close()


# ---------------------------------------------------------------- failure paths
def test_wait_timeout_is_reported_and_context_survives(gpulib):
    ctx = gpulib.Context()
    ctx.set_spin_limit(1000)
    assert ctx.selftest_wait_timeout() == gpulib.SG_DEVICE_TIMEOUT
    ctx.set_spin_limit(0)
    s = box_scene(6)
    ctx.upload_ball2d(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"])
    st = ctx.step(5)
    assert st["status"] in (gpulib.SG_OK, gpulib.SG_NOT_CONVERGED)
    ctx.close()


def test_bad_inputs_rejected(gpulib):
    with pytest.raises(gpulib.SgError):
        gpulib.Context(dt=-1.0)
    ctx = gpulib.Context()
    with pytest.raises(gpulib.SgError):
        ctx.upload_ball2d([0.0, 0.0], [0.0, 0.0], [-1.0], [1.0], [0.0, 0.0], [0.0, 1.0])
    ctx.close()
