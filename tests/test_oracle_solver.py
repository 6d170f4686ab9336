"""Properties of the oracle's Coulomb solver restatement (So-bogus semantics).

Pins what the reference's asserts and closed forms fix:
* local solves satisfy the Coulomb law exactly (FB error ~ 0),
* an isolated frictionless ball-ball impact matches
  BallBallConstraint::resolveImpact (ball2d/Constraints/BallBallConstraint.cpp:45-63),
* ball-ball-only contact sets conserve momentum (GeometricImpactFrictionMap.cpp:396-410),
* mu = 0 gives beta = 0 (Sobogus.cpp:320-327),
* frictionless KKT conditions hold at the solution.
"""
import numpy as np
import pytest


def spd2(rng):
    a = rng.normal(size=(2, 2))
    W = a @ a.T + 0.1 * np.eye(2)
    return np.array([W[0, 0], W[0, 1], W[1, 1]]), W


def spd3(rng):
    a = rng.normal(size=(3, 3))
    W = a @ a.T + 0.1 * np.eye(3)
    return np.array([W[0, 0], W[0, 1], W[0, 2], W[1, 1], W[1, 2], W[2, 2]]), W


@pytest.mark.parametrize("dim", [2, 3])
def test_local_solve_satisfies_coulomb(oracle, dim):
    rng = np.random.default_rng(11 + dim)
    worst = 0.0
    for _ in range(2000):
        Wp, W = spd2(rng) if dim == 2 else spd3(rng)
        b = rng.normal(size=dim)
        mu = rng.choice([0.0, 0.1, 0.5, 1.0, 2.0])
        r = oracle.local_solve(dim, Wp, b, mu)
        u = W @ r + b
        e = oracle.fb_error(dim, r, u, mu) / (1.0 + np.abs(b).max())
        worst = max(worst, e)
    assert worst <= 1e-9


def test_local_solve_isotropic_3d_exact(oracle):
    rng = np.random.default_rng(5)
    for _ in range(500):
        wn, wt = rng.uniform(0.5, 2, 2)
        Wp = np.array([wn, 0, 0, wt, 0, wt])
        b = rng.normal(size=3)
        mu = rng.uniform(0, 1)
        r = oracle.local_solve(3, Wp, b, mu)
        u = np.diag([wn, wt, wt]) @ r + b
        assert oracle.fb_error(3, r, u, mu) <= 1e-12 * (1 + np.abs(b).max())


def test_local_solve_weak_slide_3d(oracle):
    """A sphere contact with isotropic W_TT where the slide barely exceeds the cone (the case
    whose sliding direction a plain fixed point cannot find): solved to the Coulomb law."""
    Wp = np.array([2104.1729537535039, -2.3361012610506652e-13, 5.840253152626663e-14, 7232.3270716106308,
                   -1.3642420526593924e-12, 7232.3270716106308])
    b = np.array([-0.61783481435953869, -1.4683859110528765, 0.017832300158811997])
    W = np.array([[Wp[0], Wp[1], Wp[2]], [Wp[1], Wp[3], Wp[4]], [Wp[2], Wp[4], Wp[5]]])
    r = oracle.local_solve(3, Wp, b, 0.6)
    u = W @ r + b
    assert oracle.fb_error(3, r, u, 0.6) <= 1e-12 * np.abs(b).max()
    assert abs(np.hypot(r[1], r[2]) - 0.6 * r[0]) <= 1e-15 * r[0] * 10  # on the cone boundary


def two_ball_problem(ma, mb, va, vb, n):
    n = np.asarray(n, float) / np.linalg.norm(n)
    t = np.array([-n[1], n[0]])
    return dict(m=np.array([ma, mb]), v0=np.concatenate([va, vb]), ia=[0], ib=[1],
                bases=np.concatenate([n, t]))


@pytest.mark.parametrize("CoR", [0.0, 0.3, 1.0])
def test_isolated_frictionless_impact_closed_form(oracle, CoR):
    P = two_ball_problem(2.0, 3.0, [1.0, 0.2], [-0.5, 0.1], [-1.0, 0.0])
    res = oracle.sobogus_solve_2d(P["m"], P["v0"], P["ia"], P["ib"], P["bases"], CoR, 0.0, 1e-14, 100)
    n = P["bases"][:2]
    ndotv = n @ (P["v0"][:2] - P["v0"][2:])
    alpha = -(1.0 + CoR) * ndotv / (1.0 / 2.0 + 1.0 / 3.0)
    assert res["succeeded"]
    assert abs(res["alpha"][0] - alpha) <= 1e-12 * abs(alpha)
    assert res["beta"][0] == 0.0
    v2 = P["v0"].copy()
    v2[:2] += n * alpha / 2.0
    v2[2:] -= n * alpha / 3.0
    assert np.abs(res["v2"] - v2).max() <= 1e-12


def random_cluster(rng, n=60, spread=1.2):
    """Balls packed loosely with random velocities; contacts from proximity."""
    q = rng.uniform(-spread, spread, (n, 2))
    r = np.full(n, 0.16)
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
    return m, v.reshape(-1), np.array(ia, np.int32), np.array(ib, np.int32), np.array(bases)


@pytest.mark.parametrize("mu", [0.0, 0.5])
def test_momentum_conservation_and_mu0(oracle, mu):
    rng = np.random.default_rng(21)
    m, v0, ia, ib, bases = random_cluster(rng)
    assert ia.size > 10
    res = oracle.sobogus_solve_2d(m, v0, ia, ib, bases, 0.2, mu, 1e-11, 20000)
    p0 = (m[:, None] * v0.reshape(-1, 2)).sum(0)
    p1 = (m[:, None] * res["v2"].reshape(-1, 2)).sum(0)
    assert np.abs(p0 - p1).max() <= 1e-6
    if mu == 0.0:
        assert (res["beta"] == 0.0).all()
    assert res["error"] <= 1e-11 or not res["succeeded"]


def test_frictionless_kkt(oracle):
    rng = np.random.default_rng(23)
    m, v0, ia, ib, bases = random_cluster(rng)
    res = oracle.sobogus_solve_2d(m, v0, ia, ib, bases, 0.0, 0.0, 1e-12, 50000)
    assert res["succeeded"]
    n = bases.reshape(-1, 4)[:, :2]
    v2 = res["v2"].reshape(-1, 2)
    gap_rate = (n * (v2[ia] - v2[ib])).sum(1)
    assert (res["alpha"] >= -1e-12).all()
    assert (gap_rate >= -1e-5).all()
    assert np.abs(res["alpha"] * gap_rate).max() <= 1e-5


def test_solve_order_permutation_is_a_valid_gs(oracle):
    """Any sweep order converges to the same frictionless solution (unique)."""
    rng = np.random.default_rng(29)
    m, v0, ia, ib, bases = random_cluster(rng, n=40)
    a = oracle.sobogus_solve_2d(m, v0, ia, ib, bases, 0.3, 0.0, 1e-13, 100000)
    perm = rng.permutation(ia.size).astype(np.int32)
    b = oracle.sobogus_solve_2d(m, v0, ia, ib, bases, 0.3, 0.0, 1e-13, 100000, order=perm)
    assert a["succeeded"] and b["succeeded"]
    # velocities are unique for the frictionless problem
    assert np.abs(a["v2"] - b["v2"]).max() <= 1e-8


def test_max_iters_returns_best_iterate(oracle):
    rng = np.random.default_rng(31)
    m, v0, ia, ib, bases = random_cluster(rng, n=80, spread=1.0)
    res = oracle.sobogus_solve_2d(m, v0, ia, ib, bases, 0.0, 0.5, 1e-30, 3)
    assert not res["succeeded"]
    assert res["iterations"] == 3
    assert np.isfinite(res["error"])


def test_warm_start_cache_reduces_iterations(oracle):
    from scisim_gb300 import scenes
    s = scenes.box_drop_1024(seed=3, n_side=12)
    common = dict(dt=s["dt"], gravity=s["gravity"], mu=s["mu"], CoR=0.0, tol=1e-8, max_iters=3000)
    cold = oracle.Ball2D(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"], **common)
    warm = oracle.Ball2D(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"],
                         cache_mode=oracle.CACHE_NORMAL_AND_FRICTION, **common)
    its_cold = its_warm = 0
    for _ in range(60):
        its_cold += cold.step()["iterations"]
        its_warm += warm.step()["iterations"]
    assert its_warm < its_cold
