"""The 1,024-disc box drop at its stated size (32 x 32 jittered lattice, radii U[0.04, 0.06],
mu 0.5, restitution 0.3, symplectic Euler dt 0.01, block Gauss-Seidel tol 1e-9 with at most 5,000
sweeps), plain FP64 method on the GPU against the oracle's sequential Gauss-Seidel (contacts swept
in active-set order, one at a time, as Sobogus.cpp's GaussSeidel does on the CPU).

Two phases, each with and without the impulse cache:

* steps 1-20, independent trajectories: the lattice falls and meets the floor; every step both
  solvers reach 1e-9, the contact sets (ia, ib) are identical, the oracle's residual of the GPU's
  impulses is at most 1e-9, and positions stay within 1e-8 of the oracle's own trajectory (measured
  about 3.5e-11 at step 20);
* steps 21-50, lockstep (the oracle restarted from the GPU's state and cache every step): from step
  21 the impacts pack the pile and neither the sequential solver nor the coloured one reaches 1e-9
  within 5,000 sweeps on most steps.  Two Gauss-Seidel orders stopped at the cap leave different
  iterates, so independent trajectories part (1e-7 at step 25, 1e-2 by step 50 for both orders
  alike).  The bars there: identical contact sets every step; wherever the oracle converges the GPU
  does too; wherever the GPU stops at the cap, so does the oracle, and over those steps the median
  of the GPU's residual over the oracle's is at most 4 (single steps measured from 0.5 to 70: where
  Gauss-Seidel stalls depends on the order); the oracle evaluates the GPU's returned impulses to the
  residual the GPU reports.
"""
import numpy as np
import pytest

from scisim_gb300 import scenes

pytestmark = pytest.mark.gpu

TOL = 1e-9


def _bases(n):
    n = n.reshape(-1, 2)
    return np.stack([n[:, 0], n[:, 1], -n[:, 1], n[:, 0]], axis=1).reshape(-1)


def _oracle_residual(oracle, s, v0, g):
    ib = np.where(g["ib"] >= 0, g["ib"], -1).astype(np.int32)
    return oracle.residual_2d(s["m"], v0, g["ia"], ib, _bases(g["n"]), s["CoR"], s["mu"], g["alpha"], g["beta"])


@pytest.mark.parametrize("cache", [0, 2])
def test_c1_box_drop_against_sequential_oracle(gpulib, oracle, cache):
    s = scenes.box_drop_1024(seed=1, n_side=32)
    assert s["r"].shape[0] == 1024
    kw = dict(dt=s["dt"], gravity=s["gravity"], mu=s["mu"], CoR=s["CoR"], tol=TOL, max_iters=5000, eval_every=1)
    ctx = gpulib.Context(cache_mode=cache, **kw)
    ctx.upload_ball2d(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"])
    seq = oracle.Ball2D(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"], cache_mode=cache, **kw)
    worst_dq = 0.0
    for it in range(1, 21):
        _, v0 = ctx.state()
        gs = ctx.step(1, first_iteration=it)
        os_ = seq.step()
        g, c = ctx.last_contacts(), seq.last_contacts()
        assert gs["n_contacts"] == os_["n_contacts"], it
        assert np.array_equal(g["ia"], c["ia"]) and np.array_equal(g["ib"], c["ib"]), it
        assert gs["succeeded"] and os_["succeeded"], it
        assert gs["error"] <= TOL and os_["error"] <= TOL, it
        if gs["n_contacts"]:
            assert _oracle_residual(oracle, s, v0, g) <= TOL * (1 + 1e-6), it
        gq, _ = ctx.state()
        oq, _ = seq.state()
        worst_dq = max(worst_dq, float(np.abs(gq - oq).max()))
        assert worst_dq <= 1e-8, (it, worst_dq)
    # Lockstep from the GPU's state (and impulse cache) for the packing impacts.
    lock = oracle.Ball2D(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"], cache_mode=cache, **kw)
    ratios = []
    for it in range(21, 51):
        q0, v0 = ctx.state()
        lock.set_state(q0, v0)
        if cache:
            prev = ctx.last_contacts()
            lock.set_cache(prev["ia"], prev["ib"], prev["alpha"], prev["beta"])
        gs = ctx.step(1, first_iteration=it)
        os_ = lock.step()
        g, c = ctx.last_contacts(), lock.last_contacts()
        assert gs["n_contacts"] == os_["n_contacts"], it
        assert np.array_equal(g["ia"], c["ia"]) and np.array_equal(g["ib"], c["ib"]), it
        res = _oracle_residual(oracle, s, v0, g)
        assert abs(res - gs["error"]) <= 1e-15 + 1e-6 * gs["error"], it
        if os_["succeeded"]:
            assert gs["succeeded"] and gs["error"] <= TOL, it
        if not gs["succeeded"]:
            assert gs["iterations"] == os_["iterations"] == 5000, it
            ratios.append(gs["error"] / os_["error"])
    # Where both stop at the cap, the iterate each order reaches varies widely from step to step
    # (single-step ratios from 0.5 to 70 measured); over the steps the coloured order does as well
    # as the sequential one.
    assert len(ratios) > 0
    assert np.median(ratios) <= 4.0, sorted(ratios)
    ctx.close()
