"""Two-level FP32 sweeps (spatial patches on shared-memory velocities, contacts between patches
by shifted tile, the rest over the grid) on a dense pile large enough to use them.

Bars, from a settled pile (a checkpoint taken after a converged step): the two-level path runs;
at least one step converges, and every step that reports convergence meets the tolerance under
the oracle's FP64 residual of the GPU's impulses; the reported residual equals the oracle's
evaluation; positions stay within 5e-3 of the one-level FP32 solve and of FP64 after four steps
from the common state (different Gauss-Seidel orders of a frictional solve, whose solution set is
not a single point, so their iterates differ within the residual they reach).
"""
import numpy as np
import pytest

from scisim_gb300 import scenes

pytestmark = pytest.mark.gpu


def pile(gpulib, s, **kw):
    cfg = dict(dt=s["dt"], gravity=s["gravity"], mu=s["mu"], CoR=s["CoR"], tol=1e-6, max_iters=2000,
               cache_mode=gpulib.CACHE_NORMAL_AND_FRICTION)
    cfg.update(kw)
    ctx = gpulib.Context(**cfg)
    ctx.upload_ball2d(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"])
    return ctx


def test_two_level_sweeps(gpulib, oracle):
    n = 32768
    s = scenes.dense_pile(n=n, seed=2, width=20.0, height=15.0)
    # Form the pile (capped solves), settle it at the full settings until a step converges, then
    # start all three solvers from that state and impulse cache (a checkpoint).
    pre = pile(gpulib, s, precision=gpulib.PRECISION_FP32_REFINE, max_iters=50)
    it = 1
    for steps, cap in ((420, 50), (200, 200), (100, 1000)):
        pre.reconfigure(max_iters=cap)
        pre.step(steps, first_iteration=it)
        it += steps
    pre.reconfigure(max_iters=2000)
    for _ in range(200):
        st = pre.step(1, first_iteration=it)
        it += 1
        if st["succeeded"]:
            break
    assert st["succeeded"]
    ck = pre.checkpoint()
    pre.close()

    def from_ck(**kw):
        c = gpulib.Context(dt=s["dt"], gravity=s["gravity"])
        c.restore(ck)
        c.reconfigure(**kw)
        return c

    two = from_ck(precision=gpulib.PRECISION_FP32_REFINE)
    one = from_ck(precision=gpulib.PRECISION_FP32_REFINE)
    f64 = from_ck(precision=gpulib.PRECISION_FP64)
    # FP32 sweeps from the start (no FP64 start near the tolerance), so the two-level path runs.
    for c in (two, one):
        c.set_tuning(fp64_factor=0)
    one.set_two_level(False)
    two.profile_enable(True)
    two.profile_read(reset=True)
    checked = 0
    for j in range(4):
        q0, v0 = two.state()
        st = two.step(1, first_iteration=it + j)
        g = two.last_contacts()
        assert st["n_contacts"] >= 20000
        bases = np.concatenate([g["n"], np.stack([-g["n"][:, 1], g["n"][:, 0]], 1)], 1).reshape(-1)
        ib = np.where(g["ib"] >= 0, g["ib"], -1)
        res = oracle.residual_2d(s["m"], v0, g["ia"], ib, bases, s["CoR"], s["mu"], g["alpha"], g["beta"])
        assert abs(res - st["error"]) <= 1e-12 + 1e-6 * st["error"]
        if st["succeeded"]:
            assert res <= 1e-6 * 1.001
            checked += 1
        one.step(1, first_iteration=it + j)
        f64.step(1, first_iteration=it + j)
    prof = two.profile_read()
    assert checked > 0
    assert prof["two_level_solves"] >= 1
    qa, _ = two.state()
    qb, _ = one.state()
    qc, _ = f64.state()
    assert np.abs(qa - qb).max() <= 5e-3 and np.abs(qa - qc).max() <= 5e-3


def test_patch_layout_is_race_free(gpulib):
    """The partition the two-level sweeps run on, read back after a step and checked on the
    host: every contact's group holds both its bodies (patch interiors by patch, contacts between
    patches by shifted tile), band flags mark exactly the bodies that blocks other than their
    patch's touch, and no body occurs twice among the contacts of one (group, colour), so the
    contacts a block or the grid updates together never share a body."""
    n = 32768
    s = scenes.dense_pile(n=n, seed=2, width=20.0, height=15.0)
    ctx = pile(gpulib, s, precision=gpulib.PRECISION_FP32_REFINE, max_iters=50)
    ctx.step(420)
    st = ctx.step(1)
    nb, nc = s["r"].shape[0], st["n_contacts"]
    g = ctx.last_contacts()
    L = ctx.patch_layout(nc, nb)
    P, Pb = L["P"], L["Pb"]
    assert 2 <= P < Pb
    grp, col = L["group"], L["color"]
    bp, bt, band = L["body_patch"], L["body_tile"], L["body_band"]
    ia, ib = g["ia"], g["ib"]
    has_b = ib >= 0
    inside = grp < P
    tile = (grp >= P) & (grp < P + Pb)
    rest = grp == P + Pb
    assert np.all(inside | tile | rest)
    assert np.all(bp[ia[inside]] == grp[inside])
    m = inside & has_b
    assert np.all(bp[ib[m]] == grp[m])
    between = ~inside
    assert np.all(has_b[between])
    assert np.all(bp[ia[between]] != bp[ib[between]])
    assert np.all(bt[ia[tile]] == grp[tile] - P) and np.all(bt[ib[tile]] == grp[tile] - P)
    assert np.all(bt[ia[rest]] != bt[ib[rest]])
    expect = np.zeros(nb, np.int32)
    expect[ia[between]] = 1
    expect[ib[between]] = 1
    assert np.array_equal(band, expect)
    key = grp.astype(np.int64) * 64 + col
    pairs = np.concatenate([np.stack([key, ia], 1), np.stack([key[has_b], ib[has_b]], 1)])
    assert np.unique(pairs, axis=0).shape[0] == pairs.shape[0]
    # Most contacts between patches are swept inside a shifted tile.
    assert tile.sum() > 0 and rest.sum() < 0.25 * between.sum()


def test_two_level_is_deterministic(gpulib):
    """The same bits from run to run on the 262,144-disc pile over the 600 capped steps that form
    it.  There the largest patches hold more contacts than fit in shared memory, so which
    contacts are staged depends on their order within a colour, which atomics set and which
    varies between runs; staged and unstaged contacts share one arithmetic, so the result does not."""
    s = scenes.dense_pile(n=262144, seed=2, width=40.0, height=60.0)
    out = []
    for _ in range(2):
        ctx = pile(gpulib, s, precision=gpulib.PRECISION_FP32_REFINE, max_iters=50)
        ctx.profile_enable(True)
        ctx.profile_read(reset=True)
        ctx.step(600)
        prof = ctx.profile_read()
        assert prof["two_level_solves"] > 100
        out.append(ctx.state())
        ctx.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("two_level,pairs", [(1, True), (1, False), (2, True), (2, False)])
def test_fp64_continuation(gpulib, oracle, two_level, pairs):
    """The FP32 form's FP64 continuation: from a settled pile, with a tolerance the eight-sweep
    FP64 probe does not reach and fp64_factor so large that every solve stays in FP64, the solves
    the probe leaves go on in FP64-precision sweeps: under the default two_level 1 one-level (with
    rate-predicted checks) for up to 160 sweeps, then on the two-level partition; under two_level 2
    on the partition from the start.  The sweeps run in float-float pairs on the FP32 pipe
    (k_gs_ff1 one-level, k_gs_patch_ff on the partition; the default) or in FP64 (k_gs_mixed,
    k_gs_patch64; sg_set_fp64_pairs 0).  The reported residual is the oracle's residual of the
    GPU's impulses, every continued solve ends below the residual the probe alone reaches from the
    same state, and every step that reports convergence meets the tolerance under it."""
    n = 32768
    s = scenes.dense_pile(n=n, seed=2, width=20.0, height=15.0)
    pre = pile(gpulib, s, precision=gpulib.PRECISION_FP32_REFINE, max_iters=50)
    it = 1
    for steps, cap in ((420, 50), (200, 200), (100, 1000)):
        pre.reconfigure(max_iters=cap)
        pre.step(steps, first_iteration=it)
        it += steps
    pre.reconfigure(max_iters=2000)
    for _ in range(200):
        st = pre.step(1, first_iteration=it)
        it += 1
        if st["succeeded"]:
            break
    ck = pre.checkpoint()
    pre.close()
    c = gpulib.Context(dt=s["dt"], gravity=s["gravity"])
    c.restore(ck)
    tol = 5e-8
    c.reconfigure(precision=gpulib.PRECISION_FP32_REFINE, tol=tol, max_iters=5000)
    c.set_tuning(fp64_factor=1000000)
    for bad in (-1, 3):
        with pytest.raises(gpulib.SgError):
            c.set_two_level(bad)
    c.set_two_level(two_level)
    c.set_fp64_pairs(pairs)
    c.profile_enable(True)
    c.profile_read(reset=True)
    continued = partitioned = 0
    for j in range(3):
        # The probe alone (eight FP64 sweeps) from the same state.
        p8 = gpulib.Context(dt=s["dt"], gravity=s["gravity"])
        p8.restore(c.checkpoint())
        p8.reconfigure(max_iters=8)
        e8 = p8.step(1, first_iteration=it + j)["error"]
        p8.close()
        q0, v0 = c.state()
        st = c.step(1, first_iteration=it + j)
        g = c.last_contacts()
        bases = np.concatenate([g["n"], np.stack([-g["n"][:, 1], g["n"][:, 0]], 1)], 1).reshape(-1)
        ib = np.where(g["ib"] >= 0, g["ib"], -1)
        res = oracle.residual_2d(s["m"], v0, g["ia"], ib, bases, s["CoR"], s["mu"], g["alpha"], g["beta"])
        assert abs(res - st["error"]) <= 1e-15 + 1e-6 * st["error"]
        if st["iterations"] > 8:  # beyond the eight-sweep FP64 probe
            continued += 1
            partitioned += int(two_level == 2 or st["iterations"] > 8 + 160)
            assert st["error"] < e8, (st["error"], e8)
        if st["succeeded"]:
            assert res <= tol * 1.001
    prof = c.profile_read()
    assert continued >= 1 and prof["fp64_start_solves"] == 3
    assert prof["two_level_solves"] == partitioned
    assert prof["contact_sweeps32"] == 0
    c.close()
