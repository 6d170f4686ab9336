"""The allocation-free solve (sg_sobogus_solve_2d_noalloc) against the regular one.

sg_sobogus_solve_2d_noalloc serves callers that cannot allocate GPU memory (code
inside another runtime's memory pool, real-time loops, allocation-forbidding
policies).  It runs the same kernels on the caller's device buffers with its
scratch in a fixed static device array, so its results must equal those of
sg_sobogus_solve_2d bit for bit.  The test owns the device buffers (allocated here
with torch, outside the entry point) and makes two calls in a row, which also shows
that the shared scratch is reset between calls.  This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def cluster(seed, n, spread):
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
        if q[i, 1] - r[i] <= -spread + 0.6:
            ia.append(i)
            ib.append(-1)
            bases += [0.0, 1.0, -1.0, 0.0]
    return m, v.reshape(-1), np.array(ia, np.int32), np.array(ib, np.int32), np.array(bases)


def noalloc_solve(gpulib, m, v0, ia, ib, bases, CoR, mu, tol, max_iters, eval_every=1):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    nc, nb = ia.shape[0], m.shape[0]

    def dbuf(a, dtype):
        return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device=dev)

    d_m, d_v0, d_bases = dbuf(m, torch.float64), dbuf(v0, torch.float64), dbuf(bases, torch.float64)
    d_ia, d_ib = dbuf(ia, torch.int32), dbuf(ib, torch.int32)
    d_cor = dbuf(np.full(nc, CoR), torch.float64)
    d_mu = dbuf(np.full(nc, mu), torch.float64)
    d_alpha = torch.zeros(max(nc, 1), dtype=torch.float64, device=dev)
    d_beta = torch.zeros(max(nc, 1), dtype=torch.float64, device=dev)
    d_v2 = torch.zeros(2 * nb, dtype=torch.float64, device=dev)
    d_f = torch.zeros(2 * nb, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    err = C.c_double(-1.0)
    its = C.c_uint32(0)
    status = gpulib.lib().sg_sobogus_solve_2d_noalloc(
        nb, d_m.data_ptr(), d_v0.data_ptr(), nc, d_ia.data_ptr(), d_ib.data_ptr(), d_bases.data_ptr(),
        d_cor.data_ptr(), d_mu.data_ptr(), max_iters, tol, eval_every, d_alpha.data_ptr(), d_beta.data_ptr(),
        d_v2.data_ptr(), d_f.data_ptr(), None, C.byref(err), C.byref(its))
    return status, dict(alpha=d_alpha.cpu().numpy()[:nc], beta=d_beta.cpu().numpy()[:nc], v2=d_v2.cpu().numpy(),
                        f=d_f.cpu().numpy(), error=err.value, iterations=its.value)


def test_noalloc_matches_regular_entry_on_two_calls_in_a_row(gpulib):
    ctx = gpulib.Context()
    calls = [(cluster(11, 300, 3.0), 0.0, 0.5, 1e-10, 300),   # friction
             (cluster(12, 180, 3.5), 0.3, 0.0, 1e-12, 2000)]  # frictionless restitution, smaller
    for (m, v0, ia, ib, bases), CoR, mu, tol, iters in calls:
        assert ia.size > 50
        ref = ctx.sobogus_solve_2d(m, v0, ia, ib, bases, CoR, mu, tol, iters)
        status, got = noalloc_solve(gpulib, m, v0, ia, ib, bases, CoR, mu, tol, iters)
        assert status in (gpulib.SG_OK, gpulib.SG_NOT_CONVERGED)
        assert (status == gpulib.SG_OK) == ref["succeeded"]
        # Same kernels, same colouring, same arithmetic: bit-identical outputs.
        for key in ("alpha", "beta", "v2", "f"):
            assert np.array_equal(got[key], ref[key]), key
        assert got["error"] == ref["error"] and got["iterations"] == ref["iterations"]
    ctx.close()


def test_noalloc_rejects_oversized_and_invalid_problems(gpulib):
    lib = gpulib.lib()
    err = C.c_double(0.0)
    its = C.c_uint32(0)
    # Beyond the fixed scratch: rejected before any device work (no pointer is touched).
    s = lib.sg_sobogus_solve_2d_noalloc(16385, 1, 1, 0, None, None, None, None, None, 10, 1e-9, 1, None, None, 1, 1,
                                        None, C.byref(err), C.byref(its))
    assert s == gpulib.SG_CAPACITY
    assert b"16384" in lib.sg_last_error_string()
    s = lib.sg_sobogus_solve_2d_noalloc(10, 1, 1, 65537, 1, 1, 1, 1, 1, 10, 1e-9, 1, 1, 1, 1, 1, None, C.byref(err),
                                        C.byref(its))
    assert s == gpulib.SG_CAPACITY
    # A contact index out of range is caught on the device before the solve runs.
    m, v0, ia, ib, bases = cluster(13, 40, 2.0)
    ib = ib.copy()
    ib[0] = 10_000
    status, _ = noalloc_solve(gpulib, m, v0, ia, ib, bases, 0.0, 0.5, 1e-9, 10)
    assert status == gpulib.SG_BAD_INPUT


def lattice(n_side, seed):
    """n_side^2 discs on a square lattice whose spacing lets each disc touch its 8 neighbours,
    resting on a floor: about 4 contacts per body, near the scratch's contact limit at 128^2."""
    rng = np.random.default_rng(seed)
    r = 0.1
    d = 2.0 * r / np.sqrt(2.0) * 0.999
    i, j = np.meshgrid(np.arange(n_side), np.arange(n_side), indexing="ij")
    idx = (i * n_side + j).reshape(-1)
    q = np.stack([j.reshape(-1) * d, i.reshape(-1) * d + r * 0.999], axis=1)
    m = rng.uniform(0.5, 2.0, n_side * n_side)
    v = rng.normal(0, 0.5, (n_side * n_side, 2))
    ia, ib = [], []
    for di, dj in ((0, 1), (1, 0), (1, 1), (1, -1)):
        ok = (i + di < n_side) & (j + dj >= 0) & (j + dj < n_side)
        a = (i * n_side + j)[ok]
        b = ((i + di) * n_side + (j + dj))[ok]
        ia.append(np.minimum(a, b))
        ib.append(np.maximum(a, b))
    ia, ib = np.concatenate(ia), np.concatenate(ib)
    order = np.lexsort((ib, ia))
    ia, ib = ia[order], ib[order]
    nrm = q[ia] - q[ib]
    nrm /= np.linalg.norm(nrm, axis=1)[:, None]
    floor = idx[q[:, 1] <= r]
    ia = np.concatenate([ia, floor]).astype(np.int32)
    ib = np.concatenate([ib, np.full(floor.shape[0], -1)]).astype(np.int32)
    nrm = np.concatenate([nrm, np.tile([0.0, 1.0], (floor.shape[0], 1))])
    bases = np.stack([nrm[:, 0], nrm[:, 1], -nrm[:, 1], nrm[:, 0]], axis=1).reshape(-1)
    return m, v.reshape(-1), ia, ib, bases


def test_noalloc_at_the_scratch_limits(gpulib):
    """Exactly 16,384 bodies and close to 65,536 contacts, bit-identical with the regular entry, twice;
    then bodies with no contacts (v2 = v0, no friction impulse)."""
    ctx = gpulib.Context()
    m, v0, ia, ib, bases = lattice(128, 21)
    assert m.shape[0] == 16384 and 64000 < ia.shape[0] <= 65536
    for _ in range(2):
        ref = ctx.sobogus_solve_2d(m, v0, ia, ib, bases, 0.2, 0.5, 1e-9, 60)
        status, got = noalloc_solve(gpulib, m, v0, ia, ib, bases, 0.2, 0.5, 1e-9, 60)
        assert status in (gpulib.SG_OK, gpulib.SG_NOT_CONVERGED)
        for key in ("alpha", "beta", "v2", "f"):
            assert np.array_equal(got[key], ref[key]), key
        assert got["error"] == ref["error"] and got["iterations"] == ref["iterations"]
    empty = np.zeros(0, np.int32)
    status, got = noalloc_solve(gpulib, m, v0, empty, empty, np.zeros(0), 0.2, 0.5, 1e-9, 60)
    assert status == gpulib.SG_OK
    assert np.array_equal(got["v2"], v0) and not got["f"].any() and got["iterations"] == 0
    ctx.close()
