"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: the oracle is a CPU restatement of the SCISim
reference algorithm used to check the GPU library (tests/, smoke) and as the
timed CPU baseline (bench.py).  Product code never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("SG_ORACLE_LIB") or os.path.join(HERE, "_build", "liboracle.so")

SYMPLECTIC_EULER, VERLET = 0, 1
CACHE_NONE, CACHE_NORMAL, CACHE_NORMAL_AND_FRICTION = 0, 1, 2
STAGGER_GEOMETRIC, STAGGER_SYMPLECTIC_EULER, STAGGER_STABILIZED = 0, 1, 2

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class GsParams(C.Structure):
    _fields_ = [("tol", C.c_double), ("max_iters", C.c_uint32), ("eval_every", C.c_uint32),
                ("order", _ip)]


class GsResult(C.Structure):
    _fields_ = [("error", C.c_double), ("iterations", C.c_uint32), ("succeeded", C.c_int32)]


class Ball2DParams(C.Structure):
    _fields_ = [("integrator", C.c_int32), ("cache_mode", C.c_int32), ("dt", C.c_double),
                ("gravity", C.c_double * 2), ("mu", C.c_double), ("CoR", C.c_double),
                ("tol", C.c_double), ("max_iters", C.c_uint32), ("eval_every", C.c_uint32),
                ("staggering", C.c_int32), ("stabilize", C.c_int32), ("penetration_threshold", C.c_double)]


class Sphere3DParams(C.Structure):
    _fields_ = [("dt", C.c_double), ("gravity", C.c_double * 3), ("mu", C.c_double), ("CoR", C.c_double),
                ("tol", C.c_double), ("max_iters", C.c_uint32), ("eval_every", C.c_uint32),
                ("staggering", C.c_int32), ("cache_mode", C.c_int32), ("stabilize", C.c_int32),
                ("penetration_threshold", C.c_double)]


class RigidBody2DParams(C.Structure):
    _fields_ = [("integrator", C.c_int32), ("cache_mode", C.c_int32), ("dt", C.c_double),
                ("gravity", C.c_double * 2), ("mu", C.c_double), ("CoR", C.c_double),
                ("tol", C.c_double), ("max_iters", C.c_uint32), ("eval_every", C.c_uint32),
                ("staggering", C.c_int32)]


class StepStats(C.Structure):
    _fields_ = [("n_contacts", C.c_int64), ("n_ball_ball", C.c_int64), ("n_ball_plane", C.c_int64),
                ("iterations", C.c_uint32), ("succeeded", C.c_int32), ("error", C.c_double)]


def build() -> str:
    """Compile the oracle with its Makefile (idempotent)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        i64 = C.c_int64
        for name in ("or_grid_overlaps_2d", "or_allpairs_overlaps_2d", "or_grid_overlaps_3d",
                     "or_allpairs_overlaps_3d"):
            f = getattr(L, name)
            f.restype = i64
            f.argtypes = [C.c_int, _dp, i64, _ip, C.POINTER(i64)]
        L.or_ccd_coeffs_2d.argtypes = [_dp, _dp, C.c_double, _dp, _dp, C.c_double, _dp]
        L.or_ccd_happens.argtypes = [_dp, _dp]
        L.or_ccd_happens.restype = C.c_int
        L.or_fb_error.argtypes = [C.c_int, _dp, _dp, C.c_double]
        L.or_fb_error.restype = C.c_double
        L.or_local_solve.argtypes = [C.c_int, _dp, _dp, C.c_double, _dp]
        L.or_sobogus_solve_2d.argtypes = [C.c_int, _dp, _dp, C.c_int, _ip, _ip, _dp, _dp, _dp,
                                          C.POINTER(GsParams), _dp, _dp, _dp, _dp, C.POINTER(GsResult)]
        L.or_sobogus_solve_2d_ex.argtypes = [C.c_int, _dp, _dp, C.c_int, _ip, _ip, _dp, _dp, _dp, _dp, _dp,
                                             C.POINTER(GsParams), _dp, _dp, _dp, _dp, C.POINTER(GsResult)]
        L.or_ball2d_create.restype = C.c_void_p
        L.or_ball2d_create.argtypes = [C.c_int, _dp, _dp, _dp, _dp, C.c_int, _dp, _dp,
                                       C.POINTER(Ball2DParams)]
        L.or_ball2d_destroy.argtypes = [C.c_void_p]
        L.or_ball2d_step.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(StepStats)]
        L.or_ball2d_step.restype = C.c_int
        L.or_ball2d_run.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.POINTER(StepStats),
                                    C.POINTER(C.c_int64)]
        L.or_ball2d_run.restype = C.c_int
        L.or_ball2d_get_state.argtypes = [C.c_void_p, _dp, _dp]
        L.or_ball2d_set_state.argtypes = [C.c_void_p, _dp, _dp]
        L.or_ball2d_last_contacts.restype = i64
        L.or_ball2d_last_contacts.argtypes = [C.c_void_p, i64, _ip, _ip, _dp, _dp, _dp]
        L.or_ball2d_active_set.restype = i64
        L.or_ball2d_active_set.argtypes = [C.c_void_p, _dp, _dp, i64, _ip, _ip]
        L.or_ball2d_umap.argtypes = [C.c_void_p, C.c_uint32, _dp, _dp, _dp, _dp]
        L.or_ball2d_set_next_order.argtypes = [C.c_void_p, C.c_int64, _ip]
        L.or_ball2d_set_cache.argtypes = [C.c_void_p, C.c_int64, _ip, _ip, _dp, _dp]
        L.or_ball2d_set_solver.argtypes = [C.c_void_p, C.c_double, C.c_uint32]
        L.or_residual_2d.argtypes = [C.c_int, _dp, _dp, C.c_int, _ip, _ip, _dp, _dp, _dp, _dp, _dp]
        L.or_residual_2d.restype = C.c_double
        L.or_residual_2d_ex.argtypes = [C.c_int, _dp, _dp, C.c_int, _ip, _ip, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        L.or_residual_2d_ex.restype = C.c_double
        L.or_mlp_param_count.restype = C.c_int
        L.or_mlp_forward.argtypes = [C.POINTER(C.c_float), C.c_int, C.POINTER(C.c_float), _dp]
        L.or_mlp_loss_grad.argtypes = [C.POINTER(C.c_float), C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float), _dp]
        L.or_mlp_loss_grad.restype = C.c_double
        L.or_sobogus_solve_3d.argtypes = [C.c_int, _dp, _dp, _dp, _dp, C.c_int, _ip, _ip, _dp, _dp, _dp,
                                          _dp, _dp, C.POINTER(GsParams), _dp, _dp, _dp, _dp,
                                          C.POINTER(GsResult)]
        L.or_sobogus_solve_3d_ex.argtypes = [C.c_int, _dp, _dp, _dp, _dp, C.c_int, _ip, _ip, _dp, _dp, _dp,
                                             _dp, _dp, _dp, _dp, C.POINTER(GsParams), _dp, _dp, _dp, _dp,
                                             C.POINTER(GsResult)]
        L.or_residual_3d.argtypes = [C.c_int, _dp, _dp, _dp, _dp, C.c_int, _ip, _ip, _dp, _dp, _dp, _dp,
                                     _dp, _dp, _dp]
        L.or_residual_3d.restype = C.c_double
        L.or_residual_3d_ex.argtypes = [C.c_int, _dp, _dp, _dp, _dp, C.c_int, _ip, _ip, _dp, _dp, _dp, _dp,
                                        _dp, _dp, _dp, _dp, _dp]
        L.or_residual_3d_ex.restype = C.c_double
        L.or_sphere_mass_inertia.argtypes = [C.c_double, C.c_double, _dp, _dp]
        L.or_sphere3d_create.restype = C.c_void_p
        L.or_sphere3d_create.argtypes = [C.c_int, _dp, _dp, _dp, _dp, _dp, C.c_int, _dp, _dp,
                                         C.POINTER(Sphere3DParams)]
        L.or_sphere3d_destroy.argtypes = [C.c_void_p]
        L.or_sphere3d_step.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(StepStats)]
        L.or_sphere3d_step.restype = C.c_int
        L.or_sphere3d_run.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.POINTER(StepStats),
                                      C.POINTER(C.c_int64)]
        L.or_sphere3d_run.restype = C.c_int
        L.or_sphere3d_get_state.argtypes = [C.c_void_p, _dp, _dp]
        L.or_sphere3d_set_state.argtypes = [C.c_void_p, _dp, _dp]
        L.or_sphere3d_world_inertia.argtypes = [C.c_void_p, _dp, _dp]
        L.or_sphere3d_umap.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp]
        L.or_sphere3d_set_solver.argtypes = [C.c_void_p, C.c_double, C.c_uint32]
        L.or_sphere3d_set_next_order.argtypes = [C.c_void_p, C.c_int64, _ip]
        L.or_sphere3d_active_set.restype = i64
        L.or_sphere3d_active_set.argtypes = [C.c_void_p, _dp, _dp, i64, _ip, _ip]
        L.or_sphere3d_last_contacts.restype = i64
        L.or_sphere3d_last_contacts.argtypes = [C.c_void_p, i64, _ip, _ip, _dp, _dp, _dp, _dp, _dp]
        L.or_rb2d_create.restype = C.c_void_p
        L.or_rb2d_create.argtypes = [C.c_int, _dp, _dp, _dp, _dp, _dp, C.c_int, _dp, _dp,
                                     C.POINTER(RigidBody2DParams)]
        L.or_rb2d_destroy.argtypes = [C.c_void_p]
        L.or_rb2d_step.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(StepStats)]
        L.or_rb2d_step.restype = C.c_int
        L.or_rb2d_run.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.POINTER(StepStats), C.POINTER(C.c_int64)]
        L.or_rb2d_run.restype = C.c_int
        L.or_rb2d_get_state.argtypes = [C.c_void_p, _dp, _dp]
        L.or_rb2d_set_state.argtypes = [C.c_void_p, _dp, _dp]
        L.or_rb2d_set_solver.argtypes = [C.c_void_p, C.c_double, C.c_uint32]
        L.or_rb2d_set_next_order.argtypes = [C.c_void_p, C.c_int64, _ip]
        L.or_rb2d_last_contacts.restype = i64
        L.or_rb2d_last_contacts.argtypes = [C.c_void_p, i64, _ip, _ip, _dp, _dp, _dp, _dp, _dp]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _pairs(fn, aabb, dim):
    aabb = f64(aabb).reshape(-1, 2 * dim)
    n = aabb.shape[0]
    total = C.c_int64(0)
    cap = max(16, 8 * n)
    while True:
        out = np.empty((cap, 2), dtype=np.int32)
        k = fn(n, _d(aabb), cap, _i(out), C.byref(total))
        if k >= 0:
            return out[:k].copy()
        cap = int(total.value) + 16


def grid_overlaps_2d(aabb):
    return _pairs(lib().or_grid_overlaps_2d, aabb, 2)


def allpairs_overlaps_2d(aabb):
    return _pairs(lib().or_allpairs_overlaps_2d, aabb, 2)


def grid_overlaps_3d(aabb):
    return _pairs(lib().or_grid_overlaps_3d, aabb, 3)


def allpairs_overlaps_3d(aabb):
    return _pairs(lib().or_allpairs_overlaps_3d, aabb, 3)


def ccd_coeffs_2d(q0a, q1a, ra, q0b, q1b, rb):
    c = np.zeros(3)
    args = [f64(x) for x in (q0a, q1a)]
    b = [f64(x) for x in (q0b, q1b)]
    lib().or_ccd_coeffs_2d(_d(args[0]), _d(args[1]), ra, _d(b[0]), _d(b[1]), rb, _d(c))
    return c


def ccd_happens(c):
    c = f64(c)
    t = C.c_double(-1.0)
    hit = lib().or_ccd_happens(_d(c), C.byref(t))
    return bool(hit), (t.value if hit else None)


def fb_error(dim, r, u, mu):
    return lib().or_fb_error(dim, _d(f64(r)), _d(f64(u)), mu)


def local_solve(dim, W, b, mu):
    r = np.zeros(dim)
    lib().or_local_solve(dim, _d(f64(W)), _d(f64(b)), mu, _d(r))
    return r


def sobogus_solve_2d(m, v0, ia, ib, bases, CoR, mu, tol, max_iters, eval_every=1, alpha=None,
                     beta=None, order=None, nrel_extra=None, drel_extra=None):
    """Ball2D FrictionSolver::solve (with the map's extra relative velocities nrel_extra, drel_extra,
    one per contact, when given).  Returns dict(alpha, beta, v2, f, error, iterations, succeeded)."""
    m, v0, bases = f64(m), f64(v0), f64(bases)
    ia, ib = i32(ia), i32(ib)
    nc = ia.shape[0]
    nb = m.shape[0]
    CoR = f64(np.broadcast_to(CoR, (nc,)))
    mu = f64(np.broadcast_to(mu, (nc,)))
    alpha = np.zeros(nc) if alpha is None else f64(alpha).copy()
    beta = np.zeros(nc) if beta is None else f64(beta).copy()
    v2 = np.zeros(2 * nb)
    f = np.zeros(2 * nb)
    order_arr = None if order is None else i32(order)
    gp = GsParams(tol, max_iters, eval_every, _i(order_arr) if order_arr is not None else None)
    gr = GsResult()
    if nrel_extra is None and drel_extra is None:
        lib().or_sobogus_solve_2d(nb, _d(m), _d(v0), nc, _i(ia), _i(ib), _d(bases), _d(CoR), _d(mu),
                                  C.byref(gp), _d(alpha), _d(beta), _d(v2), _d(f), C.byref(gr))
    else:
        nr = None if nrel_extra is None else f64(nrel_extra)
        dr = None if drel_extra is None else f64(drel_extra)
        lib().or_sobogus_solve_2d_ex(nb, _d(m), _d(v0), nc, _i(ia), _i(ib), _d(bases), _d(CoR), _d(mu),
                                     _d(nr) if nr is not None else None, _d(dr) if dr is not None else None,
                                     C.byref(gp), _d(alpha), _d(beta), _d(v2), _d(f), C.byref(gr))
    return dict(alpha=alpha, beta=beta, v2=v2, f=f, error=gr.error, iterations=gr.iterations,
                succeeded=bool(gr.succeeded))


def residual_2d(m, v0, ia, ib, bases, CoR, mu, alpha, beta, nrel_extra=None, drel_extra=None):
    """The solver's Coulomb residual of given impulses (alpha, beta), with the map's extra relative
    velocities folded into the forcing terms when given."""
    m, v0, bases = f64(m), f64(v0), f64(bases)
    ia, ib = i32(ia), i32(ib)
    nc = ia.shape[0]
    CoR = f64(np.broadcast_to(CoR, (nc,)))
    mu = f64(np.broadcast_to(mu, (nc,)))
    a, b = f64(alpha), f64(beta)
    if nrel_extra is not None or drel_extra is not None:
        nr = None if nrel_extra is None else f64(nrel_extra)
        dr = None if drel_extra is None else f64(drel_extra)
        return lib().or_residual_2d_ex(m.shape[0], _d(m), _d(v0), nc, _i(ia), _i(ib), _d(bases), _d(CoR), _d(mu),
                                       _d(nr) if nr is not None else None, _d(dr) if dr is not None else None,
                                       _d(a), _d(b))
    return lib().or_residual_2d(m.shape[0], _d(m), _d(v0), nc, _i(ia), _i(ib), _d(bases), _d(CoR), _d(mu),
                                _d(a), _d(b))


class Ball2D:
    """Ball2D system stepped by GeometricImpactFrictionMap + Sobogus (CPU oracle)."""

    def __init__(self, q, v, r, m, plane_x, plane_n, *, dt, gravity=(0.0, -9.81), mu=0.5, CoR=0.0,
                 tol=1e-9, max_iters=5000, eval_every=1, integrator=SYMPLECTIC_EULER,
                 cache_mode=CACHE_NONE, staggering=0, stabilize=False, penetration_threshold=0.0):
        self.q, self.v = f64(q), f64(v)
        self.r, self.m = f64(r), f64(m)
        self.nb = self.r.shape[0]
        px, pn = f64(plane_x).reshape(-1), f64(plane_n).reshape(-1)
        self.np = px.shape[0] // 2
        p = Ball2DParams(integrator, cache_mode, dt, (C.c_double * 2)(*gravity), mu, CoR, tol,
                         max_iters, eval_every, staggering, 1 if stabilize else 0, penetration_threshold)
        self._h = lib().or_ball2d_create(self.nb, _d(self.q), _d(self.v), _d(self.r), _d(self.m),
                                         self.np, _d(px), _d(pn), C.byref(p))
        self.iteration = 0

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().or_ball2d_destroy(h)
            self._h = None

    def step(self):
        self.iteration += 1
        st = StepStats()
        lib().or_ball2d_step(self._h, self.iteration, C.byref(st))
        return dict(n_contacts=st.n_contacts, n_ball_ball=st.n_ball_ball, n_ball_plane=st.n_ball_plane,
                    iterations=st.iterations, succeeded=bool(st.succeeded), error=st.error)

    def run(self, n_steps):
        """n_steps steps in C; returns (last step stats, total contacts, unconverged steps)."""
        st = StepStats()
        tot = C.c_int64(0)
        bad = lib().or_ball2d_run(self._h, self.iteration + 1, n_steps, C.byref(st), C.byref(tot))
        self.iteration += n_steps
        return (dict(n_contacts=st.n_contacts, iterations=st.iterations, succeeded=bool(st.succeeded),
                     error=st.error), tot.value, bad)

    def state(self):
        q = np.zeros(2 * self.nb)
        v = np.zeros(2 * self.nb)
        lib().or_ball2d_get_state(self._h, _d(q), _d(v))
        return q, v

    def set_state(self, q, v):
        q, v = f64(q), f64(v)
        lib().or_ball2d_set_state(self._h, _d(q), _d(v))

    def set_cache(self, ia, ib, alpha, beta):
        """Replaces the impulse cache with the given contacts' impulses (ib = -1 - plane)."""
        ia, ib, a, b = i32(ia), i32(ib), f64(alpha), f64(beta)
        lib().or_ball2d_set_cache(self._h, ia.shape[0], _i(ia), _i(ib), _d(a), _d(b))

    def set_solver(self, tol, max_iters):
        lib().or_ball2d_set_solver(self._h, tol, max_iters)

    def set_next_order(self, order):
        """Sweep order for the next step's solve (e.g. the GPU's colour order)."""
        order = i32(order)
        lib().or_ball2d_set_next_order(self._h, order.shape[0], _i(order))

    def last_contacts(self):
        L = lib()
        nc = L.or_ball2d_last_contacts(self._h, 0, None, None, None, None, None)
        nc = -nc - 1 if nc < 0 else nc
        ia = np.zeros(nc, np.int32)
        ib = np.zeros(nc, np.int32)
        n = np.zeros(2 * nc)
        a = np.zeros(nc)
        b = np.zeros(nc)
        L.or_ball2d_last_contacts(self._h, nc, _i(ia), _i(ib), _d(n), _d(a), _d(b))
        return dict(ia=ia, ib=ib, n=n.reshape(-1, 2), alpha=a, beta=b)

    def active_set(self, q0, q1):
        q0, q1 = f64(q0), f64(q1)
        L = lib()
        cap = 8 * self.nb + 16
        while True:
            ia = np.zeros(cap, np.int32)
            ib = np.zeros(cap, np.int32)
            k = L.or_ball2d_active_set(self._h, _d(q0), _d(q1), cap, _i(ia), _i(ib))
            if k >= 0:
                return ia[:k].copy(), ib[:k].copy()
            cap = -k + 15

    def umap(self, q0, v0):
        q0, v0 = f64(q0), f64(v0)
        q1 = np.zeros_like(q0)
        v1 = np.zeros_like(v0)
        lib().or_ball2d_umap(self._h, self.iteration + 1, _d(q0), _d(v0), _d(q1), _d(v1))
        return q1, v1


# ------------------------------------------------------------------ RigidBody3D spheres
def sphere_mass_inertia(r, density):
    """RigidBodySphere::computeMassAndInertia: (mass, principal moment)."""
    M, I = C.c_double(0.0), C.c_double(0.0)
    lib().or_sphere_mass_inertia(r, density, C.byref(M), C.byref(I))
    return M.value, I.value


def sobogus_solve_3d(m, Iinv, Iw, v0, ia, ib, bases, arm_a, arm_b, CoR, mu, tol, max_iters, eval_every=1,
                     alpha=None, beta=None, order=None, nrel_extra=None, drel_extra=None):
    """RigidBodies3D FrictionSolver::solve (with the map's extra relative velocities nrel_extra (1 per
    contact) and drel_extra (2 per contact) when given).  Returns dict(alpha, beta, v2, f, error,
    iterations, succeeded)."""
    m, Iinv, Iw, v0 = f64(m), f64(Iinv), f64(Iw), f64(v0)
    bases, arm_a, arm_b = f64(bases), f64(arm_a), f64(arm_b)
    ia, ib = i32(ia), i32(ib)
    nc, nb = ia.shape[0], m.shape[0]
    CoR = f64(np.broadcast_to(CoR, (nc,)))
    mu = f64(np.broadcast_to(mu, (nc,)))
    alpha = np.zeros(nc) if alpha is None else f64(alpha).copy()
    beta = np.zeros(2 * nc) if beta is None else f64(beta).copy()
    v2, f = np.zeros(6 * nb), np.zeros(6 * nb)
    order_arr = None if order is None else i32(order)
    gp = GsParams(tol, max_iters, eval_every, _i(order_arr) if order_arr is not None else None)
    gr = GsResult()
    if nrel_extra is None and drel_extra is None:
        lib().or_sobogus_solve_3d(nb, _d(m), _d(Iinv), _d(Iw), _d(v0), nc, _i(ia), _i(ib), _d(bases), _d(arm_a),
                                  _d(arm_b), _d(CoR), _d(mu), C.byref(gp), _d(alpha), _d(beta), _d(v2), _d(f),
                                  C.byref(gr))
    else:
        nr = None if nrel_extra is None else f64(nrel_extra)
        dr = None if drel_extra is None else f64(drel_extra)
        lib().or_sobogus_solve_3d_ex(nb, _d(m), _d(Iinv), _d(Iw), _d(v0), nc, _i(ia), _i(ib), _d(bases),
                                     _d(arm_a), _d(arm_b), _d(CoR), _d(mu), _d(nr) if nr is not None else None,
                                     _d(dr) if dr is not None else None, C.byref(gp), _d(alpha), _d(beta),
                                     _d(v2), _d(f), C.byref(gr))
    return dict(alpha=alpha, beta=beta, v2=v2, f=f, error=gr.error, iterations=gr.iterations,
                succeeded=bool(gr.succeeded))


def residual_3d(m, Iinv, Iw, v0, ia, ib, bases, arm_a, arm_b, CoR, mu, alpha, beta, nrel_extra=None,
                drel_extra=None):
    """The 3D solver's Coulomb residual of given impulses (alpha, beta), with the map's extra relative
    velocities folded into the forcing terms when given."""
    m, Iinv, Iw, v0 = f64(m), f64(Iinv), f64(Iw), f64(v0)
    bases, arm_a, arm_b = f64(bases), f64(arm_a), f64(arm_b)
    ia, ib = i32(ia), i32(ib)
    nc = ia.shape[0]
    CoR = f64(np.broadcast_to(CoR, (nc,)))
    mu = f64(np.broadcast_to(mu, (nc,)))
    a, b = f64(alpha), f64(beta)
    if nrel_extra is not None or drel_extra is not None:
        nr = None if nrel_extra is None else f64(nrel_extra)
        dr = None if drel_extra is None else f64(drel_extra)
        return lib().or_residual_3d_ex(m.shape[0], _d(m), _d(Iinv), _d(Iw), _d(v0), nc, _i(ia), _i(ib), _d(bases),
                                       _d(arm_a), _d(arm_b), _d(CoR), _d(mu), _d(nr) if nr is not None else None,
                                       _d(dr) if dr is not None else None, _d(a), _d(b))
    return lib().or_residual_3d(m.shape[0], _d(m), _d(Iinv), _d(Iw), _d(v0), nc, _i(ia), _i(ib), _d(bases),
                                _d(arm_a), _d(arm_b), _d(CoR), _d(mu), _d(a), _d(b))


class Sphere3D:
    """RigidBody3D spheres stepped by SplitHam + GeometricImpactFrictionMap + Sobogus (CPU oracle)."""

    def __init__(self, q, v, r, m, I0, plane_x, plane_n, *, dt, gravity=(0.0, 0.0, -9.81), mu=0.5,
                 CoR=0.0, tol=1e-9, max_iters=5000, eval_every=1, staggering=STAGGER_GEOMETRIC,
                 cache_mode=CACHE_NONE, stabilize=False, penetration_threshold=0.0):
        self.q, self.v = f64(q), f64(v)
        self.r, self.m, self.I0 = f64(r), f64(m), f64(I0)
        self.nb = self.r.shape[0]
        px, pn = f64(plane_x).reshape(-1), f64(plane_n).reshape(-1)
        self.np = px.shape[0] // 3
        p = Sphere3DParams(dt, (C.c_double * 3)(*gravity), mu, CoR, tol, max_iters, eval_every, staggering,
                           cache_mode, 1 if stabilize else 0, penetration_threshold)
        self._h = lib().or_sphere3d_create(self.nb, _d(self.q), _d(self.v), _d(self.r), _d(self.m),
                                           _d(self.I0), self.np, _d(px), _d(pn), C.byref(p))
        self.iteration = 0

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().or_sphere3d_destroy(h)
            self._h = None

    def step(self):
        self.iteration += 1
        st = StepStats()
        lib().or_sphere3d_step(self._h, self.iteration, C.byref(st))
        return dict(n_contacts=st.n_contacts, n_sphere_sphere=st.n_ball_ball, n_sphere_plane=st.n_ball_plane,
                    iterations=st.iterations, succeeded=bool(st.succeeded), error=st.error)

    def run(self, n_steps):
        st = StepStats()
        tot = C.c_int64(0)
        bad = lib().or_sphere3d_run(self._h, self.iteration + 1, n_steps, C.byref(st), C.byref(tot))
        self.iteration += n_steps
        return (dict(n_contacts=st.n_contacts, iterations=st.iterations, succeeded=bool(st.succeeded),
                     error=st.error), tot.value, bad)

    def state(self):
        q, v = np.zeros(12 * self.nb), np.zeros(6 * self.nb)
        lib().or_sphere3d_get_state(self._h, _d(q), _d(v))
        return q, v

    def set_state(self, q, v):
        q, v = f64(q), f64(v)
        lib().or_sphere3d_set_state(self._h, _d(q), _d(v))

    def world_inertia(self):
        Iw, Iinv = np.zeros(9 * self.nb), np.zeros(9 * self.nb)
        lib().or_sphere3d_world_inertia(self._h, _d(Iw), _d(Iinv))
        return Iw, Iinv

    def set_solver(self, tol, max_iters):
        lib().or_sphere3d_set_solver(self._h, tol, max_iters)

    def set_next_order(self, order):
        order = i32(order)
        lib().or_sphere3d_set_next_order(self._h, order.shape[0], _i(order))

    def last_contacts(self):
        L = lib()
        nc = L.or_sphere3d_last_contacts(self._h, 0, None, None, None, None, None, None, None)
        ia, ib = np.zeros(nc, np.int32), np.zeros(nc, np.int32)
        E, ra, rb = np.zeros(9 * nc), np.zeros(3 * nc), np.zeros(3 * nc)
        a, b = np.zeros(nc), np.zeros(2 * nc)
        L.or_sphere3d_last_contacts(self._h, nc, _i(ia), _i(ib), _d(E), _d(ra), _d(rb), _d(a), _d(b))
        return dict(ia=ia, ib=ib, bases=E.reshape(-1, 3, 3), arm_a=ra.reshape(-1, 3), arm_b=rb.reshape(-1, 3),
                    alpha=a, beta=b.reshape(-1, 2))

    def active_set(self, q0, q1):
        q0, q1 = f64(q0), f64(q1)
        L = lib()
        k = L.or_sphere3d_active_set(self._h, _d(q0), _d(q1), 0, None, None)
        ia, ib = np.zeros(k, np.int32), np.zeros(k, np.int32)
        L.or_sphere3d_active_set(self._h, _d(q0), _d(q1), k, _i(ia), _i(ib))
        return ia, ib

    def umap(self, q0, v0):
        q0, v0 = f64(q0), f64(v0)
        q1, v1 = np.zeros_like(q0), np.zeros_like(v0)
        lib().or_sphere3d_umap(self._h, _d(q0), _d(v0), _d(q1), _d(v1))
        return q1, v1


# ------------------------------------------------------------------ warm-start network
def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def mlp_param_count():
    return lib().or_mlp_param_count()


def mlp_forward(params, x):
    params = np.ascontiguousarray(params, dtype=np.float32)
    x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, 12)
    y = np.zeros((x.shape[0], 3))
    lib().or_mlp_forward(_fp(params), x.shape[0], _fp(x), _d(y))
    return y


def mlp_loss_grad(params, x, t):
    params = np.ascontiguousarray(params, dtype=np.float32)
    x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, 12)
    t = np.ascontiguousarray(t, dtype=np.float32).reshape(-1, 3)
    g = np.zeros(params.shape[0])
    loss = lib().or_mlp_loss_grad(_fp(params), x.shape[0], _fp(x), _fp(t), _d(g))
    return loss, g


def circle_mass_inertia(r, density):
    """CircleGeometry::computeMassAndInertia (rigidbody2d/CircleGeometry.cpp:29-33): m = rho pi r^2,
    I = 0.5 m r^2."""
    r = f64(r)
    m = density * np.pi * r * r
    return m, 0.5 * m * r * r


class RigidBody2D:
    """RigidBody2D circles stepped by GeometricImpactFrictionMap + Sobogus(RigidBody2D) (CPU oracle).
    q, v: 3 per body ([x y theta], [vx vy omega]); r, m, I per body; planes 2 each."""

    def __init__(self, q, v, r, m, I, plane_x, plane_n, *, dt, gravity=(0.0, -9.81), mu=0.5, CoR=0.0,
                 tol=1e-9, max_iters=5000, eval_every=1, integrator=SYMPLECTIC_EULER, cache_mode=CACHE_NONE,
                 staggering=STAGGER_GEOMETRIC):
        self.q, self.v = f64(q), f64(v)
        self.r, self.m, self.I = f64(r), f64(m), f64(I)
        self.nb = self.r.shape[0]
        px, pn = f64(plane_x).reshape(-1), f64(plane_n).reshape(-1)
        self.np = px.shape[0] // 2
        p = RigidBody2DParams(integrator, cache_mode, dt, (C.c_double * 2)(*gravity), mu, CoR, tol, max_iters,
                              eval_every, staggering)
        self._h = lib().or_rb2d_create(self.nb, _d(self.q), _d(self.v), _d(self.r), _d(self.m), _d(self.I),
                                       self.np, _d(px), _d(pn), C.byref(p))
        self.iteration = 0

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().or_rb2d_destroy(h)
            self._h = None

    def step(self):
        self.iteration += 1
        st = StepStats()
        lib().or_rb2d_step(self._h, self.iteration, C.byref(st))
        return dict(n_contacts=st.n_contacts, n_circle_circle=st.n_ball_ball, n_circle_plane=st.n_ball_plane,
                    iterations=st.iterations, succeeded=bool(st.succeeded), error=st.error)

    def run(self, n_steps):
        st = StepStats()
        tot = C.c_int64(0)
        bad = lib().or_rb2d_run(self._h, self.iteration + 1, n_steps, C.byref(st), C.byref(tot))
        self.iteration += n_steps
        return (dict(n_contacts=st.n_contacts, iterations=st.iterations, succeeded=bool(st.succeeded),
                     error=st.error), tot.value, bad)

    def state(self):
        q, v = np.zeros(3 * self.nb), np.zeros(3 * self.nb)
        lib().or_rb2d_get_state(self._h, _d(q), _d(v))
        return q, v

    def set_state(self, q, v):
        q, v = f64(q), f64(v)
        lib().or_rb2d_set_state(self._h, _d(q), _d(v))

    def set_solver(self, tol, max_iters):
        lib().or_rb2d_set_solver(self._h, tol, max_iters)

    def set_next_order(self, order):
        order = i32(order)
        lib().or_rb2d_set_next_order(self._h, order.shape[0], _i(order))

    def last_contacts(self):
        L = lib()
        nc = L.or_rb2d_last_contacts(self._h, 0, None, None, None, None, None, None, None)
        nc = -nc - 1 if nc < 0 else nc
        ia, ib = np.zeros(nc, np.int32), np.zeros(nc, np.int32)
        n, ta, tb, a, b = np.zeros(2 * nc), np.zeros(nc), np.zeros(nc), np.zeros(nc), np.zeros(nc)
        L.or_rb2d_last_contacts(self._h, nc, _i(ia), _i(ib), _d(n), _d(ta), _d(tb), _d(a), _d(b))
        return dict(ia=ia, ib=ib, n=n.reshape(-1, 2), ta=ta, tb=tb, alpha=a, beta=b)
