"""ctypes binding of libscisim_gb300.so (the C ABI declared in include/scisim_gpu.h).

The library is the only compute path: if it is missing or cannot be loaded, every
call raises.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libscisim_gb300.so")

SG_OK, SG_NOT_CONVERGED, SG_BAD_INPUT, SG_DEVICE_TIMEOUT, SG_CUDA_ERROR, SG_CAPACITY = range(6)
STATUS_NAMES = {0: "SG_OK", 1: "SG_NOT_CONVERGED", 2: "SG_BAD_INPUT", 3: "SG_DEVICE_TIMEOUT",
                4: "SG_CUDA_ERROR", 5: "SG_CAPACITY"}
SYMPLECTIC_EULER, VERLET, SPLIT_HAM = 0, 1, 2
CACHE_NONE, CACHE_NORMAL, CACHE_NORMAL_AND_FRICTION = 0, 1, 2
PRECISION_FP64, PRECISION_FP32_REFINE = 0, 1
STAGGER_GEOMETRIC, STAGGER_SYMPLECTIC_EULER, STAGGER_STABILIZED = 0, 1, 2

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_i64 = C.c_int64


class SgConfig(C.Structure):
    _fields_ = [("integrator", C.c_int32), ("cache_mode", C.c_int32), ("precision", C.c_int32),
                ("device", C.c_int32), ("dt", C.c_double), ("gravity", C.c_double * 3), ("mu", C.c_double),
                ("CoR", C.c_double), ("tol", C.c_double), ("max_iters", C.c_uint32),
                ("eval_every", C.c_uint32)]


class SgStepStats(C.Structure):
    _fields_ = [("n_contacts", C.c_int64), ("n_ball_ball", C.c_int64), ("n_ball_plane", C.c_int64),
                ("iterations", C.c_uint32), ("succeeded", C.c_int32), ("error", C.c_double),
                ("n_colors", C.c_uint32), ("reserved", C.c_uint32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class SgTuning(C.Structure):
    _fields_ = [("two_level", C.c_int32), ("check_interval", C.c_int32), ("two_level_min_contacts", C.c_int32),
                ("fp64_factor", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class SgProfile(C.Structure):
    _fields_ = [("gs_ms", C.c_double), ("gs_launches", C.c_uint64), ("contact_sweeps", C.c_uint64),
                ("contact_evals", C.c_uint64), ("kernel_launches", C.c_uint64), ("steps", C.c_uint64),
                ("contacts", C.c_uint64), ("contact_sweeps32", C.c_uint64), ("contact_lifts", C.c_uint64),
                ("body_lifts", C.c_uint64), ("two_level_solves", C.c_uint64), ("patch_interior_ms", C.c_double),
                ("patch_wait_ms", C.c_double), ("patch_boundary_ms", C.c_double), ("boundary_contacts", C.c_uint64),
                ("boundary_colors", C.c_uint64), ("patch_interior_max_ms", C.c_double),
                ("patch_slowest_block", C.c_int64), ("patch_contacts_staged", C.c_uint64),
                ("fp64_start_solves", C.c_uint64), ("stage_ms", C.c_double * 8)]


class SgError(RuntimeError):
    def __init__(self, status, where):
        self.status = status
        msg = lib().sg_last_error_string().decode(errors="replace") if _lib is not None else ""
        super().__init__("%s returned %s%s" % (where, STATUS_NAMES.get(status, status), (": " + msg) if msg else ""))


# Every symbol the header declares, with its ctypes signature.
SIGNATURES = {
    "sg_last_error_string": (C.c_char_p, []),
    "sg_ctx_create": (C.c_int, [C.POINTER(SgConfig), C.POINTER(C.c_void_p)]),
    "sg_ctx_destroy": (None, [C.c_void_p]),
    "sg_ctx_reconfigure": (C.c_int, [C.c_void_p, C.POINTER(SgConfig)]),
    "sg_ball2d_upload": (C.c_int, [C.c_void_p, C.c_int32, _dp, _dp, _dp, _dp, C.c_int32, _dp, _dp]),
    "sg_sphere3d_upload": (C.c_int, [C.c_void_p, C.c_int32, _dp, _dp, _dp, _dp, _dp, C.c_int32, _dp, _dp]),
    "sg_batch2d_upload": (C.c_int, [C.c_void_p, C.c_int32, _ip, _dp, _dp, _dp, _dp, _ip, _dp, _dp, _dp, _dp]),
    "sg_batch2d_scene_stats": (C.c_int, [C.c_void_p, _ip, C.POINTER(C.c_uint32), _dp, _ip]),
    "sg_batch2d_set_capacity": (C.c_int, [C.c_void_p, C.c_int32]),
    "sg_rigidbody2d_upload": (C.c_int, [C.c_void_p, C.c_int32, _dp, _dp, _dp, _dp, _dp, C.c_int32, _dp, _dp]),
    "sg_rigidbody2d_last_contacts": (_i64, [C.c_void_p, _i64, _ip, _ip, _dp, _dp, _dp, _dp, _dp]),
    "sg_sphere3d_batch_upload": (C.c_int, [C.c_void_p, C.c_int32, _ip, _dp, _dp, _dp, _dp, _dp, _ip, _dp, _dp, _dp,
                                           _dp]),
    "sg_step": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.POINTER(SgStepStats), C.POINTER(_i64)]),
    "sg_flow": (C.c_int, [C.c_void_p, C.c_uint32, _dp, _dp, _dp, _dp, C.POINTER(SgStepStats)]),
    "sg_download_state": (C.c_int, [C.c_void_p, _dp, _dp]),
    "sg_last_contacts": (_i64, [C.c_void_p, _i64, _ip, _ip, _dp, _dp, _dp]),
    "sg_sphere3d_last_contacts": (_i64, [C.c_void_p, _i64, _ip, _ip, _dp, _dp, _dp]),
    "sg_sphere3d_world_inertia": (C.c_int, [C.c_void_p, _dp, _dp]),
    "sg_last_solve_order": (_i64, [C.c_void_p, _i64, _ip, _ip, _ip]),
    "sg_sobogus_solve_2d": (C.c_int, [C.c_void_p, C.c_int32, _dp, _dp, C.c_int32, _ip, _ip, _dp, _dp, _dp,
                                      C.c_uint32, C.c_double, C.c_uint32, _dp, _dp, _dp, _dp, _dp,
                                      C.POINTER(C.c_uint32)]),
    "sg_sobogus_solve_2d_ex": (C.c_int, [C.c_void_p, C.c_int32, _dp, _dp, C.c_int32, _ip, _ip, _dp, _dp, _dp, _dp,
                                         _dp, C.c_uint32, C.c_double, C.c_uint32, _dp, _dp, _dp, _dp, _dp,
                                         C.POINTER(C.c_uint32)]),
    "sg_sobogus_solve_3d": (C.c_int, [C.c_void_p, C.c_int32, _dp, _dp, _dp, _dp, C.c_int32, _ip, _ip, _dp, _dp, _dp,
                                      _dp, _dp, _dp, _dp, C.c_uint32, C.c_double, C.c_uint32, _dp, _dp, _dp, _dp, _dp,
                                      C.POINTER(C.c_uint32)]),
    "sg_sobogus_solve_2d_noalloc": (C.c_int, [C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p,
                                              C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_double,
                                              C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                              C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_uint32)]),
    "sg_broadphase_2d": (C.c_int, [C.c_void_p, C.c_int32, _dp, _i64, _ip, C.POINTER(_i64)]),
    "sg_ccd_2d": (C.c_int, [C.c_void_p, C.c_int32, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _ip, _dp]),
    "sg_mlp_param_count": (C.c_int, []),
    "sg_mlp_load": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_int32]),
    "sg_mlp_enable": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "sg_mlp_last_samples": (_i64, [C.c_void_p, _i64, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "sg_mlp_train": (C.c_int, [C.c_void_p, _i64, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int32, C.c_int32,
                               C.c_float, C.c_uint64, C.POINTER(C.c_float), _dp]),
    "sg_mlp_grad": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_int32, C.POINTER(C.c_float),
                              C.POINTER(C.c_float), C.POINTER(C.c_float), _dp]),
    "sg_mlp_infer": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_int32, C.POINTER(C.c_float),
                               C.POINTER(C.c_float), C.c_int32]),
    "sg_mlp_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "sg_profile_enable": (C.c_int, [C.c_void_p, C.c_int32]),
    "sg_profile_read": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32]),
    "sg_set_two_level": (C.c_int, [C.c_void_p, C.c_int32]),
    "sg_set_fp64_pairs": (C.c_int, [C.c_void_p, C.c_int32]),
    "sg_set_staggering": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_double]),
    "sg_get_tuning": (C.c_int, [C.c_void_p, C.c_void_p]),
    "sg_set_tuning": (C.c_int, [C.c_void_p, C.c_void_p]),
    "sg_autotune": (C.c_int, [C.c_void_p, C.c_int32, C.c_uint32, C.c_void_p, _dp]),
    "sg_checkpoint_size": (_i64, [C.c_void_p]),
    "sg_checkpoint_save": (C.c_int, [C.c_void_p, C.c_void_p, _i64]),
    "sg_checkpoint_load": (C.c_int, [C.c_void_p, C.c_void_p, _i64]),
    "sg_last_patch_layout": (C.c_int, [C.c_void_p, _i64, _i64, _ip, _ip, _ip, _ip, _ip, _ip]),
    "sg_ctx_stream": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "sg_set_spin_limit": (C.c_int, [C.c_void_p, C.c_uint64]),
    "sg_selftest_wait_timeout": (C.c_int, [C.c_void_p]),
}

_lib = None


def lib():
    """Loads the library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libscisim_gb300.so is not built (run __graft_entry__.build()); "
                               "there is no CPU fallback")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status, where):
    if status not in (SG_OK, SG_NOT_CONVERGED):
        raise SgError(status, where)
    return status


def dptr(a):
    return a.ctypes.data_as(_dp)


def iptr(a):
    return a.ctypes.data_as(_ip)


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def mlp_param_count():
    return lib().sg_mlp_param_count()


def mlp_init(seed=0):
    """Initial network parameters (scaled normal weights, zero biases), packed as the C ABI
    expects: W1 (64x12), b1, W2 (64x64), b2, W3 (3x64), b3."""
    rng = np.random.default_rng(seed)
    parts = []
    for fan_in, fan_out in ((12, 64), (64, 64), (64, 3)):
        parts.append(rng.normal(0.0, (2.0 / (fan_in + fan_out)) ** 0.5, (fan_out, fan_in)).reshape(-1))
        parts.append(np.zeros(fan_out))
    p = np.concatenate(parts).astype(np.float32)
    assert p.shape[0] == mlp_param_count()
    return p


def _g3(gravity):
    g = tuple(float(x) for x in gravity)
    if not 2 <= len(g) <= 3:
        raise ValueError("gravity has 2 (Ball2D) or 3 (RigidBody3D) components")
    return (C.c_double * 3)(*(g + (0.0,) * (3 - len(g))))


class Context:
    """Owns one sg_ctx (device memory, stream, impulse cache)."""

    def __init__(self, *, dt=0.01, gravity=(0.0, -9.81), mu=0.5, CoR=0.0, tol=1e-9, max_iters=5000,
                 eval_every=1, integrator=SYMPLECTIC_EULER, cache_mode=CACHE_NONE,
                 precision=PRECISION_FP64, device=0):
        self.config = SgConfig(integrator, cache_mode, precision, device, dt, _g3(gravity), mu,
                               CoR, tol, max_iters, eval_every)
        h = C.c_void_p()
        check(lib().sg_ctx_create(C.byref(self.config), C.byref(h)), "sg_ctx_create")
        self._h = h
        self.nb = 0
        self.dim = 2
        self.rb2d = False

    @property
    def handle(self):
        return self._h

    def reconfigure(self, **changes):
        """New solver settings on the same scene and impulse cache."""
        c = self.config
        fields = {k: getattr(c, k) for k, _ in SgConfig._fields_}
        fields["gravity"] = tuple(c.gravity)
        fields.update(changes)
        cfg = SgConfig(fields["integrator"], fields["cache_mode"], fields["precision"], fields["device"],
                       fields["dt"], _g3(fields["gravity"]), fields["mu"], fields["CoR"],
                       fields["tol"], fields["max_iters"], fields["eval_every"])
        check(lib().sg_ctx_reconfigure(self._h, C.byref(cfg)), "sg_ctx_reconfigure")
        self.config = cfg

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().sg_ctx_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- scene ---------------------------------------------------------------
    def upload_ball2d(self, q, v, r, m, plane_x, plane_n):
        q, v, r, m = f64(q).reshape(-1), f64(v).reshape(-1), f64(r).reshape(-1), f64(m).reshape(-1)
        px, pn = f64(plane_x).reshape(-1), f64(plane_n).reshape(-1)
        self.nb = r.shape[0]
        self.dim = 2
        self.rb2d = False
        self._keep = (q, v, r, m, px, pn)
        check(lib().sg_ball2d_upload(self._h, self.nb, dptr(q), dptr(v), dptr(r), dptr(m), px.shape[0] // 2,
                                     dptr(px), dptr(pn)), "sg_ball2d_upload")

    def upload_batch2d(self, body_off, q, v, r, m, plane_off, plane_x, plane_n, mu, CoR):
        """Independent Ball2D scenes stepped together (global body and plane indices)."""
        bo, po = i32(body_off).reshape(-1), i32(plane_off).reshape(-1)
        q, v, r, m = f64(q).reshape(-1), f64(v).reshape(-1), f64(r).reshape(-1), f64(m).reshape(-1)
        px, pn = f64(plane_x).reshape(-1), f64(plane_n).reshape(-1)
        mu, CoR = f64(mu).reshape(-1), f64(CoR).reshape(-1)
        S = bo.shape[0] - 1
        if po.shape[0] != S + 1 or mu.shape[0] != S or CoR.shape[0] != S or r.shape[0] != bo[-1]:
            raise ValueError("inconsistent batch sizes")
        self.nb = r.shape[0]
        self.dim = 2
        self.rb2d = False
        self.n_scenes = S
        self._keep = (bo, po, q, v, r, m, px, pn, mu, CoR)
        check(lib().sg_batch2d_upload(self._h, S, iptr(bo), dptr(q), dptr(v), dptr(r), dptr(m), iptr(po), dptr(px),
                                      dptr(pn), dptr(mu), dptr(CoR)), "sg_batch2d_upload")

    def upload_sphere3d_batch(self, body_off, q, v, r, m, I0, plane_off, plane_x, plane_n, mu, CoR):
        """Independent sphere scenes stepped together: q = [x (3N) | R (9N)], v = [v (3N) | w (3N)]
        over all bodies, global body and plane indices."""
        bo, po = i32(body_off).reshape(-1), i32(plane_off).reshape(-1)
        q, v, r, m = f64(q).reshape(-1), f64(v).reshape(-1), f64(r).reshape(-1), f64(m).reshape(-1)
        I0, px, pn = f64(I0).reshape(-1), f64(plane_x).reshape(-1), f64(plane_n).reshape(-1)
        mu, CoR = f64(mu).reshape(-1), f64(CoR).reshape(-1)
        S = bo.shape[0] - 1
        N = int(bo[-1])
        if (po.shape[0] != S + 1 or mu.shape[0] != S or CoR.shape[0] != S or r.shape[0] != N or
                q.shape[0] != 12 * N or v.shape[0] != 6 * N or I0.shape[0] != 3 * N):
            raise ValueError("inconsistent batch sizes")
        self.nb = N
        self.dim = 3
        self.rb2d = False
        self.n_scenes = S
        self._keep = (bo, po, q, v, r, m, I0, px, pn, mu, CoR)
        check(lib().sg_sphere3d_batch_upload(self._h, S, iptr(bo), dptr(q), dptr(v), dptr(r), dptr(m), dptr(I0),
                                             iptr(po), dptr(px), dptr(pn), dptr(mu), dptr(CoR)),
              "sg_sphere3d_batch_upload")

    def batch_set_capacity(self, contacts):
        check(lib().sg_batch2d_set_capacity(self._h, int(contacts)), "sg_batch2d_set_capacity")

    def batch_scene_stats(self):
        S = self.n_scenes
        nc, it = np.empty(S, np.int32), np.empty(S, np.uint32)
        err, ok = np.empty(S), np.empty(S, np.int32)
        check(lib().sg_batch2d_scene_stats(self._h, iptr(nc), it.ctypes.data_as(C.POINTER(C.c_uint32)), dptr(err),
                                           iptr(ok)), "sg_batch2d_scene_stats")
        return dict(n_contacts=nc, iterations=it, error=err, succeeded=ok.astype(bool))

    def upload_rigidbody2d(self, q, v, r, m, I, plane_x, plane_n):
        """RigidBody2D circles: q, v 3 per body ([x y theta], [vx vy omega]), r, m, I per body."""
        q, v, r, m, I = f64(q).reshape(-1), f64(v).reshape(-1), f64(r).reshape(-1), f64(m).reshape(-1), f64(I).reshape(-1)
        px, pn = f64(plane_x).reshape(-1), f64(plane_n).reshape(-1)
        nb = r.shape[0]
        if q.shape[0] != 3 * nb or v.shape[0] != 3 * nb or m.shape[0] != nb or I.shape[0] != nb:
            raise ValueError("inconsistent RigidBody2D state sizes")
        self.nb = nb
        self.dim = 2
        self.rb2d = True
        self._keep = (q, v, r, m, I, px, pn)
        check(lib().sg_rigidbody2d_upload(self._h, nb, dptr(q), dptr(v), dptr(r), dptr(m), dptr(I),
                                          px.shape[0] // 2, dptr(px), dptr(pn)), "sg_rigidbody2d_upload")

    def rigidbody2d_last_contacts(self):
        L = lib()
        nc = L.sg_rigidbody2d_last_contacts(self._h, 0, None, None, None, None, None, None, None)
        nc = -nc - 1 if nc < 0 else nc
        ia, ib = np.empty(nc, np.int32), np.empty(nc, np.int32)
        n, ta, tb = np.empty(2 * nc), np.empty(nc), np.empty(nc)
        a, b = np.empty(nc), np.empty(nc)
        got = L.sg_rigidbody2d_last_contacts(self._h, nc, iptr(ia), iptr(ib), dptr(n), dptr(ta), dptr(tb), dptr(a),
                                              dptr(b))
        if got != nc:
            raise SgError(SG_BAD_INPUT, "sg_rigidbody2d_last_contacts")
        return dict(ia=ia, ib=ib, n=n.reshape(-1, 2), ta=ta, tb=tb, alpha=a, beta=b)

    def upload_sphere3d(self, q, v, r, m, I0, plane_x, plane_n):
        """RigidBody3D spheres: q 12nb [x | R row-major], v 6nb [v | omega], r, m, I0 (3 per body)."""
        q, v, r, m = f64(q).reshape(-1), f64(v).reshape(-1), f64(r).reshape(-1), f64(m).reshape(-1)
        I0 = f64(I0).reshape(-1)
        px, pn = f64(plane_x).reshape(-1), f64(plane_n).reshape(-1)
        nb = r.shape[0]
        if q.shape[0] != 12 * nb or v.shape[0] != 6 * nb or m.shape[0] != nb or I0.shape[0] != 3 * nb:
            raise ValueError("inconsistent RigidBody3D state sizes")
        self.nb = nb
        self.dim = 3
        self.rb2d = False
        self._keep = (q, v, r, m, I0, px, pn)
        check(lib().sg_sphere3d_upload(self._h, nb, dptr(q), dptr(v), dptr(r), dptr(m), dptr(I0), px.shape[0] // 3,
                                       dptr(px), dptr(pn)), "sg_sphere3d_upload")

    def step(self, n_steps=1, first_iteration=1):
        st = SgStepStats()
        tot = _i64(0)
        s = check(lib().sg_step(self._h, first_iteration, n_steps, C.byref(st), C.byref(tot)), "sg_step")
        d = st.as_dict()
        d["total_contacts"] = tot.value
        d["status"] = s
        return d

    def flow(self, iteration, q0, v0, q1=None, v1=None):
        q0, v0 = f64(q0), f64(v0)
        q1 = np.empty_like(q0) if q1 is None else q1
        v1 = np.empty_like(v0) if v1 is None else v1
        st = SgStepStats()
        s = check(lib().sg_flow(self._h, iteration, dptr(q0), dptr(v0), dptr(q1), dptr(v1), C.byref(st)),
                  "sg_flow")
        d = st.as_dict()
        d["status"] = s
        return q1, v1, d

    def state(self):
        q = np.empty((12 if self.dim == 3 else 3 if self.rb2d else 2) * self.nb)
        v = np.empty((6 if self.dim == 3 else 3 if self.rb2d else 2) * self.nb)
        check(lib().sg_download_state(self._h, dptr(q), dptr(v)), "sg_download_state")
        return q, v

    def last_contacts(self):
        L = lib()
        nc = L.sg_last_contacts(self._h, 0, None, None, None, None, None)
        nc = -nc - 1 if nc < 0 else nc
        ia, ib = np.empty(nc, np.int32), np.empty(nc, np.int32)
        n, a, b = np.empty(2 * nc), np.empty(nc), np.empty(nc)
        got = L.sg_last_contacts(self._h, nc, iptr(ia), iptr(ib), dptr(n), dptr(a), dptr(b))
        if got != nc:
            raise SgError(SG_CUDA_ERROR, "sg_last_contacts")
        return dict(ia=ia, ib=ib, n=n.reshape(-1, 2), alpha=a, beta=b)

    def sphere3d_last_contacts(self):
        L = lib()
        nc = L.sg_sphere3d_last_contacts(self._h, 0, None, None, None, None, None)
        nc = -nc - 1 if nc < 0 else nc
        ia, ib = np.empty(nc, np.int32), np.empty(nc, np.int32)
        E, a, b = np.empty(9 * nc), np.empty(nc), np.empty(2 * nc)
        got = L.sg_sphere3d_last_contacts(self._h, nc, iptr(ia), iptr(ib), dptr(E), dptr(a), dptr(b))
        if got != nc:
            raise SgError(SG_CUDA_ERROR, "sg_sphere3d_last_contacts")
        return dict(ia=ia, ib=ib, bases=E.reshape(-1, 3, 3), alpha=a, beta=b.reshape(-1, 2))

    def sphere3d_world_inertia(self):
        Iw, Iinv = np.empty(9 * self.nb), np.empty(9 * self.nb)
        check(lib().sg_sphere3d_world_inertia(self._h, dptr(Iw), dptr(Iinv)), "sg_sphere3d_world_inertia")
        return Iw, Iinv

    def last_solve_order(self):
        L = lib()
        nc = L.sg_last_solve_order(self._h, 0, None, None, None)
        nc = -nc - 1 if nc < 0 else nc
        order = np.empty(nc, np.int32)
        offs = np.empty(65, np.int32)
        ncol = C.c_int32(0)
        L.sg_last_solve_order(self._h, nc, iptr(order), iptr(offs), C.byref(ncol))
        return order, offs[: ncol.value + 1].copy()

    # -- learned warm start ------------------------------------------------------
    def mlp_load(self, params):
        params = f32(params)
        check(lib().sg_mlp_load(self._h, fptr(params), params.shape[0]), "sg_mlp_load")

    def mlp_enable(self, warm_start=True, record=False):
        check(lib().sg_mlp_enable(self._h, 1 if warm_start else 0, 1 if record else 0), "sg_mlp_enable")

    def mlp_last_samples(self):
        L = lib()
        n = L.sg_mlp_last_samples(self._h, 0, None, None)
        if n == -(2 ** 63):
            raise SgError(SG_BAD_INPUT, "sg_mlp_last_samples")
        n = -n - 1 if n < 0 else n
        x, t = np.empty((n, 12), np.float32), np.empty((n, 3), np.float32)
        got = L.sg_mlp_last_samples(self._h, n, fptr(x), fptr(t))
        if got != n:
            raise SgError(SG_CUDA_ERROR, "sg_mlp_last_samples")
        return x, t

    def mlp_train(self, x, t, params, epochs=5, batch=4096, lr=1e-3, seed=0):
        x, t = f32(x).reshape(-1, 12), f32(t).reshape(-1, 3)
        p = f32(params).copy()
        losses = np.zeros(epochs)
        check(lib().sg_mlp_train(self._h, x.shape[0], fptr(x), fptr(t), epochs, batch, lr, seed, fptr(p),
                                 dptr(losses)), "sg_mlp_train")
        return p, losses

    def mlp_grad(self, params, x, t):
        params, x, t = f32(params), f32(x).reshape(-1, 12), f32(t).reshape(-1, 3)
        g = np.zeros(params.shape[0], np.float32)
        loss = C.c_double(0.0)
        check(lib().sg_mlp_grad(self._h, fptr(params), x.shape[0], fptr(x), fptr(t), fptr(g), C.byref(loss)),
              "sg_mlp_grad")
        return loss.value, g

    def mlp_infer(self, params, x, tensor_cores=True):
        params, x = f32(params), f32(x).reshape(-1, 12)
        y = np.zeros((x.shape[0], 3), np.float32)
        check(lib().sg_mlp_infer(self._h, fptr(params), x.shape[0], fptr(x), fptr(y), 1 if tensor_cores else 0),
              "sg_mlp_infer")
        return y

    def mlp_stats(self):
        a, b = C.c_uint64(0), C.c_uint64(0)
        check(lib().sg_mlp_stats(self._h, C.byref(a), C.byref(b)), "sg_mlp_stats")
        return dict(evaluated=a.value, network_start=b.value)

    def profile_enable(self, on=True):
        check(lib().sg_profile_enable(self._h, 1 if on else 0), "sg_profile_enable")

    def profile_read(self, reset=False):
        p = SgProfile()
        check(lib().sg_profile_read(self._h, C.byref(p), 1 if reset else 0), "sg_profile_read")
        d = {k: getattr(p, k) for k, _ in p._fields_}
        d["stage_ms"] = list(p.stage_ms)
        return d

    def set_two_level(self, on=True):
        """0 / False: one-level sweeps; 1 / True (default): two-level FP32 sweeps, and for a solve the
        FP64 probe leaves near tol up to 160 one-level FP64 sweeps before two-level ones; 2: two-level
        FP64 sweeps for such a solve from the start."""
        check(lib().sg_set_two_level(self._h, int(on)), "sg_set_two_level")

    def set_fp64_pairs(self, on=True):
        """The FP32 form's FP64 sweeps after the probe for discs (one-level and two-level) in
        float-float pairs (True, default) or in FP64 (False)."""
        check(lib().sg_set_fp64_pairs(self._h, int(on)), "sg_set_fp64_pairs")

    def set_staggering(self, staggering=STAGGER_GEOMETRIC, stabilize=False, penetration_threshold=0.0):
        """GeometricImpactFrictionMap (default), SymplecticEulerImpactFrictionMap or
        StabilizedImpactFrictionMap for this Ball2D scene."""
        check(lib().sg_set_staggering(self._h, int(staggering), 1 if stabilize else 0, float(penetration_threshold)),
              "sg_set_staggering")

    def tuning(self):
        t = SgTuning()
        check(lib().sg_get_tuning(self._h, C.byref(t)), "sg_get_tuning")
        return t.as_dict()

    def set_tuning(self, **changes):
        t = SgTuning(**{**self.tuning(), **changes})
        check(lib().sg_set_tuning(self._h, C.byref(t)), "sg_set_tuning")

    def autotune(self, trial_steps=3, first_iteration=1):
        """Times each candidate tuning from the current state, keeps the fastest (sg_autotune).
        Returns (chosen tuning, ms per step of the 6 candidates, NaN where not applicable)."""
        best = SgTuning()
        ms = np.full(6, np.nan)
        check(lib().sg_autotune(self._h, trial_steps, first_iteration, C.byref(best), dptr(ms)), "sg_autotune")
        return best.as_dict(), ms

    def checkpoint(self):
        """The context's settings, scene and impulse cache as bytes (sg_checkpoint_save)."""
        n = lib().sg_checkpoint_size(self._h)
        if n < 0:
            raise SgError(SG_BAD_INPUT, "sg_checkpoint_size")
        buf = C.create_string_buffer(int(n))
        check(lib().sg_checkpoint_save(self._h, buf, n), "sg_checkpoint_save")
        return buf.raw

    def restore(self, data):
        """Replaces settings, scene and impulse cache with a checkpoint's (sg_checkpoint_load)."""
        data = bytes(data)
        check(lib().sg_checkpoint_load(self._h, data, len(data)), "sg_checkpoint_load")
        # Header: magic[8], version, dim, nb, np (int32), prev_n (int64), sg_config.
        _, dim, nb, _ = np.frombuffer(data, np.int32, 4, 8)
        self.dim, self.nb = int(dim), int(nb)
        cfg = SgConfig.from_buffer_copy(data, 32)
        cfg.device = self.config.device
        self.config = cfg

    def patch_layout(self, nc, nb):
        """Layout of the last two-level solve: patches P, shifted tiles Pb, each contact's group
        and colour, each body's patch, shifted tile and band flag."""
        counts = np.zeros(2, np.int32)
        group = np.zeros(nc, np.int32)
        color = np.zeros(nc, np.int32)
        bp = np.zeros(nb, np.int32)
        bt = np.zeros(nb, np.int32)
        band = np.zeros(nb, np.int32)
        check(lib().sg_last_patch_layout(self._h, nc, nb, iptr(counts), iptr(group), iptr(color), iptr(bp),
                                         iptr(bt), iptr(band)), "sg_last_patch_layout")
        return {"P": int(counts[0]), "Pb": int(counts[1]), "group": group, "color": color, "body_patch": bp,
                "body_tile": bt, "body_band": band}

    def stream_ptr(self):
        s = C.c_void_p()
        check(lib().sg_ctx_stream(self._h, C.byref(s)), "sg_ctx_stream")
        return s.value or 0

    def set_spin_limit(self, spins):
        check(lib().sg_set_spin_limit(self._h, spins), "sg_set_spin_limit")

    def selftest_wait_timeout(self):
        return lib().sg_selftest_wait_timeout(self._h)

    # -- standalone entry points ----------------------------------------------
    def sobogus_solve_2d(self, m, v0, ia, ib, bases, CoR, mu, tol, max_iters, eval_every=1, alpha=None,
                         beta=None, nrel_extra=None, drel_extra=None):
        """FrictionSolver::solve for Ball2D (sg_sobogus_solve_2d; with nrel_extra / drel_extra, one per
        contact, sg_sobogus_solve_2d_ex)."""
        m, v0, bases = f64(m), f64(v0), f64(bases)
        ia, ib = i32(ia), i32(ib)
        nc, nb = ia.shape[0], m.shape[0]
        CoR = f64(np.broadcast_to(CoR, (nc,)))
        mu = f64(np.broadcast_to(mu, (nc,)))
        alpha = np.zeros(nc) if alpha is None else f64(alpha).copy()
        beta = np.zeros(nc) if beta is None else f64(beta).copy()
        v2, f = np.zeros(2 * nb), np.zeros(2 * nb)
        err = C.c_double(0.0)
        its = C.c_uint32(0)
        if nrel_extra is None and drel_extra is None:
            s = check(lib().sg_sobogus_solve_2d(self._h, nb, dptr(m), dptr(v0), nc, iptr(ia), iptr(ib), dptr(bases),
                                                dptr(CoR), dptr(mu), max_iters, tol, eval_every, dptr(alpha),
                                                dptr(beta), dptr(v2), dptr(f), C.byref(err), C.byref(its)),
                      "sg_sobogus_solve_2d")
        else:
            nr = None if nrel_extra is None else f64(nrel_extra).reshape(-1)
            dr = None if drel_extra is None else f64(drel_extra).reshape(-1)
            if (nr is not None and nr.shape[0] != nc) or (dr is not None and dr.shape[0] != nc):
                raise ValueError("nrel_extra and drel_extra take one value per contact")
            s = check(lib().sg_sobogus_solve_2d_ex(self._h, nb, dptr(m), dptr(v0), nc, iptr(ia), iptr(ib),
                                                   dptr(bases), dptr(CoR), dptr(mu), dptr(nr) if nr is not None
                                                   else None, dptr(dr) if dr is not None else None, max_iters, tol,
                                                   eval_every, dptr(alpha), dptr(beta), dptr(v2), dptr(f),
                                                   C.byref(err), C.byref(its)), "sg_sobogus_solve_2d_ex")
        return dict(alpha=alpha, beta=beta, v2=v2, f=f, error=err.value, iterations=its.value,
                    succeeded=(s == SG_OK))

    def sobogus_solve_3d(self, m, Iw, Iinv, v0, ia, ib, bases, arm_a, arm_b, CoR, mu, tol, max_iters, eval_every=1,
                         alpha=None, beta=None, nrel_extra=None, drel_extra=None):
        """FrictionSolver::solve for RigidBody3D spheres (sg_sobogus_solve_3d): m (nb), Iw, Iinv (9 per body),
        v0 (6nb, [v | omega]); bases (9 per contact, column-major [n s t]), arms (3 per contact)."""
        m, Iw, Iinv, v0 = f64(m), f64(Iw).reshape(-1), f64(Iinv).reshape(-1), f64(v0).reshape(-1)
        bases, arm_a, arm_b = f64(bases).reshape(-1), f64(arm_a).reshape(-1), f64(arm_b).reshape(-1)
        ia, ib = i32(ia), i32(ib)
        nc, nb = ia.shape[0], m.shape[0]
        CoR = f64(np.broadcast_to(CoR, (nc,)))
        mu = f64(np.broadcast_to(mu, (nc,)))
        alpha = np.zeros(nc) if alpha is None else f64(alpha).copy()
        beta = np.zeros(2 * nc) if beta is None else f64(beta).reshape(-1).copy()
        nr = None if nrel_extra is None else f64(nrel_extra).reshape(-1)
        dr = None if drel_extra is None else f64(drel_extra).reshape(-1)
        if (Iw.shape[0] != 9 * nb or Iinv.shape[0] != 9 * nb or v0.shape[0] != 6 * nb or bases.shape[0] != 9 * nc or
                arm_a.shape[0] != 3 * nc or arm_b.shape[0] != 3 * nc or beta.shape[0] != 2 * nc or
                (nr is not None and nr.shape[0] != nc) or (dr is not None and dr.shape[0] != 2 * nc)):
            raise ValueError("inconsistent RigidBody3D solve sizes")
        v2, f = np.zeros(6 * nb), np.zeros(6 * nb)
        err = C.c_double(0.0)
        its = C.c_uint32(0)
        s = check(lib().sg_sobogus_solve_3d(self._h, nb, dptr(m), dptr(Iw), dptr(Iinv), dptr(v0), nc, iptr(ia),
                                            iptr(ib), dptr(bases), dptr(arm_a), dptr(arm_b), dptr(CoR), dptr(mu),
                                            dptr(nr) if nr is not None else None,
                                            dptr(dr) if dr is not None else None, max_iters, tol, eval_every,
                                            dptr(alpha), dptr(beta), dptr(v2), dptr(f), C.byref(err),
                                            C.byref(its)), "sg_sobogus_solve_3d")
        return dict(alpha=alpha, beta=beta, v2=v2, f=f, error=err.value, iterations=its.value,
                    succeeded=(s == SG_OK))

    def broadphase_2d(self, aabb):
        aabb = f64(aabb).reshape(-1, 4)
        n = aabb.shape[0]
        tot = _i64(0)
        cap = 8 * n + 16
        while True:
            out = np.empty((cap, 2), np.int32)
            s = lib().sg_broadphase_2d(self._h, n, dptr(aabb), cap, iptr(out), C.byref(tot))
            if s == SG_CAPACITY and tot.value > cap:
                cap = tot.value
                continue
            check(s, "sg_broadphase_2d")
            return out[: tot.value].copy()

    def ccd_2d(self, q0a, q1a, ra, q0b, q1b, rb):
        arrs = [f64(x).reshape(-1) for x in (q0a, q1a, ra, q0b, q1b, rb)]
        n = arrs[2].shape[0]
        coeffs, hit, t = np.empty(3 * n), np.empty(n, np.int32), np.empty(n)
        check(lib().sg_ccd_2d(self._h, n, *[dptr(a) for a in arrs], dptr(coeffs), iptr(hit), dptr(t)),
              "sg_ccd_2d")
        return coeffs.reshape(-1, 3), hit.astype(bool), t
