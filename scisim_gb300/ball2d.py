"""SCISim's Ball2D plugin interfaces on the GB300 library.

Mirrors the reference's operator/plugin API for the contact path so that a SCISim
driver loop reads the same:

    sim = Ball2DSim(Ball2DState(q, v, r, m, [StaticPlane(x, n), ...]), gravity=(0, -9.81))
    umap = SymplecticEulerMap()                       # ball2d/SymplecticEulerMap.h
    solver = Sobogus(SobogusSolverType.Balls2D, 1)    # scisim/ConstrainedMaps/Sobogus.h
    ifmap = GeometricImpactFrictionMap(1e-9, 5000, ImpulsesToCache.NONE)
    for it in range(1, n + 1):
        sim.flow(it, dt, umap, CoR, mu, solver, ifmap)   # ball2d/Ball2DSim.cpp:305-326

Every step runs entirely on the GPU (predictor, broad and narrow phase, contact
assembly, coloured block Gauss-Seidel, impulse cache, final map); the host only
moves (q, v) in and out, exactly like the reference's ImpactFrictionMap::flow
signature (scisim/ConstrainedMaps/ImpactFrictionMap.h:36).
"""
from __future__ import annotations

import enum
import itertools

import numpy as np

from . import _lib


class ImpulsesToCache(enum.IntEnum):
    """scisim/ConstrainedMaps/ImpulsesToCache.h"""
    NONE = _lib.CACHE_NONE
    NORMAL = _lib.CACHE_NORMAL
    NORMAL_AND_FRICTION = _lib.CACHE_NORMAL_AND_FRICTION


class SobogusSolverType(enum.Enum):
    """scisim/ConstrainedMaps/Sobogus.h (RigidBody2D is not built here)."""
    Balls2D = "balls_2d"
    RigidBodies3D = "rigid_bodies_3d"


class UnconstrainedMap:
    """scisim/UnconstrainedMaps/UnconstrainedMap.h:13-43"""
    integrator = None

    def name(self) -> str:
        raise NotImplementedError


class SymplecticEulerMap(UnconstrainedMap):
    """ball2d/SymplecticEulerMap.cpp:21-32 (executed on the GPU inside each step)."""
    integrator = _lib.SYMPLECTIC_EULER

    def name(self):
        return "symplectic_euler"


class VerletMap(UnconstrainedMap):
    """ball2d/VerletMap.cpp:15-41 (executed on the GPU inside each step)."""
    integrator = _lib.VERLET

    def name(self):
        return "verlet"


class FrictionSolver:
    """scisim/ConstrainedMaps/FrictionSolver.h:16-40"""

    def numFrictionImpulsesPerNormal(self, ambient_space_dimensions: int) -> int:
        raise NotImplementedError


class Sobogus(FrictionSolver):
    """Sobogus FrictionSolver (scisim/ConstrainedMaps/Sobogus.cpp:862-1096) on the GPU.

    precision: "fp64" (plain method) or "fp32_refine" (FP32 sweeps, FP64 residual
    and closing FP64 refinement).
    """

    def __init__(self, solver_type=SobogusSolverType.Balls2D, eval_every: int = 1, precision: str = "fp64",
                 device: int = 0):
        if solver_type not in (SobogusSolverType.Balls2D, SobogusSolverType.RigidBodies3D):
            raise ValueError("SobogusSolverType.RigidBody2D is not available")
        if eval_every < 1:
            raise ValueError("eval_every must be positive")
        self.solver_type = solver_type
        self.eval_every = int(eval_every)
        self.precision = {"fp64": _lib.PRECISION_FP64, "fp32_refine": _lib.PRECISION_FP32_REFINE}[precision]
        self.device = device
        self._ctx = None

    def name(self):
        return "sobogus"

    def numFrictionImpulsesPerNormal(self, ambient_space_dimensions):
        dim = 2 if self.solver_type == SobogusSolverType.Balls2D else 3
        if ambient_space_dimensions != dim:
            raise ValueError("solver type %s is %dD" % (self.solver_type.value, dim))
        return dim - 1

    def solve(self, M_diag, v0, body_a, body_b, contact_bases, CoR, mu, max_iters, tol, alpha, beta):
        """FrictionSolver::solve (Sobogus.cpp:880-1088) for Ball2D contacts.

        M_diag: per-body masses; v0: 2nb; body_a/body_b: contact bodies (-1 = static);
        contact_bases: 2 x 2nc matrix [n0 t0 n1 t1 ...] as SCISim builds it; alpha/beta
        are the warm start, updated in place.  Returns (f, v2, solve_succeeded, error).
        """
        if self.solver_type != SobogusSolverType.Balls2D:
            raise ValueError("the standalone solve takes Balls2D contacts; sphere scenes solve inside each step")
        if self._ctx is None:
            self._ctx = _lib.Context(precision=self.precision, device=self.device)
        B = np.asarray(contact_bases, dtype=np.float64)
        nc = len(body_a)
        bases = np.ascontiguousarray(B.reshape(2, 2 * nc).T.reshape(nc, 2, 2).reshape(-1))  # column-major blocks
        res = self._ctx.sobogus_solve_2d(M_diag, v0, body_a, body_b, bases, CoR, mu, tol, max_iters,
                                         self.eval_every, alpha, beta)
        alpha[...] = res["alpha"]
        beta[...] = res["beta"]
        return res["f"], res["v2"], res["succeeded"], res["error"]


class GeometricImpactFrictionMap:
    """scisim/ConstrainedMaps/GeometricImpactFrictionMap.cpp:267-442 on the GPU."""

    def __init__(self, abs_tol: float, max_iters: int, impulses_to_cache=ImpulsesToCache.NONE):
        if abs_tol < 0.0:
            raise ValueError("abs_tol must be non-negative")
        self.abs_tol = float(abs_tol)
        self.max_iters = int(max_iters)
        self.impulses_to_cache = ImpulsesToCache(impulses_to_cache)
        self._ctx = None
        self._key = None
        self.last_stats = None

    def name(self):
        return "geometric_impact_friction_map"

    def resetCachedData(self):
        self._ctx = None
        self._key = None

    def _context(self, sim, umap, solver, dt, CoR, mu):
        key = (sim.nbodies, sim.system_id, umap.integrator, solver.eval_every, solver.precision, float(dt), float(CoR),
               float(mu), tuple(sim.gravity))
        if self._ctx is None or key != self._key:
            self._ctx = _lib.Context(dt=dt, gravity=sim.gravity, mu=mu, CoR=CoR, tol=self.abs_tol,
                                     max_iters=self.max_iters, eval_every=solver.eval_every,
                                     integrator=umap.integrator, cache_mode=int(self.impulses_to_cache),
                                     precision=solver.precision, device=solver.device)
            sim.upload(self._ctx)
            self._key = key
        return self._ctx

    def flow(self, sim, umap, friction_solver, iteration, dt, CoR, mu, q0, v0):
        """ImpactFrictionMap::flow: returns (q1, v1) from (q0, v0); host buffers in and out."""
        ctx = self._context(sim, umap, friction_solver, dt, CoR, mu)
        q1, v1, st = ctx.flow(iteration, q0, v0)
        self.last_stats = st
        if not st["succeeded"] and st["n_contacts"] > 0:
            # GeometricImpactFrictionMap.cpp:346-350 warns and continues with the best iterate.
            pass
        return q1, v1

    def last_contacts(self):
        if self._ctx is None:
            return None
        return self._ctx.sphere3d_last_contacts() if self._ctx.dim == 3 else self._ctx.last_contacts()


class SymplecticEulerImpactFrictionMap(GeometricImpactFrictionMap):
    """scisim/ConstrainedMaps/SymplecticEulerImpactFrictionMap.cpp:201-407 on the GPU: the force acts
    first, the solve gets N^T vdelta and D^T vdelta (and the pose stabilisation if enabled), and the
    step ends with a linear update; the unconstrained map passed to flow() is not used.  CoR must
    be 0 (the reference asserts it)."""

    def __init__(self, abs_tol: float, max_iters: int, impulses_to_cache=ImpulsesToCache.NONE,
                 stabilize: bool = False, penetration_threshold: float = 0.0):
        super().__init__(abs_tol, max_iters, impulses_to_cache)
        if penetration_threshold < 0.0:
            raise ValueError("penetration_threshold must be non-negative")
        self.stabilize = bool(stabilize)
        self.penetration_threshold = float(penetration_threshold)

    def name(self):
        return "symplectic_euler_impact_friction_map"

    def _context(self, sim, umap, solver, dt, CoR, mu):
        if CoR != 0.0:
            raise ValueError("the symplectic Euler staggering needs CoR = 0")
        fresh = self._ctx is None
        ctx = super()._context(sim, umap, solver, dt, CoR, mu)
        if fresh or ctx is not getattr(self, "_staggered", None):
            ctx.set_staggering(_lib.STAGGER_SYMPLECTIC_EULER, self.stabilize, self.penetration_threshold)
            self._staggered = ctx
        return ctx


class StabilizedImpactFrictionMap(GeometricImpactFrictionMap):
    """scisim/ConstrainedMaps/StabilizedImpactFrictionMap.cpp:48-167 on the GPU: the unconstrained step,
    a cold solve from its velocity (no impulse cache), then q1 = q0 + dt v1."""

    def __init__(self, abs_tol: float, max_iters: int):
        super().__init__(abs_tol, max_iters, ImpulsesToCache.NONE)

    def name(self):
        return "stabilized_impact_friction_map"

    def _context(self, sim, umap, solver, dt, CoR, mu):
        fresh = self._ctx is None
        ctx = super()._context(sim, umap, solver, dt, CoR, mu)
        if fresh or ctx is not getattr(self, "_staggered", None):
            ctx.set_staggering(_lib.STAGGER_STABILIZED)
            self._staggered = ctx
        return ctx


class StaticPlane:
    """ball2d/StaticGeometry/StaticPlane.cpp:10-19 (normal normalised on upload)."""

    def __init__(self, x, n):
        self.x = np.asarray(x, dtype=np.float64).reshape(2)
        self.n = np.asarray(n, dtype=np.float64).reshape(2)


class Ball2DState:
    """ball2d/Ball2DState.h: interleaved q, v; radii; masses; static planes."""

    def __init__(self, q, v, r, m, static_planes=()):
        self.q = np.ascontiguousarray(q, dtype=np.float64).reshape(-1)
        self.v = np.ascontiguousarray(v, dtype=np.float64).reshape(-1)
        self.r = np.ascontiguousarray(r, dtype=np.float64).reshape(-1)
        self.m = np.ascontiguousarray(m, dtype=np.float64).reshape(-1)
        self.static_planes = list(static_planes)
        if self.q.shape[0] != 2 * self.r.shape[0] or self.v.shape != self.q.shape or self.m.shape != self.r.shape:
            raise ValueError("inconsistent Ball2D state sizes")

    def nballs(self):
        return self.r.shape[0]

    def plane_x(self):
        return np.array([p.x for p in self.static_planes]).reshape(-1)

    def plane_n(self):
        return np.array([p.n for p in self.static_planes]).reshape(-1)


# Identities of simulations: a map's context holds one simulation's scene (radii, masses, planes),
# and id() of a collected object can be reused, so each simulation draws its own number.
_SYSTEM_IDS = itertools.count(1)


def next_system_id() -> int:
    return next(_SYSTEM_IDS)


class Ball2DSim:
    """ball2d/Ball2DSim.h: owns the state; flow() advances one step (Ball2DSim.cpp:305-326).  A map
    keeps the radii, masses and planes from its first flow with this simulation; after changing
    them in place call the map's resetCachedData()."""

    def __init__(self, state: Ball2DState, gravity=(0.0, -9.81)):
        self.state = state
        self.gravity = tuple(float(g) for g in gravity)
        self.system_id = next_system_id()

    @property
    def nballs(self):
        return self.state.nballs()

    @property
    def nbodies(self):
        return self.state.nballs()

    def upload(self, ctx):
        st = self.state
        ctx.upload_ball2d(st.q, st.v, st.r, st.m, st.plane_x(), st.plane_n())

    def flow(self, iteration, dt, umap, CoR, mu, solver, ifmap):
        q1, v1 = ifmap.flow(self, umap, solver, iteration, dt, CoR, mu, self.state.q, self.state.v)
        self.state.q, self.state.v = q1, v1
        return ifmap.last_stats
