"""SCISim's RigidBody3D plugin interfaces (spheres) on the GB300 library.

Mirrors the reference's driver loop for sphere scenes:

    spheres = [RigidBodySphere(r) for r in radii]
    state = RigidBody3DState.from_spheres(x, v, omega, spheres, density, [StaticPlane(x, n), ...])
    sim = RigidBody3DSim(state, gravity=(0.0, -9.81, 0.0))   # NearEarthGravityForce
    umap = SplitHamMap()                                       # rigidbody3d/UnconstrainedMaps/SplitHamMap.h
    solver = Sobogus(SobogusSolverType.RigidBodies3D, 1)
    ifmap = GeometricImpactFrictionMap(1e-9, 5000, ImpulsesToCache.NONE)
    for it in range(1, n + 1):
        sim.flow(it, dt, umap, CoR, mu, solver, ifmap)         # rigidbody3d/RigidBody3DSim.cpp:557-630

Each step runs on the GPU: split-Hamiltonian predictor, q1 grid broad phase, sphere and
plane narrow phase, velocity-dependent contact bases, coloured 3x3-block Gauss-Seidel,
final map and the world-inertia update.  The reference's 3D geometric map keeps no impulse
cache (rigidbody3dutils/RigidBody3DSceneParser.cpp:1877-1880), so only ImpulsesToCache.NONE
is accepted.
"""
from __future__ import annotations

import math

import numpy as np

from . import _lib
from .ball2d import (GeometricImpactFrictionMap, ImpulsesToCache, Sobogus, SobogusSolverType,  # noqa: F401
                     UnconstrainedMap, next_system_id)


class SplitHamMap(UnconstrainedMap):
    """rigidbody3d/UnconstrainedMaps/SplitHamMap.cpp:17-182 (executed on the GPU inside each step)."""
    integrator = _lib.SPLIT_HAM

    def name(self):
        return "split_ham"


class RigidBodySphere:
    """rigidbody3d/Geometry/RigidBodySphere.cpp"""

    def __init__(self, r):
        if not r > 0.0:
            raise ValueError("sphere radius must be positive")
        self.r = float(r)

    def computeMassAndInertia(self, density):
        """RigidBodySphere.cpp:10-18: (M, CM, I, R) with the reference's operation order."""
        r = self.r
        M = 4.0 * math.pi * r * r * r / 3.0
        I = 2.0 * M * r * r / 5.0
        M *= density
        I *= density
        return M, np.zeros(3), np.full(3, I), np.eye(3)


class StaticPlane:
    """rigidbody3d/StaticGeometry/StaticPlane.cpp:10-15 (normal normalised on upload)."""

    def __init__(self, x, n):
        self.x = np.asarray(x, dtype=np.float64).reshape(3)
        self.n = np.asarray(n, dtype=np.float64).reshape(3)


class RigidBody3DState:
    """rigidbody3d/RigidBody3DState.h restricted to spheres: q = [x (3nb) | R row-major (9nb)],
    v = [v (3nb) | omega (3nb)], radii, masses and principal inertias."""

    def __init__(self, q, v, r, m, I0, static_planes=()):
        self.q = np.ascontiguousarray(q, dtype=np.float64).reshape(-1)
        self.v = np.ascontiguousarray(v, dtype=np.float64).reshape(-1)
        self.r = np.ascontiguousarray(r, dtype=np.float64).reshape(-1)
        self.m = np.ascontiguousarray(m, dtype=np.float64).reshape(-1)
        self.I0 = np.ascontiguousarray(I0, dtype=np.float64).reshape(-1)
        self.static_planes = list(static_planes)
        nb = self.r.shape[0]
        if (self.q.shape[0] != 12 * nb or self.v.shape[0] != 6 * nb or self.m.shape[0] != nb
                or self.I0.shape[0] != 3 * nb):
            raise ValueError("inconsistent RigidBody3D state sizes")

    @classmethod
    def from_spheres(cls, x, v, omega, spheres, density=1.0, static_planes=(), R=None):
        n = len(spheres)
        mass = np.empty(n)
        I0 = np.empty(3 * n)
        for i, s in enumerate(spheres):
            M, _, I, _ = s.computeMassAndInertia(density)
            mass[i] = M
            I0[3 * i:3 * i + 3] = I
        R = np.tile(np.eye(3).reshape(-1), n) if R is None else np.asarray(R, dtype=np.float64).reshape(-1)
        q = np.concatenate([np.asarray(x, dtype=np.float64).reshape(-1), R])
        vv = np.concatenate([np.asarray(v, dtype=np.float64).reshape(-1),
                             np.asarray(omega, dtype=np.float64).reshape(-1)])
        return cls(q, vv, [s.r for s in spheres], mass, I0, static_planes)

    def nbodies(self):
        return self.r.shape[0]

    def plane_x(self):
        return np.array([p.x for p in self.static_planes]).reshape(-1)

    def plane_n(self):
        return np.array([p.n for p in self.static_planes]).reshape(-1)


class RigidBody3DSim:
    """rigidbody3d/RigidBody3DSim.h: owns the state; flow() advances one step
    (RigidBody3DSim.cpp:557-630, world inertia updated from the new orientations)."""

    def __init__(self, state: RigidBody3DState, gravity=(0.0, -9.81, 0.0)):
        self.state = state
        self.gravity = tuple(float(g) for g in gravity)
        if len(self.gravity) != 3:
            raise ValueError("NearEarthGravityForce takes a 3-vector")
        self.system_id = next_system_id()

    @property
    def nbodies(self):
        return self.state.nbodies()

    def upload(self, ctx):
        st = self.state
        ctx.upload_sphere3d(st.q, st.v, st.r, st.m, st.I0, st.plane_x(), st.plane_n())

    def flow(self, iteration, dt, umap, CoR, mu, solver, ifmap):
        from .ball2d import StabilizedImpactFrictionMap, SymplecticEulerImpactFrictionMap
        if isinstance(ifmap, StabilizedImpactFrictionMap):
            raise ValueError("sphere scenes step with the geometric or the symplectic Euler map")
        if not isinstance(ifmap, SymplecticEulerImpactFrictionMap):
            # The symplectic-Euler map integrates by exponential Euler and keeps its 3D cache.
            if not isinstance(umap, SplitHamMap):
                raise ValueError("sphere scenes step with SplitHamMap")
            if ifmap.impulses_to_cache != ImpulsesToCache.NONE:
                raise ValueError("the 3D geometric map keeps no impulse cache (RigidBody3DSceneParser.cpp:1877-1880)")
        q1, v1 = ifmap.flow(self, umap, solver, iteration, dt, CoR, mu, self.state.q, self.state.v)
        self.state.q, self.state.v = q1, v1
        return ifmap.last_stats
