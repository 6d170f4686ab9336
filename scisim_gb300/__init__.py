"""GB300-native (sm_103a) SCISim contact path: Ball2D discs and RigidBody3D spheres.

The compute path is libscisim_gb300.so (CUDA kernels behind the C ABI in
include/scisim_gpu.h); this package is its host-side mirror of SCISim's
UnconstrainedMap / FrictionSolver / ImpactFrictionMap interfaces.
"""
from ._lib import Context, SgError  # noqa: F401
from .ball2d import (Ball2DSim, Ball2DState, GeometricImpactFrictionMap, ImpulsesToCache, Sobogus,  # noqa: F401
                     SobogusSolverType, StabilizedImpactFrictionMap, StaticPlane, SymplecticEulerImpactFrictionMap,
                     SymplecticEulerMap, VerletMap)
from .rigidbody3d import RigidBody3DSim, RigidBody3DState, RigidBodySphere, SplitHamMap  # noqa: F401

__all__ = ["Context", "SgError", "Ball2DSim", "Ball2DState", "GeometricImpactFrictionMap", "ImpulsesToCache",
           "Sobogus", "SobogusSolverType", "StabilizedImpactFrictionMap", "StaticPlane", "SymplecticEulerImpactFrictionMap", "SymplecticEulerMap",
           "VerletMap", "RigidBody3DSim",
           "RigidBody3DState", "RigidBodySphere", "SplitHamMap"]
