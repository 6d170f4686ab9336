"""The oracle under AddressSanitizer and UndefinedBehaviorSanitizer, as the reference runs its own
C++ (CMakeLists.txt:261, SANITIZER=address|undefined): the Makefile's `sanitize` build of the same
sources is loaded in a child process with libasan preloaded, and a workout of every oracle entry
point the tests use (broad phase, CCD, the Ball2D, symplectic-Euler, stabilized, sphere (both
staggerings) and RigidBody2D steppers with and without the impulse cache, the standalone solves, the residuals
and the MLP) must finish without a sanitizer report.
"""
import os
import shutil
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKOUT = r'''
import numpy as np
from oracle import oracle as O
from scisim_gb300 import scenes

assert O.LIB_PATH.endswith("liboracle_san.so"), O.LIB_PATH
rng = np.random.default_rng(0)
lo = rng.uniform(0, 10, (300, 2))
aabb = np.concatenate([lo, lo + rng.uniform(0.05, 0.5, (300, 2))], 1)
assert O.grid_overlaps_2d(aabb).shape == O.allpairs_overlaps_2d(aabb).shape
s = scenes.box_drop_1024(seed=4, n_side=8)
for kw in (dict(cache_mode=O.CACHE_NORMAL_AND_FRICTION, integrator=O.VERLET, CoR=0.3),
           dict(cache_mode=O.CACHE_NORMAL, staggering=O.STAGGER_SYMPLECTIC_EULER, stabilize=True,
                penetration_threshold=1e-4, CoR=0.0),
           dict(staggering=O.STAGGER_STABILIZED, CoR=0.3)):
    b = O.Ball2D(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"], dt=s["dt"], gravity=s["gravity"],
                 mu=0.5, tol=1e-9, max_iters=200, **kw)
    b.run(40)
    b.last_contacts()
sp = scenes.sphere_pile(n=64, seed=3, width=1.0, depth=1.0)
o = O.Sphere3D(sp["q"], sp["v"], sp["r"], sp["m"], sp["I0"], sp["plane_x"], sp["plane_n"], dt=sp["dt"],
               gravity=sp["gravity"], mu=sp["mu"], CoR=sp["CoR"], tol=1e-9, max_iters=200)
o.run(30)
o.last_contacts()
o.world_inertia()
se = O.Sphere3D(sp["q"], sp["v"], sp["r"], sp["m"], sp["I0"], sp["plane_x"], sp["plane_n"], dt=sp["dt"],
                gravity=sp["gravity"], mu=sp["mu"], CoR=0.0, tol=1e-9, max_iters=200,
                staggering=O.STAGGER_SYMPLECTIC_EULER, cache_mode=O.CACHE_NORMAL_AND_FRICTION, stabilize=True,
                penetration_threshold=1e-5)
se.run(30)
n = 24
r = rng.uniform(0.1, 0.2, n)
m, I = O.circle_mass_inertia(r, 1.0)
xy = np.stack([np.tile(np.arange(6) * 0.45 - 1.1, 4), np.repeat(np.arange(4) * 0.45 + 0.25, 6)], 1)
q = np.concatenate([xy, rng.uniform(-1, 1, (n, 1))], 1).reshape(-1)
v = np.concatenate([rng.normal(0, 0.5, (n, 2)), rng.normal(0, 1, (n, 1))], 1).reshape(-1)
for stag, cache in ((O.STAGGER_GEOMETRIC, O.CACHE_NORMAL_AND_FRICTION), (O.STAGGER_STABILIZED, O.CACHE_NONE)):
    rb = O.RigidBody2D(q, v, r, m, I, [[0.0, 0.0], [-1.5, 0.0], [1.5, 0.0]], [[0.0, 1.0], [1.0, 0.0], [-1.0, 0.0]],
                       dt=0.005, mu=0.4, CoR=0.2, tol=1e-10, max_iters=500, cache_mode=cache, staggering=stag)
    rb.run(100)
    rb.last_contacts()
x = rng.normal(size=(16, 12)).astype(np.float32)
t = rng.normal(size=(16, 3)).astype(np.float32)
params = rng.normal(scale=0.1, size=O.mlp_param_count()).astype(np.float32)
O.mlp_forward(params, x)
O.mlp_loss_grad(params, x, t)
print("workout ok")
'''


@pytest.mark.timeout(600)
def test_oracle_under_asan_and_ubsan():
    if shutil.which("make") is None or shutil.which("g++") is None:
        pytest.skip("no C++ toolchain")
    asan = subprocess.run(["g++", "-print-file-name=libasan.so"], capture_output=True, text=True).stdout.strip()
    if not os.path.isabs(asan) or not os.path.exists(asan):
        pytest.skip("libasan not available")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "sanitize"], check=True, timeout=600)
    env = dict(os.environ, LD_PRELOAD=asan, SG_ORACLE_LIB=os.path.join(ROOT, "oracle", "_build", "liboracle_san.so"),
               ASAN_OPTIONS="detect_leaks=0:abort_on_error=0", UBSAN_OPTIONS="print_stacktrace=1:halt_on_error=1",
               PYTHONPATH=ROOT)
    p = subprocess.run([sys.executable, "-c", WORKOUT], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=600)
    report = p.stderr[-4000:]
    assert p.returncode == 0, report
    assert "runtime error" not in p.stderr and "AddressSanitizer" not in p.stderr, report
    assert "workout ok" in p.stdout
