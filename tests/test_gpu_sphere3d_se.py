"""GPU parity tests for spheres under SymplecticEulerImpactFrictionMap (sg_set_staggering on a sphere
scene): libscisim_gb300.so against the oracle's restatement (se_step in oracle/sphere3d_oracle.cpp,
SymplecticEulerImpactFrictionMap.cpp:48-407).

The map acts with the force first (vdelta), detects on the exponential-Euler predictor, solves with
the extra relative velocities N^T vdelta and D^T vdelta (and the pose stabilisation), warm-starts from
an impulse cache whose cached force is turned from the cached normal onto the new one, and ends with
v1 = v2 + vdelta and an exponential-Euler configuration update.

Bars, every step, the oracle started from the GPU's state and replaying the GPU's colour order: the
contact sets and bases, the impulses, the sweeps and the residual bit-exact; positions and linear
velocities bit-exact; orientations and angular velocities within 1e-13 (CUDA's sin/cos and the host's
may differ in the last bit).
"""
import numpy as np
import pytest

from scisim_gb300 import scenes

pytestmark = pytest.mark.gpu


def run(gpulib, oracle, cache, stabilize, steps=60, warm=40, n=700):
    s = scenes.sphere_pile(n=n, seed=11, width=1.6, depth=1.6)
    nb = s["r"].shape[0]
    kw = dict(dt=s["dt"], gravity=s["gravity"], mu=s["mu"], CoR=0.0, tol=1e-10, max_iters=500)
    ctx = gpulib.Context(integrator=gpulib.SPLIT_HAM, cache_mode=cache, **kw)
    ctx.upload_sphere3d(s["q"], s["v"], s["r"], s["m"], s["I0"], s["plane_x"], s["plane_n"])
    ctx.set_staggering(gpulib.STAGGER_SYMPLECTIC_EULER, stabilize, 1e-5)
    ctx.step(warm)
    q0, v0 = ctx.state()
    sim = oracle.Sphere3D(q0, v0, s["r"], s["m"], s["I0"], s["plane_x"], s["plane_n"],
                          staggering=oracle.STAGGER_SYMPLECTIC_EULER, cache_mode=cache, stabilize=stabilize,
                          penetration_threshold=1e-5, **kw)
    # The oracle's impulse cache starts empty: the GPU restarts from this state with its cache
    # cleared as well (a new upload).
    ctx.upload_sphere3d(q0, v0, s["r"], s["m"], s["I0"], s["plane_x"], s["plane_n"])
    ctx.set_staggering(gpulib.STAGGER_SYMPLECTIC_EULER, stabilize, 1e-5)
    seen = 0
    for it in range(steps):
        q0, v0 = ctx.state()
        st = ctx.step(1)
        order, _ = ctx.last_solve_order()
        g = ctx.sphere3d_last_contacts()
        q1, v1 = ctx.state()
        if it > 0:
            # The GPU's state (world inertia as a step leaves it; at it = 0 both hold the state as
            # uploaded, with the inertia as the reference's constructor inserts it).
            sim.set_state(q0, v0)
        if st["n_contacts"] > 0:
            sim.set_next_order(order)
            seen += 1
        so = sim.step()
        c = sim.last_contacts()
        assert st["n_contacts"] == so["n_contacts"], it
        assert np.array_equal(g["ia"], c["ia"]) and np.array_equal(g["ib"], c["ib"]), it
        assert np.array_equal(g["bases"], c["bases"]), it
        assert st["iterations"] == so["iterations"] and st["error"] == so["error"], it
        assert np.array_equal(g["alpha"], c["alpha"]) and np.array_equal(g["beta"], c["beta"]), it
        qo, vo = sim.state()
        assert np.array_equal(q1[: 3 * nb], qo[: 3 * nb]), it
        assert np.array_equal(v1[: 3 * nb], vo[: 3 * nb]), it
        assert np.abs(q1[3 * nb:] - qo[3 * nb:]).max() <= 1e-13, it
        w_scale = max(1.0, np.abs(vo[3 * nb:]).max())
        assert np.abs(v1[3 * nb:] - vo[3 * nb:]).max() <= 1e-13 * w_scale, it
    ctx.close()
    return seen


@pytest.mark.parametrize("cache,stabilize", [(2, False), (2, True), (1, False)])
def test_sphere_symplectic_euler_matches_oracle(gpulib, oracle, cache, stabilize):
    seen = run(gpulib, oracle, cache, stabilize)
    assert seen >= 50


def test_sphere_symplectic_euler_checkpoint_keeps_cache(gpulib):
    """A checkpoint holds the sphere cache (normal and force per contact): a context restored from
    it steps on bit for bit like the one it was taken from."""
    s = scenes.sphere_pile(n=300, seed=13, width=1.0, depth=1.0)
    kw = dict(dt=s["dt"], gravity=s["gravity"], mu=s["mu"], CoR=0.0, tol=1e-9, max_iters=500,
              integrator=gpulib.SPLIT_HAM, cache_mode=gpulib.CACHE_NORMAL_AND_FRICTION)
    a = gpulib.Context(**kw)
    a.upload_sphere3d(s["q"], s["v"], s["r"], s["m"], s["I0"], s["plane_x"], s["plane_n"])
    a.set_staggering(gpulib.STAGGER_SYMPLECTIC_EULER, False, 0.0)
    a.step(120)
    ck = a.checkpoint()
    b = gpulib.Context(**kw)
    b.restore(ck)
    for _ in range(5):
        sa, sb = a.step(1), b.step(1)
        assert sa["iterations"] == sb["iterations"] and sa["n_contacts"] == sb["n_contacts"] > 0
    qa, va = a.state()
    qb, vb = b.state()
    assert np.array_equal(qa, qb) and np.array_equal(va, vb)
    a.close()
    b.close()


SE_SCENE = """<rigidbody3d_scene>
  <integrator type="dmv" dt="0.004"/>
  <sobogus_friction_solver mu="0.5" CoR="0.0" max_iters="500" tol="1.0e-9" eval_every="1"
     staggering="symplectic_euler" cache_impulses="normal_and_friction" stabilization="1"
     penetration_threshold="1.0e-5"/>
  <near_earth_gravity f="0.0 -9.81 0.0"/>
  <static_plane x="0 0 0" n="0 1 0"/>
  <static_plane x="-1 0 0" n="1 0 0"/>
  <static_plane x="1 0 0" n="-1 0 0"/>
  <geometry type="sphere" r="0.2"/>
  <geometry type="sphere" r="0.15"/>
  <rigid_body_with_density x="0.0 0.2 0.0" v="0.3 0.0 0.0" omega="0.0 1.0 0.0" rho="1.0" fixed="0" geo_idx="0"/>
  <rigid_body_with_density x="0.1 0.6 0.05" v="0 0 0" omega="0 0 2" rho="1.0" fixed="0" geo_idx="1"/>
  <rigid_body_with_density x="-0.3 0.9 0.0" v="0 -1 0" omega="1 0 0" rho="2.0" fixed="0" geo_idx="0"/>
</rigidbody3d_scene>"""


def test_sphere_symplectic_euler_scene_through_the_reference_classes(gpulib):
    """A sphere scene with staggering="symplectic_euler" read by scene_io and stepped through the
    mirror of the reference's classes (RigidBody3DSim::flow with SymplecticEulerImpactFrictionMap)
    gives, step for step, the bits of the C ABI path (sg_set_staggering on a sphere context)."""
    from scisim_gb300 import scene_io
    sc = scene_io.load_rigidbody3d_scene(SE_SCENE)
    sim, umap, solver, ifmap = scene_io.rigidbody3d_objects(sc)
    assert ifmap.name() == "symplectic_euler_impact_friction_map"
    ctx = gpulib.Context(dt=sc["dt"], gravity=sc["gravity"], mu=sc["mu"], CoR=sc["CoR"], tol=sc["tol"],
                         max_iters=sc["max_iters"], eval_every=sc["eval_every"], integrator=gpulib.SPLIT_HAM,
                         cache_mode=sc["cache_mode"])
    ctx.upload_sphere3d(sc["q"], sc["v"], sc["r"], sc["m"], sc["I0"], sc["plane_x"], sc["plane_n"])
    ctx.set_staggering(gpulib.STAGGER_SYMPLECTIC_EULER, sc["stabilization"], sc["penetration_threshold"])
    contacts = 0
    for it in range(1, 301):
        st = sim.flow(it, sc["dt"], umap, sc["CoR"], sc["mu"], solver, ifmap)
        s2 = ctx.step(1, first_iteration=it)
        q, v = ctx.state()
        assert st["n_contacts"] == s2["n_contacts"] and st["iterations"] == s2["iterations"], it
        assert np.array_equal(sim.state.q, q) and np.array_equal(sim.state.v, v), it
        contacts += s2["n_contacts"]
    assert contacts > 300
    # The spheres come to rest on the floor (no sinking: the lowest centre stays above its radius).
    nb = sc["r"].shape[0]
    y = q[1:3 * nb:3]
    assert np.all(y >= sc["r"] - 1e-3)
    ctx.close()
