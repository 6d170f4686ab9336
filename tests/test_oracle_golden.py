"""Pins the CPU oracle against the reference's own known-answer tests.

* 2D broad phase: the three AABB fixtures of ball2dtests/collision_detection_tests.cpp
  with the reference's criterion (grid pairs == all pairs, :34-40).
* CCD narrow phase: the 11 cases of scisimtests/narrowphase_tests.cpp.
* Analytic friction: the ball-on-slope scenes registered in
  ball2dcli/CMakeLists.txt:78-98 (geometric staggering) and :102-122 (symplectic Euler
  staggering with the impulse cache), checked against the closed forms of
  assets/ball2d/shell_scripts/sliding_particle_test.py:44-54 and
  static_particle_test.py:32-47 with the registered tolerances.
"""
import gzip
import hashlib
import json
import math
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def load_fixture(tag):
    with gzip.open(os.path.join(GOLDEN, "aabb2d_fixture_%s.txt.gz" % tag), "rt") as fh:
        return np.array([float(t) for t in fh.read().split()]).reshape(-1, 4)


def digest(pairs):
    return hashlib.sha256(np.ascontiguousarray(pairs, dtype=np.int32).tobytes()).hexdigest()


EXPECTED = json.load(open(os.path.join(GOLDEN, "aabb2d_expected.json")))
CCD = json.load(open(os.path.join(GOLDEN, "ccd_cases.json")))
SLOPES = json.load(open(os.path.join(GOLDEN, "slope_scenes.json")))


@pytest.mark.parametrize("tag", ["00", "01", "02"])
def test_aabb_fixture_grid_equals_allpairs(oracle, tag):
    aabb = load_fixture(tag)
    assert aabb.shape[0] == EXPECTED[tag]["n_aabbs"]
    assert (aabb[:, :2] < aabb[:, 2:]).all()
    grid = oracle.grid_overlaps_2d(aabb)
    allp = oracle.allpairs_overlaps_2d(aabb)
    assert np.array_equal(grid, allp)
    assert grid.shape[0] == EXPECTED[tag]["n_pairs"]
    assert digest(grid) == EXPECTED[tag]["sha256"]


def test_grid_3d_equals_allpairs(oracle):
    rng = np.random.default_rng(3)
    c = rng.uniform(-5, 5, (3000, 3))
    e = rng.uniform(0.05, 0.4, (3000, 3))
    aabb = np.concatenate([c - e, c + e], axis=1)
    assert np.array_equal(oracle.grid_overlaps_3d(aabb), oracle.allpairs_overlaps_3d(aabb))


def _eval_expr(expr):
    return float(eval(expr, {"sqrt": math.sqrt}))


@pytest.mark.parametrize("case", CCD, ids=[c["name"] for c in CCD])
def test_ccd_cases(oracle, case):
    c = oracle.ccd_coeffs_2d(case["q0a"], case["q1a"], case["ra"], case["q0b"], case["q1b"], case["rb"])
    if case["cexpected"] is not None:
        assert np.abs(c - np.array(case["cexpected"])).max() <= 1e-9
    hit, t = oracle.ccd_happens(c)
    assert hit == case["hit"]
    if case["time_expr"] is not None:
        assert abs(t - _eval_expr(case["time_expr"])) <= case["time_tol"]


def analytic_error(scene, q, v, time):
    """Closed forms of the reference's sliding/static checkers."""
    g, mu = 10.0, 0.5
    n = scene["plane_n"]
    if scene["kind"] == "static":
        return [abs(q[0]), abs(q[1]), abs(v[0]), abs(v[1])]
    theta = abs(math.atan2(n[0], n[1]))
    dpl = 0.5 * time * time * (-g * math.sin(theta) + g * mu * math.cos(theta))
    dx = dpl * math.cos(theta) * (-1.0 if n[0] > 0 else 1.0)
    dy = dpl * math.sin(theta)
    vpl = time * (-g * math.sin(theta) + g * mu * math.cos(theta))
    vx = vpl * math.cos(theta) * (-1.0 if n[0] > 0 else 1.0)
    vy = vpl * math.sin(theta)
    return [abs(q[0] - dx), abs(q[1] - dy), abs(vx - v[0]), abs(vy - v[1])]


CACHE = {"none": 0, "normal": 1, "normal_and_friction": 2}
STAGGER = {"geometric": 0, "symplectic_euler": 1}


def make_slope_oracle(oracle, s):
    b = s["ball"]
    return oracle.Ball2D([b["x"], b["y"]], [b["vx"], b["vy"]], [b["r"]], [b["m"]], s["plane_x"], s["plane_n"],
                         dt=s["dt"], gravity=s["gravity"], mu=s["mu"], CoR=s["CoR"], tol=s["tol"],
                         max_iters=s["max_iters"], eval_every=s["eval_every"],
                         integrator=oracle.VERLET if s["integrator"] == "verlet" else oracle.SYMPLECTIC_EULER,
                         cache_mode=CACHE[s["cache_impulses"]], staggering=STAGGER[s["staggering"]],
                         stabilize=bool(s["stabilization"]), penetration_threshold=s["penetration_threshold"])


@pytest.mark.parametrize("scene", SLOPES, ids=[s["name"] for s in SLOPES])
def test_slope_scene_closed_form(oracle, scene):
    sim = make_slope_oracle(oracle, scene)
    per = int(round(scene["output_frequency"] / scene["dt"]))
    for k in range(1, int(round(scene["end_time"] / scene["output_frequency"])) + 1):
        sim.run(per)
        q, v = sim.state()
        err = analytic_error(scene, q, v, sim.iteration * scene["dt"])
        assert all(e <= t for e, t in zip(err, scene["tolerances"])), (k, err, scene["tolerances"])


def test_stabilized_map_is_drift_safe(oracle):
    """StabilizedImpactFrictionMap on the reference's drift-safe scene
    (assets/ball2d/tests_serialization/drift_safe_ball_on_plane.xml, registered in
    ball2dcli/CMakeLists.txt:23): a ball dropped on a plane comes to rest above it and then does not
    move at all (each step's solve cancels the unconstrained step's normal velocity)."""
    sim = oracle.Ball2D([0.0, 1.0], [0.0, 0.0], [0.5], [8.0], [[0.0, 0.0]], [[0.0, 1.0]], dt=0.01,
                        gravity=(0.0, -10.0), mu=0.5, CoR=0.0, tol=1e-12, max_iters=5000, eval_every=1,
                        integrator=oracle.VERLET, cache_mode=oracle.CACHE_NONE,
                        staggering=oracle.STAGGER_STABILIZED)
    sim.run(200)
    q_rest, v_rest = sim.state()
    assert 0.5 - 1e-12 <= q_rest[1] <= 0.5 + 0.2 and np.all(v_rest == 0.0)
    sim.run(250)
    q, v = sim.state()
    assert np.array_equal(q, q_rest) and np.all(v == 0.0)
