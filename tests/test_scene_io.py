"""XML scene reader (scisim_gb300/scene_io.py) for the reference's ball2d_scene and rigidbody3d_scene
formats: values as the reference's parsers read them, unsupported features rejected by name, and the
reference's own asset scenes (when the reference tree is present) either loaded or rejected cleanly.
"""
import glob
import os
from fractions import Fraction

import numpy as np
import pytest

from scisim_gb300 import scene_io, scenes

BALL2D = """<ball2d_scene>
  <camera cx="0" cy="0" scale_factor="1" fps="50" render_at_fps="1" locked="1"/>
  <integrator type="verlet" dt="1/300"/>
  <end_time t="0.5"/>
  <sobogus_friction_solver mu="0.4" CoR="0.2" max_iters="800" tol="1.0e-9" eval_every="2"
     staggering="geometric" cache_impulses="normal_and_friction"/>
  <gravity fx="0.5" fy="-9.81"/>
  <static_plane x="0.0 -1.0" n="0.1 1.0"/>
  <static_plane x="3.0 0.0" n="-1 0"/>
  <ball x="0.1" y="0.25" vx="1.5" vy="-0.5" m="2.0" r="0.25" fixed="0"/>
  <ball x="0.7" y="0.1" vx="0" vy="0" m="1.0" r="0.2" fixed="0"/>
</ball2d_scene>"""

SPHERES = """<rigidbody3d_scene>
  <camera_perspective theta="1" phi="0.4" rho="12" lookat="0 0 0" up="0 1 0" fps="100" render_at_fps="1" locked="0"/>
  <integrator type="split_ham" dt="0.001"/>
  <sobogus_friction_solver mu="0.3" CoR="0.1" max_iters="500" tol="1.0e-10" eval_every="1" staggering="geometric"
     cache_impulses="normal_and_friction"/>
  <near_earth_gravity f="0.0 -9.81 0.0"/>
  <static_plane x="0 0 0" n="0 1 0"/>
  <geometry type="sphere" r="0.5"/>
  <geometry type="sphere" r="0.25"/>
  <rigid_body_with_density x="0.0 0.5 0.0" v="0.1 0.0 0.0" omega="0.0 1.0 0.0" rho="2.0" fixed="0" geo_idx="0"/>
  <rigid_body_with_density x="1.0 0.3 0.0" v="0 0 0" omega="0 0 0" rho="1.0" fixed="0" geo_idx="-1"/>
</rigidbody3d_scene>"""


def test_ball2d_scene_values():
    s = scene_io.load_ball2d_scene(BALL2D)
    assert s["integrator"] == "verlet" and s["dt_rational"] == Fraction(1, 300) and s["dt"] == 1.0 / 300.0
    assert s["end_time"] == 0.5 and scene_io.steps_to(s["end_time"], s["dt_rational"]) == 150
    assert (s["mu"], s["CoR"], s["tol"], s["max_iters"], s["eval_every"], s["cache_mode"]) == (0.4, 0.2, 1e-9, 800, 2, 2)
    assert s["gravity"] == (0.5, -9.81)
    assert np.array_equal(s["q"], [0.1, 0.25, 0.7, 0.1]) and np.array_equal(s["v"], [1.5, -0.5, 0.0, 0.0])
    assert np.array_equal(s["m"], [2.0, 1.0]) and np.array_equal(s["r"], [0.25, 0.2])
    assert np.array_equal(s["plane_x"], [[0.0, -1.0], [3.0, 0.0]]) and np.array_equal(s["plane_n"], [[0.1, 1.0], [-1, 0]])
    sim, umap, solver, ifmap = scene_io.ball2d_objects(s)
    assert umap.name() == "verlet" and sim.state.nballs() == 2


def test_decimal_dt_is_exact():
    s = scene_io.load_ball2d_scene(BALL2D.replace('dt="1/300"', 'dt="0.00001"'))
    assert s["dt_rational"] == Fraction(1, 100000) and s["dt"] == 1.0 / 100000.0


UNSUPPORTED = {
    "static_drum": BALL2D.replace('<ball x="0.7"', '<static_drum x="0" y="0" r="5"/>\n  <ball x="0.7"'),
    "fixed": BALL2D.replace('m="1.0" r="0.2" fixed="0"', 'm="1.0" r="0.2" fixed="1"'),
    "staggering": BALL2D.replace('staggering="geometric"', 'staggering="staggered_projections"'),
    "integrator": BALL2D.replace('type="verlet"', 'type="explicit_euler"'),
}


@pytest.mark.parametrize("word", sorted(UNSUPPORTED))
def test_ball2d_unsupported_features_are_rejected(word):
    with pytest.raises(scene_io.SceneError, match=word):
        scene_io.load_ball2d_scene(UNSUPPORTED[word])


def test_sphere_scene_values():
    s = scene_io.load_rigidbody3d_scene(SPHERES)
    m, i0 = scenes.sphere_mass_inertia(np.array([0.5, 0.25]), 1.0)
    assert s["m"][1] == m[1] and s["I0"][3] == i0[1]
    m2, i2 = scenes.sphere_mass_inertia(np.array([0.5]), 2.0)
    assert s["m"][0] == m2[0] and s["I0"][0] == i2[0]
    assert np.array_equal(s["q"][:6], [0.0, 0.5, 0.0, 1.0, 0.3, 0.0])
    assert np.array_equal(s["q"][6:15], np.eye(3).reshape(-1))
    assert np.array_equal(s["v"], [0.1, 0, 0, 0, 0, 0, 0, 1.0, 0, 0, 0, 0])
    assert s["cache_mode"] == 0 and s["gravity"] == (0.0, -9.81, 0.0)
    sim, umap, solver, ifmap = scene_io.rigidbody3d_objects(s)
    assert umap.name() == "split_ham"
    with pytest.raises(scene_io.SceneError, match="orientation"):
        scene_io.load_rigidbody3d_scene(SPHERES.replace('geo_idx="0"/>', 'geo_idx="0" R="0 0 1"/>'))


ASSETS = "/root/reference/assets"


@pytest.mark.skipif(not os.path.isdir(ASSETS), reason="reference assets not present")
def test_reference_assets_load_or_are_rejected_by_name():
    ok = bad = 0
    for path in sorted(glob.glob(ASSETS + "/ball2d/**/*.xml", recursive=True)):
        try:
            s = scene_io.load_ball2d_scene(path)
        except scene_io.SceneError:
            bad += 1
            continue
        ok += 1
        assert s["dt"] > 0 and s["q"].shape[0] == 2 * s["r"].shape[0]
    assert ok >= 10 and bad >= 1


@pytest.mark.skipif(not os.path.isdir(ASSETS), reason="reference assets not present")
def test_reference_rigidbody2d_assets_load_or_are_rejected_by_name():
    """Circle scenes load with the reference's mass and inertia from rho; boxes, portals, fixed
    bodies and scripting are rejected with a SceneError naming them."""
    ok, reasons = 0, set()
    for path in sorted(glob.glob(ASSETS + "/rigidbody2d/**/*.xml", recursive=True)):
        try:
            s = scene_io.load_rigidbody2d_scene(path)
        except scene_io.SceneError as e:
            reasons.add(str(e).split(":")[0])
            continue
        ok += 1
        n = s["r"].shape[0]
        assert s["q"].shape[0] == 3 * n and s["v"].shape[0] == 3 * n
        assert np.all(s["I"] == 0.5 * s["m"] * s["r"] * s["r"])
    assert ok >= 22 and "geometry" in reasons


def test_rigidbody2d_scene_values():
    text = """<rigidbody2d_scene>
      <integrator type="verlet" dt="1/200"/>
      <sobogus_friction_solver mu="0.3" CoR="0.1" max_iters="100" eval_every="5" tol="1e-8"
                               staggering="geometric" cache_impulses="normal"/>
      <near_earth_gravity f="0.0 -10.0"/>
      <static_plane x="0 0" n="0 2"/>
      <geometry type="circle" r="0.5"/>
      <rigid_body x="1.0 2.0" theta="0.25" v="0.5 -1.0" omega="3.0" rho="2.0" geo_idx="0"/>
    </rigidbody2d_scene>"""
    s = scene_io.load_rigidbody2d_scene(text)
    assert s["dt_rational"] == Fraction(1, 200) and s["integrator"] == "verlet" and s["gravity"] == (0.0, -10.0)
    assert list(s["q"]) == [1.0, 2.0, 0.25] and list(s["v"]) == [0.5, -1.0, 3.0]
    assert s["m"][0] == 2.0 * np.pi * 0.5 * 0.5 and s["I"][0] == 0.5 * s["m"][0] * 0.5 * 0.5
    assert (s["mu"], s["CoR"], s["max_iters"], s["eval_every"], s["cache_mode"]) == (0.3, 0.1, 100, 5, 1)
    for bad in (text.replace('type="circle" r="0.5"', 'type="box" r="0.5 0.5"'),
                text.replace('geo_idx="0"', 'geo_idx="0" fixed="1"'),
                text.replace('staggering="geometric"', 'staggering="symplectic_euler"'),
                text.replace('staggering="geometric"', 'staggering="stabilized"')):  # with a cache
        with pytest.raises(scene_io.SceneError):
            scene_io.load_rigidbody2d_scene(bad)


@pytest.mark.skipif(not os.path.isdir(ASSETS), reason="reference assets not present")
def test_registered_slope_scenes_match_the_golden_extraction():
    """The 18 slope scenes registered in ball2dcli/CMakeLists.txt, read by this reader, equal the
    values tests/golden/make_golden.py extracted from the same files with its own code."""
    import json
    golden = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "slope_scenes.json")))
    for g in golden:
        s = scene_io.load_ball2d_scene(os.path.join(os.path.dirname(ASSETS), g["xml"]))
        assert s["integrator"] == g["integrator"] and s["dt"] == g["dt"]
        assert (s["mu"], s["CoR"], s["tol"], s["max_iters"], s["eval_every"]) == (
            g["mu"], g["CoR"], g["tol"], g["max_iters"], g["eval_every"])
        assert s["cache_mode"] == scene_io.CACHE_MODES[g["cache_impulses"]]
        assert list(s["gravity"]) == g["gravity"]
        assert list(s["plane_x"][0]) == g["plane_x"] and list(s["plane_n"][0]) == g["plane_n"]
        b = g["ball"]
        assert list(s["q"]) == [b["x"], b["y"]] and list(s["v"]) == [b["vx"], b["vy"]]
        assert s["m"][0] == b["m"] and s["r"][0] == b["r"]


def test_symplectic_euler_staggering():
    text = BALL2D.replace('CoR="0.2"', 'CoR="0.0"').replace(
        'staggering="geometric"', 'staggering="symplectic_euler" stabilization="1" penetration_threshold="1.0e-5"')
    s = scene_io.load_ball2d_scene(text)
    assert s["staggering"] == "symplectic_euler" and s["stabilization"] and s["penetration_threshold"] == 1e-5
    _, _, _, ifmap = scene_io.ball2d_objects(s)
    assert ifmap.name() == "symplectic_euler_impact_friction_map" and ifmap.stabilize
    with pytest.raises(scene_io.SceneError, match="CoR"):
        scene_io.load_ball2d_scene(text.replace('CoR="0.0"', 'CoR="0.5"'))


def test_stabilized_staggering():
    text = BALL2D.replace('staggering="geometric"', 'staggering="stabilized"')
    with pytest.raises(scene_io.SceneError, match="cache"):
        scene_io.load_ball2d_scene(text)
    s = scene_io.load_ball2d_scene(text.replace('cache_impulses="normal_and_friction"', 'cache_impulses="none"'))
    assert s["staggering"] == "stabilized"
    assert scene_io.ball2d_objects(s)[3].name() == "stabilized_impact_friction_map"


RATIONAL_TESTS = "/root/reference/scisimtests/rational_number_tests.cpp"


def _registered_rational_cases():
    """(input string, expected double) of every parsing case in the reference's rational-number
    test program: `extractFromString( "<in>", ... )` followed by `fabs( <expected> - scalar(...) )`."""
    import re
    src = open(RATIONAL_TESTS).read()
    cases = re.findall(r'extractFromString\(\s*"([^"]*)"\s*,\s*rational_number\s*\).*?fabs\(\s*([^)]*?)\s+-\s+scalar',
                       src, flags=re.S)
    out = []
    for text, expr in cases:
        assert re.fullmatch(r"[-+0-9. /]+", expr), expr
        out.append((text, float(eval(expr))))  # a numeric literal or a quotient of two
    return out


@pytest.mark.skipif(not os.path.isfile(RATIONAL_TESTS), reason="reference tests not present")
def test_rational_matches_reference_tests():
    """scene_io.rational reads every string of the reference's registered rational-number parsing
    tests (scisimtests/CMakeLists.txt:9-19) to exactly the double the test expects."""
    cases = _registered_rational_cases()
    assert len(cases) == 11
    for text, want in cases:
        got = scene_io.rational(text)
        assert float(got.numerator) / float(got.denominator) == want, (text, got, want)


def test_rational_reference_rules():
    """The rules of the reference's extraction beyond its registered cases: stream extraction of
    each part (trailing characters ignored), the fraction digits taking the integer part's sign,
    and rejected forms."""
    r = scene_io.rational
    assert r("1/100") == Fraction(1, 100) and r(" 3 / 6 ") == Fraction(1, 2)
    assert r("0.0010") == Fraction(1, 1000) and r("7") == 7
    assert r("-0.5") == Fraction(1, 2)      # integer part -0 is not negative
    assert r("-1.5") == Fraction(-3, 2)
    assert r("1.5e-3") == Fraction(1, 1) + Fraction(5, 10000)  # "5e-3" extracts as 5 over 10^4
    assert r("+") == 0 and r(" - . ") == 0   # a bare sign is read as 0
    for bad in ("1/2/3/4", "1.2/3", "abc", "1/0", "./", "1..2.3"):
        with pytest.raises(scene_io.SceneError):
            r(bad)


def test_scalar_stream_extraction_rules():
    """Scalars as `std::stringstream >> double` reads them (the longest decimal prefix, the rest
    ignored; no nan, no digit separators), and vectors as readScalarList with single spaces."""
    d = scene_io.stream_double
    assert d("0.25") == 0.25 and d("  -3.5e2") == -350.0 and d("1.5abc") == 1.5 and d(".5") == 0.5
    assert d("7.") == 7.0 and d("2e3x") == 2000.0
    for bad in ("", "abc", "- 1", "nan", "1e", "1e+", "inf"):
        assert d(bad) is None, bad
    import xml.etree.ElementTree as ET
    nd = ET.fromstring('<b x="1 2 3" y="1  2 3" z="-inf 0 inf" w="1 2 3 "/>')
    assert scene_io._vector(nd, "x", 3, "b") == [1.0, 2.0, 3.0]
    assert scene_io._vector(nd, "z", 3, "b")[0] == float("-inf")
    for name in ("y", "w"):
        with pytest.raises(scene_io.SceneError):
            scene_io._vector(nd, name, 3, "b")
