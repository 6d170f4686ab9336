"""Regenerates the golden fixtures in this folder from the SCISim sources.

Run in a checkout that has the reference sources (default location given by
--ref).  The tests read only the committed outputs:

  aabb2d_fixture_{00,01,02}.txt.gz  2D AABB known-answer fixtures (5k/10k/20k boxes),
                                    copied number-for-number from
                                    ball2dtests/collision_detection_tests.cpp:12,14,16
  aabb2d_expected.json              pair count and SHA-256 of the all-pairs overlap
                                    set of each fixture (the test's criterion,
                                    collision_detection_tests.cpp:34-40), computed by
                                    the CPU oracle's all-pairs routine
  ccd_cases.json                    the 11 ball-ball CCD cases of
                                    scisimtests/narrowphase_tests.cpp:6-466
  slope_scenes.json                 the analytic ball-on-slope friction scenes
                                    (assets/ball2d/tests_friction/ball_plane/mu_0p5/*)
                                    with the tolerances registered in
                                    ball2dcli/CMakeLists.txt:78-98
  sphere_inertia.json               the sphere mass/inertia known answer of
                                    rigidbody3dtests/rigidbody3d_inertia_tests.cpp:17-47
  rigidbody2d_scenes.json           the reference's circle-only rigidbody2d scenes
                                    (assets/rigidbody2d/**/*.xml) as scisim_gb300.scene_io
                                    reads them (state, planes, map and solver settings), for the
                                    GPU tests, which cannot read the reference's assets
"""
from __future__ import annotations

import argparse
import gzip
import hashlib
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def extract_aabb_arrays(ref):
    src = open(os.path.join(ref, "ball2dtests", "collision_detection_tests.cpp")).read()
    out = {}
    for m in re.finditer(r"const scalar (test_\d\d)_data\[\] = \{([^}]*)\};", src):
        out[m.group(1)] = [t.strip() for t in m.group(2).split(",") if t.strip()]
    return out


def pairset_digest(pairs):
    pairs = np.ascontiguousarray(pairs, dtype=np.int32)
    return hashlib.sha256(pairs.tobytes()).hexdigest()


_num = r"(-?[0-9.]+(?:e-?[0-9]+)?)"


def extract_ccd_cases(ref):
    src = open(os.path.join(ref, "scisimtests", "narrowphase_tests.cpp")).read()
    bodies = re.split(r"static int executeCCDTest(\d\d)\(\)", src)[1:]
    cases = []
    for idx in range(0, len(bodies), 2):
        num, body = bodies[idx], bodies[idx + 1]
        body = body.split("int main(")[0]

        def vec(name):
            m = re.search(r"const Vector2s %s\{ %s, %s \};" % (name, _num, _num), body)
            return [float(m.group(1)), float(m.group(2))]

        def sc(name):
            m = re.search(r"constexpr scalar %s\{ %s \};" % (name, _num), body)
            return float(m.group(1)) if m else None

        case = dict(name="ball_ball_ccd_" + num, q0a=vec("q0a"), q1a=vec("q1a"), ra=sc("ra"),
                    q0b=vec("q0b"), q1b=vec("q1b"), rb=sc("rb"))
        m = re.search(r"const Vector3s cexpected\{ %s, %s, %s \};" % (_num, _num, _num), body)
        case["cexpected"] = [float(m.group(i)) for i in (1, 2, 3)] if m else None
        case["hit"] = "Collision incorrectly missed" in body
        # expected collision time, as an expression of the test source
        t = None
        m = re.search(r"collision_happens\.second != 0\.0", body)
        if m:
            t = "0.0"
        m = re.search(r"fabs\( collision_happens\.second - (.*?) \) > 1\.0e-9", body)
        if m:
            t = m.group(1)
        m = re.search(r"fabs\( collision_happens\.second \) > 1\.0e-9", body)
        if m:
            t = "0.0"
        ct = sc("collision_time")
        if ct is not None:
            t = repr(ct)
        case["time_expr"] = t
        case["time_tol"] = 1.0e-7 if ct is not None else 1.0e-9
        cases.append(case)
    return cases


def extract_slope_scenes(ref):
    cm = open(os.path.join(ref, "ball2dcli", "CMakeLists.txt")).read()
    scenes = []
    for m in re.finditer(r"add_test\( (ball2d_(?:st_)?(static|sliding)_friction_\w+) assets/shell_scripts/\w+\.sh "
                         r"assets/(tests_(?:friction|st)/\S+\.xml) ([0-9.]+) (\d+) (\S+) (\S+) (\S+) (\S+) \)", cm):
        name, kind, rel, end_time, freq = m.group(1), m.group(2), m.group(3), m.group(4), m.group(5)
        tols = [float(m.group(i)) for i in (6, 7, 8, 9)]
        xml = open(os.path.join(ref, "assets", "ball2d", rel)).read()

        def attr(tag, name, default=None):
            mm = re.search(r"<%s[^>]*\s%s=\"([^\"]*)\"" % (tag, name), xml)
            return mm.group(1) if mm else default

        px = [float(t) for t in attr("static_plane", "x").split()]
        pn = [float(t) for t in attr("static_plane", "n").split()]
        scenes.append(dict(
            name=name, kind=kind, xml="assets/ball2d/" + rel, end_time=float(end_time),
            output_frequency=int(freq), tolerances=tols,
            integrator=attr("integrator", "type"), dt=float(attr("integrator", "dt")),
            mu=float(attr("sobogus_friction_solver", "mu")), CoR=float(attr("sobogus_friction_solver", "CoR")),
            max_iters=int(attr("sobogus_friction_solver", "max_iters")),
            tol=float(attr("sobogus_friction_solver", "tol")),
            eval_every=int(attr("sobogus_friction_solver", "eval_every")),
            staggering=attr("sobogus_friction_solver", "staggering"),
            cache_impulses=attr("sobogus_friction_solver", "cache_impulses"),
            stabilization=int(attr("sobogus_friction_solver", "stabilization", "0")),
            penetration_threshold=float(attr("sobogus_friction_solver", "penetration_threshold", "0")),
            gravity=[float(attr("gravity", "fx")), float(attr("gravity", "fy"))],
            plane_x=px, plane_n=pn,
            ball=dict(x=float(attr("ball", "x")), y=float(attr("ball", "y")), vx=float(attr("ball", "vx")),
                      vy=float(attr("ball", "vy")), m=float(attr("ball", "m")), r=float(attr("ball", "r")))))
    return scenes


def extract_sphere_inertia(ref):
    src = open(os.path.join(ref, "rigidbody3dtests", "rigidbody3d_inertia_tests.cpp")).read()
    body = src.split("static int testSpherePoolBreak()")[1].split("static int")[0]
    r = re.search(r"RigidBodySphere sphere\{ %s \};" % _num, body).group(1)
    rho = re.search(r"computeMassAndInertia\( %s," % _num, body).group(1)
    M, tolM = re.search(r"fabs\( M - %s \) > %s" % (_num, _num), body).groups()
    I, tolI = re.search(r"Vector3s::Constant\( %s \) \)\.lpNorm<Eigen::Infinity>\(\) > %s" % (_num, _num),
                        body).groups()
    return [dict(r=float(r), density=float(rho), M=float(M), I=float(I), tol_M=float(tolM), tol_I=float(tolI))]


def extract_rigidbody2d_scenes(ref):
    import glob

    from scisim_gb300 import scene_io
    base = os.path.join(ref, "assets", "rigidbody2d")
    out = []
    for f in sorted(glob.glob(os.path.join(base, "**", "*.xml"), recursive=True)):
        try:
            sc = scene_io.load_rigidbody2d_scene(f)
        except scene_io.SceneError:
            continue
        d = {k: (v.tolist() if isinstance(v, np.ndarray) else v) for k, v in sc.items()
             if k not in ("dt_rational", "end_time")}
        d["gravity"] = list(sc["gravity"])
        d["xml"] = "assets/rigidbody2d/" + os.path.relpath(f, base)
        out.append(d)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    args = ap.parse_args()
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from oracle import oracle  # the oracle computes the all-pairs criterion

    arrays = extract_aabb_arrays(args.ref)
    expected = {}
    for name, toks in sorted(arrays.items()):
        tag = name.split("_")[1]
        path = os.path.join(HERE, "aabb2d_fixture_%s.txt.gz" % tag)
        with gzip.GzipFile(path, "wb", mtime=0) as fh:
            fh.write(("\n".join(toks) + "\n").encode())
        aabb = np.array([float(t) for t in toks]).reshape(-1, 4)
        pairs = oracle.allpairs_overlaps_2d(aabb)
        expected[tag] = dict(n_aabbs=int(aabb.shape[0]), n_pairs=int(pairs.shape[0]),
                             sha256=pairset_digest(pairs))
    with open(os.path.join(HERE, "aabb2d_expected.json"), "w") as fh:
        json.dump(expected, fh, indent=1, sort_keys=True)
    with open(os.path.join(HERE, "ccd_cases.json"), "w") as fh:
        json.dump(extract_ccd_cases(args.ref), fh, indent=1)
    with open(os.path.join(HERE, "slope_scenes.json"), "w") as fh:
        json.dump(extract_slope_scenes(args.ref), fh, indent=1)
    with open(os.path.join(HERE, "sphere_inertia.json"), "w") as fh:
        json.dump(extract_sphere_inertia(args.ref), fh, indent=1)
    with open(os.path.join(HERE, "rigidbody2d_scenes.json"), "w") as fh:
        json.dump(extract_rigidbody2d_scenes(args.ref), fh)


if __name__ == "__main__":
    main()
