"""Reader of SCISim's XML scene files, for the scenes this library steps.

Ball2D (`<ball2d_scene>`, ball2dutils/Ball2DSceneParser.cpp) and RigidBody3D sphere scenes
(`<rigidbody3d_scene>`, rigidbody3dutils/RigidBody3DSceneParser.cpp) with the elements of the contact
path: integrator, `sobogus_friction_solver` with geometric staggering (and, for Ball2D, the
symplectic_euler and stabilized staggerings), gravity, static planes, balls or spheres.  Values are read the way the reference reads them: scalars as C++ stream extraction of
a decimal (Python's float of the same text rounds the same way), the time step as an exact rational
(`Rational<intmax_t>` from a decimal or `a/b`, Rational.h:204-260) taken as numerator / denominator.
Elements of features outside the contact path (drums, portals, penalty forces, other solvers and
staggerings, fixed bodies, scripting) raise SceneError naming them, instead of being dropped.
"""
from __future__ import annotations

import math
import os
import re
import xml.etree.ElementTree as ET
from fractions import Fraction

import numpy as np

from . import scenes

CACHE_MODES = {"none": 0, "normal": 1, "normal_and_friction": 2}


class SceneError(ValueError):
    pass


def _root(source):
    if isinstance(source, (str, os.PathLike)) and os.path.exists(source):
        return ET.parse(source).getroot()
    return ET.fromstring(source)


def _attr(node, name, tag):
    v = node.get(name)
    if v is None:
        raise SceneError("%s: missing attribute %s" % (tag, name))
    return v


_MANTISSA = re.compile(r"\s*[+-]?(?:[0-9]+(?:\.[0-9]*)?|\.[0-9]+)")
_EXPONENT = re.compile(r"[eE][+-]?[0-9]+")


def stream_double(text: str):
    """`std::stringstream >> double` (StringUtilities.h:64-69): leading whitespace skipped, the
    longest decimal prefix read and the rest ignored; an exponent marker without digits fails, as
    the whole accumulated token must convert.  Returns None on failure."""
    m = _MANTISSA.match(text)
    if m is None:
        return None
    end = m.end()
    if end < len(text) and text[end] in "eE":
        e = _EXPONENT.match(text, end)
        if e is None:
            return None
        end = e.end()
    return float(text[:end])


def _scalar(node, name, tag):
    v = stream_double(_attr(node, name, tag))
    if v is None:
        raise SceneError("%s: %s is not a scalar" % (tag, name))
    return v


def _vector(node, name, n, tag):
    """readScalarList with a space delimiter (StringUtilities.h:92-112): exactly n tokens between
    single spaces (StringUtilities.cpp:123-142: a doubled or trailing space makes an empty token),
    each read by extractScalarFromString, which also takes "inf" and "-inf"."""
    text = _attr(node, name, tag)
    tokens = text.split(" ")  # the reference's tokenizer gives the same tokens
    if len(tokens) != n:
        raise SceneError("%s: %s needs %d scalars" % (tag, name, n))
    out = []
    for t in tokens:
        v = stream_double(t)
        if v is None:
            v = {"-inf": -math.inf, "inf": math.inf}.get(t)
        if v is None:
            raise SceneError("%s: %s needs %d scalars" % (tag, name, n))
        out.append(v)
    return out


def _bool(node, name, tag):
    v = _attr(node, name, tag).strip()
    if v not in ("0", "1"):
        raise SceneError("%s: %s must be 0 or 1" % (tag, name))
    return v == "1"


def _stream_int(text: str, what: str) -> int:
    """`std::stringstream >> integer` on whitespace-free text: an optional sign and at least one
    digit at the start; anything after the digits is ignored (StringUtilities.h:64-69)."""
    m = re.match(r"[+-]?[0-9]+", text)
    if m is None:
        raise SceneError("%s: malformed rational %r" % (what, text))
    return int(m.group(0))


def rational(text: str, what: str = "dt") -> Fraction:
    """Rational<intmax_t> extraction as scisim/Math/Rational.h:203-260 does it: at most one slash
    or one period; whitespace removed; `a/b` as two integers; otherwise split at the last period,
    trailing zeros of the fraction digits dropped, an empty or bare-sign integer part read as 0,
    and the fraction digits added with the integer part's sign (so "-0.5" reads as +1/2 there,
    as in the reference).  Exact; the caller converts with numerator / denominator."""
    slashes, periods = text.count("/"), text.count(".")
    if slashes > 2 or periods > 2 or (slashes == 1 and periods != 0) or (periods == 1 and slashes != 0):
        raise SceneError("%s: malformed rational %r" % (what, text))
    t = "".join(text.split())
    if slashes != 1:
        pos = t.rfind(".")
        left, right = (t, "") if pos < 0 else (t[:pos], t[pos + 1:])
        right = right.rstrip("0")
        left = {"": "0", "+": "+0", "-": "-0"}.get(left, left)
        li = _stream_int(left, what)
        ri = _stream_int(right, what) if right else 0
        den = 10 ** len(right)
        num = li * den + (-1 if li < 0 else 1) * ri
    else:
        pos = t.rfind("/")
        num, den = _stream_int(t[:pos], what), _stream_int(t[pos + 1:], what)
    if den == 0:
        raise SceneError("%s: zero denominator in %r" % (what, text))
    return Fraction(num, den)


def _check_tags(root, allowed):
    bad = sorted({c.tag for c in root} - set(allowed))
    if bad:
        raise SceneError("unsupported scene elements for this library's contact path: " + ", ".join(bad))


def _solver(root, tag_3d=False):
    nodes = root.findall("sobogus_friction_solver")
    if len(nodes) != 1:
        raise SceneError("needs exactly one sobogus_friction_solver")
    nd = nodes[0]
    tag = "sobogus_friction_solver"
    stag = _attr(nd, "staggering", tag)
    allowed = ("geometric", "symplectic_euler") if tag_3d else ("geometric", "symplectic_euler", "stabilized")
    if stag not in allowed:
        raise SceneError("%s: staggering %r is not supported (%s)" % (tag, stag, ", ".join(allowed)))
    cache = _attr(nd, "cache_impulses", tag)
    if cache not in CACHE_MODES:
        raise SceneError("%s: cache_impulses must be none, normal or normal_and_friction" % tag)
    out = dict(mu=_scalar(nd, "mu", tag), CoR=_scalar(nd, "CoR", tag), tol=_scalar(nd, "tol", tag),
               max_iters=int(_attr(nd, "max_iters", tag)), eval_every=int(_attr(nd, "eval_every", tag)),
               cache_mode=CACHE_MODES[cache])
    out["staggering"] = stag
    if stag == "stabilized" and out["cache_mode"] != 0:
        # Ball2DSceneParser.cpp:1400-1408
        raise SceneError("%s: the stabilized staggering keeps no impulse cache" % tag)
    if stag == "symplectic_euler":
        # Ball2DSceneParser.cpp:1354-1398: CoR must be 0; stabilization and its threshold.
        if out["CoR"] != 0.0:
            raise SceneError("%s: CoR must be 0 for the symplectic_euler staggering" % tag)
        out["stabilization"] = _bool(nd, "stabilization", tag)
        out["penetration_threshold"] = _scalar(nd, "penetration_threshold", tag)
        if out["penetration_threshold"] < 0.0:
            raise SceneError("%s: penetration_threshold must be non-negative" % tag)
    if tag_3d and stag == "geometric":
        out["cache_mode"] = 0  # the 3D geometric map keeps no cache (RigidBody3DSceneParser.cpp:1877-1880)
    return out


def _dt(root, types):
    nodes = root.findall("integrator")
    if len(nodes) != 1:
        raise SceneError("needs exactly one integrator")
    nd = nodes[0]
    kind = _attr(nd, "type", "integrator")
    if kind not in types:
        raise SceneError("integrator type %r is not supported (%s)" % (kind, ", ".join(types)))
    dt = rational(_attr(nd, "dt", "integrator"))
    if dt <= 0:
        raise SceneError("integrator: dt must be positive")
    return kind, dt


def _end_time(root):
    nd = root.find("end_time")
    return None if nd is None else _scalar(nd, "t", "end_time")


def load_ball2d_scene(source) -> dict:
    """A `<ball2d_scene>` file or text as arrays and settings (Ball2DSceneParser.cpp:1486-1651).
    Returns q, v (2 per ball), r, m, plane_x, plane_n (2 per plane), dt (float) and dt_rational,
    integrator ('verlet' / 'symplectic_euler'), gravity, mu, CoR, tol, max_iters, eval_every,
    cache_mode, end_time (None if absent)."""
    root = _root(source)
    if root.tag != "ball2d_scene":
        raise SceneError("not a ball2d_scene")
    _check_tags(root, ("camera", "end_time", "integrator", "sobogus_friction_solver", "gravity", "static_plane",
                       "ball"))
    kind, dt = _dt(root, ("verlet", "symplectic_euler"))
    grav = root.findall("gravity")
    if len(grav) > 1:
        raise SceneError("more than one gravity force (their sum would round differently)")
    g = (0.0, 0.0) if not grav else (_scalar(grav[0], "fx", "gravity"), _scalar(grav[0], "fy", "gravity"))
    px, pn = [], []
    for nd in root.findall("static_plane"):
        px.append(_vector(nd, "x", 2, "static_plane"))
        pn.append(_vector(nd, "n", 2, "static_plane"))
    q, v, r, m = [], [], [], []
    for nd in root.findall("ball"):
        if _bool(nd, "fixed", "ball"):
            raise SceneError("ball: fixed balls are not supported")
        q += [_scalar(nd, "x", "ball"), _scalar(nd, "y", "ball")]
        v += [_scalar(nd, "vx", "ball"), _scalar(nd, "vy", "ball")]
        m.append(_scalar(nd, "m", "ball"))
        r.append(_scalar(nd, "r", "ball"))
    out = dict(q=np.array(q, np.float64), v=np.array(v, np.float64), r=np.array(r, np.float64),
               m=np.array(m, np.float64), plane_x=np.array(px, np.float64).reshape(-1, 2),
               plane_n=np.array(pn, np.float64).reshape(-1, 2), dt=float(dt), dt_rational=dt, integrator=kind,
               gravity=g, end_time=_end_time(root))
    out.update(_solver(root))
    return out


def load_rigidbody2d_scene(source) -> dict:
    """A `<rigidbody2d_scene>` of circles as arrays and settings (RigidBody2DSceneParser.cpp), for
    the geometric or stabilized staggering: `rigid_body` elements with a circle geometry, mass and inertia from
    rho (CircleGeometry::computeMassAndInertia, rigidbody2d/CircleGeometry.cpp:29-33: m = rho pi r^2,
    I = m r^2 / 2).  Returns q, v (3 per body: x, y, theta / vx, vy, omega), r, m, I, plane_x,
    plane_n (2 per plane), dt, dt_rational, integrator, gravity, the solver settings and end_time.
    Boxes, fixed bodies, portals and scripting are rejected by name.  The library steps these
    scenes only through the oracle so far (no GPU path for RigidBody2D)."""
    root = _root(source)
    if root.tag != "rigidbody2d_scene":
        raise SceneError("not a rigidbody2d_scene")
    _check_tags(root, ("camera", "end_time", "integrator", "sobogus_friction_solver", "near_earth_gravity",
                       "static_plane", "geometry", "rigid_body"))
    kind, dt = _dt(root, ("verlet", "symplectic_euler"))
    grav = root.findall("near_earth_gravity")
    if len(grav) > 1:
        raise SceneError("more than one near_earth_gravity force")
    g = (0.0, 0.0) if not grav else tuple(_vector(grav[0], "f", 2, "near_earth_gravity"))
    px, pn = [], []
    for nd in root.findall("static_plane"):
        px.append(_vector(nd, "x", 2, "static_plane"))
        pn.append(_vector(nd, "n", 2, "static_plane"))
    radii = []
    for nd in root.findall("geometry"):
        if _attr(nd, "type", "geometry") != "circle":
            raise SceneError("geometry: only circles are supported")
        radii.append(_scalar(nd, "r", "geometry"))
    q, v, r, m, inertia = [], [], [], [], []
    for nd in root.findall("rigid_body"):
        tag = "rigid_body"
        if nd.get("fixed") is not None and _bool(nd, "fixed", tag):
            raise SceneError("%s: fixed bodies are not supported" % tag)
        k = int(_attr(nd, "geo_idx", tag))
        if not 0 <= k < len(radii):
            raise SceneError("%s: invalid geo_idx" % tag)
        rho = _scalar(nd, "rho", tag)
        if not rho > 0.0:
            raise SceneError("%s: rho must be positive" % tag)
        x, vel = _vector(nd, "x", 2, tag), _vector(nd, "v", 2, tag)
        q += [x[0], x[1], _scalar(nd, "theta", tag)]
        v += [vel[0], vel[1], _scalar(nd, "omega", tag)]
        rk = radii[k]
        mk = rho * math.pi * rk * rk
        r.append(rk)
        m.append(mk)
        inertia.append(0.5 * mk * rk * rk)
    solver = _solver(root)
    if solver["staggering"] not in ("geometric", "stabilized"):
        # RigidBody2DSceneParser.cpp:1054-1061 knows these two
        raise SceneError("sobogus_friction_solver: rigidbody2d takes the geometric or stabilized staggering")
    out = dict(q=np.array(q, np.float64), v=np.array(v, np.float64), r=np.array(r, np.float64),
               m=np.array(m, np.float64), I=np.array(inertia, np.float64),
               plane_x=np.array(px, np.float64).reshape(-1, 2), plane_n=np.array(pn, np.float64).reshape(-1, 2),
               dt=float(dt), dt_rational=dt, integrator=kind, gravity=g, end_time=_end_time(root))
    out.update(solver)
    return out


def load_rigidbody3d_scene(source) -> dict:
    """A `<rigidbody3d_scene>` of spheres as arrays and settings (RigidBody3DSceneParser.cpp), for
    the geometric staggering with the split_ham integrator, or the symplectic_euler staggering
    (whose map does not call the integrator, so `dmv` is accepted there; the GPU library and the
    oracle step both).  Bodies: `rigid_body_with_density` with a
    sphere geometry, mass and inertia from rho (RigidBodySphere::computeMassAndInertia), identity
    orientation (an `R` attribute, an Eigen AngleAxis, is not supported).  Returns q = [x | R],
    v = [v | omega], r, m, I0, plane_x, plane_n (3 per plane), dt, gravity and the solver settings."""
    root = _root(source)
    if root.tag != "rigidbody3d_scene":
        raise SceneError("not a rigidbody3d_scene")
    _check_tags(root, ("camera_perspective", "camera_orthographic", "end_time", "integrator",
                       "sobogus_friction_solver", "near_earth_gravity", "static_plane", "geometry",
                       "rigid_body_with_density", "static_plane_renderer"))
    kind, dt = _dt(root, ("split_ham", "dmv"))
    grav = root.findall("near_earth_gravity")
    if len(grav) > 1:
        raise SceneError("more than one near_earth_gravity force")
    g = (0.0, 0.0, 0.0) if not grav else tuple(_vector(grav[0], "f", 3, "near_earth_gravity"))
    px, pn = [], []
    for nd in root.findall("static_plane"):
        px.append(_vector(nd, "x", 3, "static_plane"))
        pn.append(_vector(nd, "n", 3, "static_plane"))
    geos = []
    for nd in root.findall("geometry"):
        if _attr(nd, "type", "geometry") != "sphere":
            raise SceneError("geometry: only spheres are supported")
        geos.append(_scalar(nd, "r", "geometry"))
    xs, vs, ws, rs, rhos = [], [], [], [], []
    for nd in root.findall("rigid_body_with_density"):
        tag = "rigid_body_with_density"
        if _bool(nd, "fixed", tag):
            raise SceneError("%s: fixed bodies are not supported" % tag)
        if nd.get("R") is not None:
            raise SceneError("%s: an initial orientation (R) is not supported" % tag)
        gi = int(_attr(nd, "geo_idx", tag))
        if gi < 0:
            gi += len(geos)
        if not 0 <= gi < len(geos):
            raise SceneError("%s: invalid geo_idx" % tag)
        xs.append(_vector(nd, "x", 3, tag))
        vs.append(_vector(nd, "v", 3, tag))
        ws.append(_vector(nd, "omega", 3, tag))
        rs.append(geos[gi])
        rhos.append(_scalar(nd, "rho", tag))
    n = len(xs)
    r = np.array(rs, np.float64)
    m = np.empty(n)
    i0 = np.empty(n)
    for k in range(n):
        mk, ik = scenes.sphere_mass_inertia(np.array([r[k]]), rhos[k])
        m[k], i0[k] = mk[0], ik[0]
    x = np.array(xs, np.float64).reshape(-1) + 0.0  # x + CM with CM = 0 for a sphere
    q = np.concatenate([x, np.tile(np.eye(3).reshape(-1), n)])
    v = np.concatenate([np.array(vs, np.float64).reshape(-1), np.array(ws, np.float64).reshape(-1)])
    out = dict(q=q, v=v, r=r, m=m, I0=np.repeat(i0, 3), plane_x=np.array(px, np.float64).reshape(-1, 3),
               plane_n=np.array(pn, np.float64).reshape(-1, 3), dt=float(dt), dt_rational=dt, integrator=kind,
               gravity=g, end_time=_end_time(root))
    out.update(_solver(root, tag_3d=True))
    if out["staggering"] == "geometric" and kind != "split_ham":
        # the geometric map runs the integrator; only SplitHamMap is built for spheres
        raise SceneError("integrator: the geometric staggering of spheres takes split_ham")
    return out


def steps_to(end_time: float, dt: Fraction) -> int:
    """Steps a driver takes to reach end_time (ceil of end_time / dt in exact arithmetic)."""
    return int(math.ceil(Fraction(end_time) / dt))


def ball2d_objects(scene: dict):
    """The reference's objects for a loaded Ball2D scene, as ball2d_cli builds them: the simulation,
    its unconstrained map, the Sobogus solver and the geometric impact-friction map.  Step with
    sim.flow(iteration, scene['dt'], umap, scene['CoR'], scene['mu'], solver, ifmap)."""
    from .ball2d import (Ball2DSim, Ball2DState, GeometricImpactFrictionMap, ImpulsesToCache, Sobogus,
                         SobogusSolverType, StabilizedImpactFrictionMap, StaticPlane, SymplecticEulerImpactFrictionMap,
                         SymplecticEulerMap, VerletMap)
    planes = [StaticPlane(x, n) for x, n in zip(scene["plane_x"], scene["plane_n"])]
    sim = Ball2DSim(Ball2DState(scene["q"], scene["v"], scene["r"], scene["m"], planes), gravity=scene["gravity"])
    umap = VerletMap() if scene["integrator"] == "verlet" else SymplecticEulerMap()
    solver = Sobogus(SobogusSolverType.Balls2D, eval_every=scene["eval_every"])
    if scene.get("staggering") == "stabilized":
        ifmap = StabilizedImpactFrictionMap(scene["tol"], scene["max_iters"])
    elif scene.get("staggering") == "symplectic_euler":
        ifmap = SymplecticEulerImpactFrictionMap(scene["tol"], scene["max_iters"], ImpulsesToCache(scene["cache_mode"]),
                                                 scene["stabilization"], scene["penetration_threshold"])
    else:
        ifmap = GeometricImpactFrictionMap(scene["tol"], scene["max_iters"], ImpulsesToCache(scene["cache_mode"]))
    return sim, umap, solver, ifmap


def rigidbody3d_objects(scene: dict):
    """As ball2d_objects for a loaded sphere scene: SplitHamMap and the geometric map without an
    impulse cache, or the symplectic-Euler map with the scene's cache and stabilisation (that map
    integrates by exponential Euler whatever the integrator)."""
    from .ball2d import (GeometricImpactFrictionMap, ImpulsesToCache, Sobogus, SobogusSolverType,
                         SymplecticEulerImpactFrictionMap)
    from .rigidbody3d import RigidBody3DSim, RigidBody3DState, SplitHamMap, StaticPlane
    stag = scene.get("staggering", "geometric")
    if stag not in ("geometric", "symplectic_euler"):
        raise SceneError("the GPU library steps spheres with the geometric or the symplectic_euler staggering")
    planes = [StaticPlane(x, n) for x, n in zip(scene["plane_x"], scene["plane_n"])]
    state = RigidBody3DState(scene["q"], scene["v"], scene["r"], scene["m"], scene["I0"], planes)
    sim = RigidBody3DSim(state, gravity=scene["gravity"])
    solver = Sobogus(SobogusSolverType.RigidBodies3D, eval_every=scene["eval_every"])
    if stag == "symplectic_euler":
        ifmap = SymplecticEulerImpactFrictionMap(scene["tol"], scene["max_iters"], ImpulsesToCache(scene["cache_mode"]),
                                                 scene["stabilization"], scene["penetration_threshold"])
    else:
        ifmap = GeometricImpactFrictionMap(scene["tol"], scene["max_iters"], ImpulsesToCache.NONE)
    return sim, SplitHamMap(), solver, ifmap
