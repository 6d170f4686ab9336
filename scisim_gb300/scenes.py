"""Seeded synthetic Ball2D scenes of the benchmark configurations.

No public dataset is involved: every scene is generated from a fixed seed.

  box_drop_1024   1,024 discs, r ~ U[0.04, 0.06], density 1, 32 x 32 lattice of
                  spacing 0.13 with U[-0.01, 0.01] jitter, v ~ N(0, 0.1^2), static
                  planes bounding [-2.5, 2.5] x [0, inf) (floor, two walls, and a lid
                  far above), gravity (0, -9.81), symplectic Euler dt 0.01, CoR 0.3,
                  mu 0.5, tol 1e-9, 5,000 iterations
  dense_pile      262,144 discs, r log-uniform [0.02, 0.06], density 1, non-overlapping
                  fill of a 40 x 60 box (area fraction ~0.5) built by size-sorted
                  shelf packing with random slack, rows shuffled, bodies permuted;
                  four walls; gravity -9.81, dt 0.005, CoR 0, mu 0.4
  hopper          262,144 discs, radii U[0.02, 0.05], filled above a V-wedge of two planes
                  at +-30 deg from the vertical (infinite planes: no outlet), mu 0.5, CoR 0.1,
                  dt 0.005
  ball2d_batch    4,096 independent Ball2D scenes of 16-4,096 discs (log-uniform), radii
                  U[0.03, 0.05], per-scene mu U[0.1, 0.8] and CoR U[0, 0.5], dt 0.01
  sphere_pile     65,536 spheres, r ~ U[0.05, 0.1], density 1, jittered lattice of spacing
                  0.2 filling a 6 x 6 footprint (volume fraction ~0.18 of a 6 x 6 x 20
                  box), v ~ N(0, 0.1^2), omega ~ N(0, 1), identity orientations; floor
                  and four walls; gravity (0, -9.81, 0), split-Hamiltonian dt 0.004,
                  CoR 0.2, mu 0.6
"""
from __future__ import annotations

import math

import numpy as np


def box_drop_1024(seed: int = 1, n_side: int = 32):
    rng = np.random.default_rng(seed)
    n = n_side * n_side
    r = rng.uniform(0.04, 0.06, n)
    m = math.pi * r * r  # density 1
    ix, iy = np.meshgrid(np.arange(n_side), np.arange(n_side), indexing="xy")
    x = (ix.reshape(-1) - (n_side - 1) / 2.0) * 0.13 + rng.uniform(-0.01, 0.01, n)
    y = 0.1 + iy.reshape(-1) * 0.13 + rng.uniform(-0.01, 0.01, n)
    q = np.stack([x, y], axis=1).reshape(-1)
    v = rng.normal(0.0, 0.1, 2 * n)
    plane_x = np.array([[0.0, 0.0], [-2.5, 0.0], [2.5, 0.0], [0.0, 1000.0]])
    plane_n = np.array([[0.0, 1.0], [1.0, 0.0], [-1.0, 0.0], [0.0, -1.0]])
    return dict(q=q, v=v, r=r, m=m, plane_x=plane_x, plane_n=plane_n, dt=0.01, gravity=(0.0, -9.81), CoR=0.3,
                mu=0.5, tol=1e-9, max_iters=5000, name="box_drop_1024")


def dense_pile(n: int = 262144, seed: int = 2, width: float = 40.0, height: float = 60.0, rmin: float = 0.02,
               rmax: float = 0.06, radii: str = "loguniform"):
    """Non-overlapping polydisperse fill of a width x height box (walls at x = +-width/2, floor y = 0)."""
    rng = np.random.default_rng(seed)
    if radii == "uniform":
        r = rng.uniform(rmin, rmax, n)
    else:
        r = np.exp(rng.uniform(math.log(rmin), math.log(rmax), n))
    order = np.argsort(-r, kind="stable")
    rs = r[order]
    # Shelf packing of the size-sorted discs: rows of similar radii.
    rows = []
    i = 0
    gap = 0.002
    while i < n:
        w = 0.0
        j = i
        while j < n and w + 2.0 * rs[j] + gap <= width:
            w += 2.0 * rs[j] + gap
            j += 1
        if j == i:
            raise ValueError("disc wider than the box")
        rows.append((i, j, w))
        i = j
    heights = np.array([2.0 * rs[a] + gap for a, _, _ in rows])
    slack_y = height - heights.sum()
    if slack_y < 0:
        raise ValueError("discs do not fit in the box")
    row_order = rng.permutation(len(rows))
    vgaps = rng.dirichlet(np.ones(len(rows) + 1)) * slack_y
    pos = np.empty((n, 2))
    y = vgaps[0]
    for k, ri in enumerate(row_order):
        a, b, w = rows[ri]
        hrow = heights[ri]
        cnt = b - a
        hgaps = rng.dirichlet(np.ones(cnt + 1)) * (width - w)
        x = -0.5 * width
        for t in range(cnt):
            rad = rs[a + t]
            x += hgaps[t] + 0.5 * gap + rad
            jit = rng.uniform(-1.0, 1.0) * (0.5 * hrow - 0.5 * gap - rad)
            pos[a + t] = (x, y + 0.5 * hrow + jit)
            x += rad + 0.5 * gap
        y += hrow + vgaps[k + 1]
    # Undo the size sort, then permute body indices.
    q = np.empty((n, 2))
    q[order] = pos
    perm = rng.permutation(n)
    q = q[perm]
    r = r[perm]
    m = math.pi * r * r
    v = np.zeros(2 * n)
    plane_x = np.array([[0.0, 0.0], [-0.5 * width, 0.0], [0.5 * width, 0.0], [0.0, height]])
    plane_n = np.array([[0.0, 1.0], [1.0, 0.0], [-1.0, 0.0], [0.0, -1.0]])
    return dict(q=q.reshape(-1), v=v, r=r, m=m, plane_x=plane_x, plane_n=plane_n, dt=0.005, gravity=(0.0, -9.81),
                CoR=0.0, mu=0.4, tol=1e-6, max_iters=5000, name="dense_pile_%d" % n)


def hopper(n: int = 262144, seed: int = 4, angle_deg: float = 30.0, outlet: float = 0.5):
    """Discs (radii U[0.02, 0.05], density 1) filled above a funnel of two static planes
    inclined angle_deg from the vertical whose lines pass through (+-outlet/2, 0).  SCISim's
    StaticPlane is an infinite line (ball2d/StaticGeometry/StaticPlane.cpp:10-23), so the two
    planes meet below the outlet and form a V-wedge with no opening.  mu 0.5, CoR 0.1,
    dt 0.005, gravity (0, -9.81)."""
    t = math.tan(math.radians(angle_deg))
    width = 30.0 * math.sqrt(n / 262144.0)
    height = 71.4 * math.sqrt(n / 262144.0)
    s = dense_pile(n=n, seed=seed, width=width, height=height, rmin=0.02, rmax=0.05, radii="uniform")
    y0 = max(0.0, (0.5 * width - 0.5 * outlet) / t) + 0.1
    q = s["q"].reshape(-1, 2).copy()
    q[:, 1] += y0
    c, sn = math.cos(math.radians(angle_deg)), math.sin(math.radians(angle_deg))
    plane_x = np.array([[-0.5 * outlet, 0.0], [0.5 * outlet, 0.0]])
    plane_n = np.array([[c, sn], [-c, sn]])
    return dict(q=q.reshape(-1), v=s["v"], r=s["r"], m=s["m"], plane_x=plane_x, plane_n=plane_n, dt=0.005,
                gravity=(0.0, -9.81), CoR=0.1, mu=0.5, tol=1e-6, max_iters=5000, name="hopper_%d" % n)


def ball2d_batch(n_scenes: int = 4096, seed: int = 3, nmin: int = 16, nmax: int = 4096, rmin: float = 0.03,
                 rmax: float = 0.05, spacing: float = 0.11):
    """Independent Ball2D scenes: disc counts log-uniform in [nmin, nmax], radii U[rmin, rmax],
    density 1, a jittered square lattice per scene above its floor between two walls,
    v ~ N(0, 0.1^2), per-scene mu ~ U[0.1, 0.8] and CoR ~ U[0, 0.5]; symplectic Euler
    dt 0.01, gravity (0, -9.81).  Every scene lives in its own coordinates."""
    rng = np.random.default_rng(seed)
    counts = np.rint(np.exp(rng.uniform(math.log(nmin), math.log(nmax), n_scenes))).astype(np.int64)
    body_off = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
    plane_off = (3 * np.arange(n_scenes + 1)).astype(np.int32)
    N = int(body_off[-1])
    q = np.empty((N, 2))
    r = rng.uniform(rmin, rmax, N)
    px = np.empty((3 * n_scenes, 2))
    pn = np.empty((3 * n_scenes, 2))
    jit = 0.5 * spacing - rmax - 1e-3
    for s in range(n_scenes):
        n = int(counts[s])
        side = int(math.ceil(math.sqrt(n)))
        k = np.arange(n)
        ix, iy = k % side, k // side
        x = (ix - 0.5 * (side - 1)) * spacing + rng.uniform(-jit, jit, n)
        y = 0.5 * spacing + iy * spacing + rng.uniform(-jit, jit, n)
        q[body_off[s]:body_off[s + 1]] = np.stack([x, y], 1)
        half = 0.5 * side * spacing + 0.05
        px[3 * s:3 * s + 3] = [[0.0, 0.0], [-half, 0.0], [half, 0.0]]
        pn[3 * s:3 * s + 3] = [[0.0, 1.0], [1.0, 0.0], [-1.0, 0.0]]
    v = rng.normal(0.0, 0.1, 2 * N)
    mu = rng.uniform(0.1, 0.8, n_scenes)
    CoR = rng.uniform(0.0, 0.5, n_scenes)
    return dict(body_off=body_off, plane_off=plane_off, q=q.reshape(-1), v=v, r=r, m=math.pi * r * r,
                plane_x=px, plane_n=pn, mu=mu, CoR=CoR, dt=0.01, gravity=(0.0, -9.81), tol=1e-6, max_iters=5000,
                name="ball2d_batch_%d" % n_scenes)


def batch_scene(b, s):
    """Scene s of a batch as a standalone Ball2D scene (local indices)."""
    b0, b1 = int(b["body_off"][s]), int(b["body_off"][s + 1])
    p0, p1 = int(b["plane_off"][s]), int(b["plane_off"][s + 1])
    return dict(q=b["q"][2 * b0:2 * b1], v=b["v"][2 * b0:2 * b1], r=b["r"][b0:b1], m=b["m"][b0:b1],
                plane_x=b["plane_x"][p0:p1], plane_n=b["plane_n"][p0:p1], mu=float(b["mu"][s]),
                CoR=float(b["CoR"][s]), dt=b["dt"], gravity=b["gravity"])


def sphere_mass_inertia(r, density=1.0):
    """Mass and principal moment of solid spheres, in the operation order of
    RigidBodySphere::computeMassAndInertia (rigidbody3d/Geometry/RigidBodySphere.cpp:10-18)."""
    r = np.asarray(r, dtype=np.float64)
    m = 4.0 * math.pi * r * r * r / 3.0
    i = 2.0 * m * r * r / 5.0
    return m * density, i * density


def sphere_pile(n: int = 65536, seed: int = 5, width: float = 6.0, depth: float = 6.0, rmin: float = 0.05,
                rmax: float = 0.1, spacing: float = 0.2):
    """Spheres on a jittered lattice above the floor y = 0 inside walls x in [0, width],
    z in [0, depth].  Lattice sites are `spacing` apart and every sphere stays inside its
    site's cube, so the initial configuration has no overlaps."""
    if 2.0 * rmax > spacing:
        raise ValueError("sphere wider than a lattice site")
    rng = np.random.default_rng(seed)
    nx, nz = int(width / spacing), int(depth / spacing)
    per_layer = nx * nz
    layers = -(-n // per_layer)
    idx = np.arange(n)
    iy, rem = np.divmod(idx, per_layer)
    iz, ix = np.divmod(rem, nx)
    r = rng.uniform(rmin, rmax, n)
    slack = 0.5 * spacing - r - 1e-4
    centre = np.stack([(ix + 0.5) * spacing, (iy + 0.5) * spacing, (iz + 0.5) * spacing], axis=1)
    x = centre + rng.uniform(-1.0, 1.0, (n, 3)) * slack[:, None]
    perm = rng.permutation(n)
    x, r = x[perm], r[perm]
    m, i0 = sphere_mass_inertia(r)
    R = np.tile(np.eye(3).reshape(-1), n)
    q = np.concatenate([x.reshape(-1), R])
    v = np.concatenate([rng.normal(0.0, 0.1, 3 * n), rng.normal(0.0, 1.0, 3 * n)])
    plane_x = np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 0.0], [width, 0.0, 0.0], [0.0, 0.0, 0.0], [0.0, 0.0, depth]])
    plane_n = np.array([[0.0, 1.0, 0.0], [1.0, 0.0, 0.0], [-1.0, 0.0, 0.0], [0.0, 0.0, 1.0], [0.0, 0.0, -1.0]])
    del layers
    return dict(q=q, v=v, r=r, m=m, I0=np.repeat(i0, 3), plane_x=plane_x, plane_n=plane_n, dt=0.004,
                gravity=(0.0, -9.81, 0.0), CoR=0.2, mu=0.6, tol=1e-6, max_iters=5000, name="sphere_pile_%d" % n)


def sphere_batch(n_scenes: int = 256, seed: int = 4, nmin: int = 64, nmax: int = 1024):
    """Independent sphere piles (C5's batched configuration): sphere counts log-uniform in
    [nmin, nmax], each a sphere_pile of its own (footprint sized to about 8 layers), per-scene
    mu ~ U[0.2, 0.8] and CoR ~ U[0, 0.4]; SplitHam dt 0.004, gravity (0, -9.81, 0).  Every scene
    lives in its own coordinates.  q = [x (3N) | R (9N)], v = [v (3N) | omega (3N)] over all N."""
    rng = np.random.default_rng(seed)
    counts = np.rint(np.exp(rng.uniform(math.log(nmin), math.log(nmax), n_scenes))).astype(np.int64)
    body_off = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
    plane_off = (5 * np.arange(n_scenes + 1)).astype(np.int32)
    xs, Rs, vs, ws, rs, ms, i0s, px, pn = [], [], [], [], [], [], [], [], []
    for s in range(n_scenes):
        n = int(counts[s])
        side = max(2, int(math.ceil(math.sqrt(n / 8.0))))
        one = sphere_pile(n=n, seed=int(rng.integers(1 << 30)), width=0.2 * side, depth=0.2 * side)
        xs.append(one["q"][:3 * n])
        Rs.append(one["q"][3 * n:])
        vs.append(one["v"][:3 * n])
        ws.append(one["v"][3 * n:])
        rs.append(one["r"])
        ms.append(one["m"])
        i0s.append(one["I0"])
        px.append(one["plane_x"])
        pn.append(one["plane_n"])
    q = np.concatenate(xs + Rs)
    v = np.concatenate(vs + ws)
    mu = rng.uniform(0.2, 0.8, n_scenes)
    CoR = rng.uniform(0.0, 0.4, n_scenes)
    return dict(body_off=body_off, plane_off=plane_off, q=q, v=v, r=np.concatenate(rs), m=np.concatenate(ms),
                I0=np.concatenate(i0s), plane_x=np.concatenate(px), plane_n=np.concatenate(pn), mu=mu, CoR=CoR,
                dt=0.004, gravity=(0.0, -9.81, 0.0), tol=1e-6, max_iters=5000, name="sphere_batch_%d" % n_scenes)


def batch_scene3(b, s, q=None, v=None):
    """Scene s of a sphere batch as a standalone sphere scene (local layout and indices); q, v
    default to the batch's initial state."""
    q = b["q"] if q is None else q
    v = b["v"] if v is None else v
    N = int(b["body_off"][-1])
    b0, b1 = int(b["body_off"][s]), int(b["body_off"][s + 1])
    p0, p1 = int(b["plane_off"][s]), int(b["plane_off"][s + 1])
    qs = np.concatenate([q[3 * b0:3 * b1], q[3 * N + 9 * b0:3 * N + 9 * b1]])
    vs = np.concatenate([v[3 * b0:3 * b1], v[3 * N + 3 * b0:3 * N + 3 * b1]])
    return dict(q=qs, v=vs, r=b["r"][b0:b1], m=b["m"][b0:b1], I0=b["I0"][3 * b0:3 * b1],
                plane_x=b["plane_x"][p0:p1], plane_n=b["plane_n"][p0:p1], mu=float(b["mu"][s]),
                CoR=float(b["CoR"][s]), dt=b["dt"], gravity=b["gravity"])


def min_gap(q, r, plane_x=None, plane_n=None):
    """Smallest pairwise gap (brute force on a grid; for tests of the generators)."""
    q = np.asarray(q).reshape(-1, 2)
    n = q.shape[0]
    h = 2.0 * r.max()
    keys = np.floor(q / h).astype(np.int64)
    cells = {}
    for i, (a, b) in enumerate(keys):
        cells.setdefault((a, b), []).append(i)
    best = np.inf
    for (a, b), idx in cells.items():
        cand = []
        for da in (-1, 0, 1):
            for db in (-1, 0, 1):
                cand += cells.get((a + da, b + db), [])
        cand = np.array(cand)
        for i in idx:
            js = cand[cand > i]
            if js.size:
                d = np.sqrt(((q[js] - q[i]) ** 2).sum(1)) - r[js] - r[i]
                best = min(best, d.min())
    if plane_x is not None:
        for x, nn in zip(np.asarray(plane_x).reshape(-1, 2), np.asarray(plane_n).reshape(-1, 2)):
            d = (q - x) @ (nn / np.linalg.norm(nn)) - r
            best = min(best, d.min())
    return best
