"""The C++ host interface (include/scisim_gb300.hpp): the mirrored SCISim classes compiled with g++
against libscisim_gb300.so and run as a test program in the reference's manner
(tests/cpp/host_api_test.cpp, one test name per run, exit status as the result).

CPU: the reference's names, SG_BAD_INPUT for invalid settings and sizes before any GPU work, and
SG_CUDA_ERROR (not a crash, not a CPU path) where no GPU can be used.
GPU: a box drop stepped through Ball2DSim::flow with the geometric, symplectic-Euler and stabilized
maps gives, bit for bit, the states of the same steps through the C ABI.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from scisim_gb300 import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "host_api_test.cpp")


@pytest.fixture(scope="module")
def host_test(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    from scisim_gb300 import build
    lib = build.build()
    libdir = os.path.dirname(os.path.abspath(lib))
    exe = str(tmp_path_factory.mktemp("cpp") / "host_api_test")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"), SRC,
           "-L", libdir, "-lscisim_gb300", "-Wl,-rpath," + libdir, "-o", exe]
    p = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-3000:]
    return exe


def run(exe, *args, timeout=120):
    return subprocess.run([exe] + list(args), capture_output=True, text=True, timeout=timeout)


@pytest.mark.parametrize("name", ["names", "validation", "identity", "no_device"])
def test_host_api_cpu(host_test, name):
    p = run(host_test, name)
    assert p.returncode == 0, p.stderr


@pytest.mark.gpu
def test_host_api_ball2d_maps_match_c_abi(host_test, gpulib, tmp_path):
    s = scenes.box_drop_1024(seed=4, n_side=14)
    n, npl = s["r"].shape[0], np.asarray(s["plane_x"]).reshape(-1, 2).shape[0]
    steps, mu, tol, max_iters = 40, 0.5, 1e-9, 500
    g = s["gravity"]
    header = [n, npl, s["dt"], g[0], g[1], mu, tol, max_iters, steps]
    scene = np.concatenate([np.asarray(header, np.float64), s["q"], s["v"], s["r"], s["m"],
                            np.asarray(s["plane_x"], np.float64).reshape(-1),
                            np.asarray(s["plane_n"], np.float64).reshape(-1)])
    scene_file, out_file = tmp_path / "scene.bin", tmp_path / "out.bin"
    scene.astype("<f8").tofile(scene_file)
    p = run(host_test, "ball2d_run", str(scene_file), str(out_file), timeout=600)
    assert p.returncode == 0, p.stderr
    got = np.fromfile(out_file, dtype="<f8").reshape(3, 2, 2 * n)

    cases = [  # integrator, CoR, cache, staggering, stabilize, threshold
        (gpulib.VERLET, 0.3, gpulib.CACHE_NORMAL_AND_FRICTION, gpulib.STAGGER_GEOMETRIC, False, 0.0),
        (gpulib.SYMPLECTIC_EULER, 0.0, gpulib.CACHE_NORMAL_AND_FRICTION, gpulib.STAGGER_SYMPLECTIC_EULER, True, 1e-4),
        (gpulib.SYMPLECTIC_EULER, 0.3, gpulib.CACHE_NONE, gpulib.STAGGER_STABILIZED, False, 0.0),
    ]
    for k, (integ, CoR, cache, stag, stab, thr) in enumerate(cases):
        ctx = gpulib.Context(dt=s["dt"], gravity=g, mu=mu, CoR=CoR, tol=tol, max_iters=max_iters, eval_every=1,
                             integrator=integ, cache_mode=cache)
        ctx.upload_ball2d(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"])
        if stag != gpulib.STAGGER_GEOMETRIC:
            ctx.set_staggering(stag, stab, thr)
        q, v = np.array(s["q"], np.float64), np.array(s["v"], np.float64)
        for it in range(1, steps + 1):
            q, v, _ = ctx.flow(it, q, v)
        ctx.close()
        assert np.array_equal(got[k, 0], q) and np.array_equal(got[k, 1], v), k


@pytest.mark.gpu
def test_host_api_solves_with_extras_match_oracle(host_test, gpulib, oracle, tmp_path):
    """Sobogus::solve (Ball2D) and Sobogus::solve3D (spheres) of the C++ interface with non-zero
    nrel_extra / drel_extra, bit-exact with the oracle replaying the solve order each reports."""
    from test_gpu_friction_solver import ball2d_problem, sphere_problem

    rng = np.random.default_rng(11)
    s2, v0, ia, ib, bases = ball2d_problem(gpulib)
    nb2, nc2 = s2["r"].shape[0], ia.shape[0]
    p2 = dict(m=s2["m"], v0=v0, ia=ia.astype(np.float64), ib=ib.astype(np.float64), bases=bases,
              CoR=rng.uniform(0.0, 0.5, nc2), mu=np.full(nc2, 0.5), nrel=rng.normal(0.0, 0.05, nc2),
              drel=rng.normal(0.0, 0.05, nc2), alpha=np.abs(rng.normal(0.0, 1e-3, nc2)),
              beta=rng.normal(0.0, 1e-4, nc2))
    s3, w0, Iw, Iinv, ja, jb, E, arm_a, arm_b = sphere_problem(gpulib)
    nb3, nc3 = s3["r"].shape[0], ja.shape[0]
    p3 = dict(m=s3["m"], Iw=Iw, Iinv=Iinv, v0=w0, ia=ja.astype(np.float64), ib=jb.astype(np.float64), bases=E,
              arm_a=arm_a, arm_b=arm_b, CoR=np.full(nc3, s3["CoR"]), mu=np.full(nc3, s3["mu"]),
              nrel=rng.normal(0.0, 0.02, nc3), drel=rng.normal(0.0, 0.02, 2 * nc3),
              alpha=np.abs(rng.normal(0.0, 1e-4, nc3)), beta=rng.normal(0.0, 1e-5, 2 * nc3))
    blob = np.concatenate([np.array([nb2, nc2, 500, 1e-9])] + list(p2.values()) +
                          [np.array([nb3, nc3, 300, 1e-10])] + list(p3.values()))
    prob, out = tmp_path / "problem.bin", tmp_path / "out.bin"
    blob.astype("<f8").tofile(prob)
    p = run(host_test, "solve_run", str(prob), str(out), timeout=600)
    assert p.returncode == 0, p.stderr
    got = np.fromfile(out, dtype="<f8")
    o = 0

    def take(n):
        nonlocal o
        o += n
        return got[o - n:o]

    g2 = dict(alpha=take(nc2), beta=take(nc2), v2=take(2 * nb2), f=take(2 * nb2))
    err2, its2 = take(2)
    order2 = take(nc2).astype(np.int32)
    r2 = oracle.sobogus_solve_2d(s2["m"], v0, ia, ib, bases, p2["CoR"], p2["mu"], 1e-9, 500, alpha=p2["alpha"],
                                 beta=p2["beta"], order=order2, nrel_extra=p2["nrel"], drel_extra=p2["drel"])
    for k in g2:
        assert np.array_equal(g2[k], r2[k]), k
    assert err2 == r2["error"] and int(its2) == r2["iterations"]
    g3 = dict(alpha=take(nc3), beta=take(2 * nc3), v2=take(6 * nb3), f=take(6 * nb3))
    err3, its3 = take(2)
    order3 = take(nc3).astype(np.int32)
    assert o == got.shape[0]
    r3 = oracle.sobogus_solve_3d(s3["m"], Iinv, Iw, w0, ja, jb, E, arm_a, arm_b, p3["CoR"], p3["mu"], 1e-10, 300,
                                 alpha=p3["alpha"], beta=p3["beta"], order=order3, nrel_extra=p3["nrel"],
                                 drel_extra=p3["drel"])
    for k in g3:
        assert np.array_equal(g3[k], r3[k]), k
    assert err3 == r3["error"] and int(its3) == r3["iterations"]
