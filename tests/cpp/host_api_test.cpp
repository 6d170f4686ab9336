// Tests of the C++ host interface (include/scisim_gb300.hpp), written the way the reference writes
// its test programs: one executable, the test name as the first argument, the exit status as the
// result (scisimtests/rational_number_tests.cpp).
//
//   names       the mirrored classes report the reference's names (e.g. ball2d/VerletMap.cpp:43-46)
//   validation  invalid settings and state sizes throw Error(SG_BAD_INPUT) before any GPU work
//   identity    a copied or assigned system gets an identity of its own (a map's context follows it)
//   no_device   where no GPU can be used, a flow throws Error(SG_CUDA_ERROR) and nothing else
//               (exits 0 at once where a context can be created)
//   ball2d_run  <scene file> <out file>: steps the scene through Ball2DSim::flow with the
//               geometric, symplectic-Euler and stabilized impact-friction maps and writes each
//               final (q, v); the test compares them with the same steps through the C ABI.
//   solve_run   <problem file> <out file>: Sobogus::solve on a Ball2D problem with the map's extra
//               relative velocities and Sobogus::solve3D on a sphere problem with extras; writes the
//               impulses, v2, f, residual, sweeps and the solve order of each, which the test
//               replays on the oracle.
//
// Scene file: little-endian doubles n, np, dt, gx, gy, mu, tol, max_iters, steps, then q (2n),
// v (2n), r (n), m (n), plane x (2np), plane n (2np).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "scisim_gb300.hpp"

using namespace scisim_gb300;

namespace {

int fail(const std::string& what) {
  std::cerr << "FAILED: " << what << std::endl;
  return EXIT_FAILURE;
}

Ball2DState two_balls() {
  Ball2DState s;
  s.q = {0.0, 0.5, 0.0, 1.6};
  s.v = {0.0, 0.0, 0.0, 0.0};
  s.r = {0.5, 0.5};
  s.m = {1.0, 1.0};
  s.planes.push_back(StaticPlane2D{{0.0, 0.0}, {0.0, 1.0}});
  return s;
}

template <class F>
bool throws_status(F&& f, int status) {
  try {
    f();
  } catch (const Error& e) {
    return e.status() == status;
  } catch (...) {
    return false;
  }
  return false;
}

int test_names() {
  if (SymplecticEulerMap().name() != "symplectic_euler") return fail("SymplecticEulerMap::name");
  if (VerletMap().name() != "verlet") return fail("VerletMap::name");
  if (SplitHamMap().name() != "split_ham") return fail("SplitHamMap::name");
  Sobogus sob(SobogusSolverType::Balls2D, 1);
  if (sob.name() != "sobogus" || sob.numFrictionImpulsesPerNormal(2) != 1) return fail("Sobogus");
  if (Sobogus(SobogusSolverType::RigidBodies3D).numFrictionImpulsesPerNormal(3) != 2) return fail("Sobogus 3D");
  if (GeometricImpactFrictionMap(1e-6, 100, ImpulsesToCache::NONE).name() != "geometric_impact_friction_map")
    return fail("GeometricImpactFrictionMap::name");
  if (SymplecticEulerImpactFrictionMap(1e-6, 100, ImpulsesToCache::NONE).name() !=
      "symplectic_euler_impact_friction_map")
    return fail("SymplecticEulerImpactFrictionMap::name");
  if (StabilizedImpactFrictionMap(1e-6, 100).name() != "stabilized_impact_friction_map")
    return fail("StabilizedImpactFrictionMap::name");
  if (std::string(status_name(SG_NOT_CONVERGED)) != "SG_NOT_CONVERGED") return fail("status_name");
  return EXIT_SUCCESS;
}

int test_validation() {
  if (!throws_status([] { Sobogus(SobogusSolverType::Balls2D, 0); }, SG_BAD_INPUT)) return fail("eval_every 0");
  if (!throws_status([] { Sobogus(SobogusSolverType::Balls2D).numFrictionImpulsesPerNormal(3); }, SG_BAD_INPUT))
    return fail("ambient dimension");
  if (!throws_status([] { GeometricImpactFrictionMap(-1.0, 10, ImpulsesToCache::NONE); }, SG_BAD_INPUT))
    return fail("negative tolerance");
  if (!throws_status([] { SymplecticEulerImpactFrictionMap(1e-6, 10, ImpulsesToCache::NONE, true, -1.0); },
                     SG_BAD_INPUT))
    return fail("negative penetration threshold");
  if (!throws_status(
          [] {
            Ball2DState s = two_balls();
            s.v.pop_back();
            Ball2DSim sim(s);
          },
          SG_BAD_INPUT))
    return fail("Ball2D state sizes");
  if (!throws_status(
          [] {
            RigidBody3DState s;
            s.r = {0.5};
            s.m = {1.0};
            s.I0 = {0.1, 0.1, 0.1};
            s.q.assign(11, 0.0);
            s.v.assign(6, 0.0);
            RigidBody3DSim sim(s);
          },
          SG_BAD_INPUT))
    return fail("RigidBody3D state sizes");
  if (!throws_status(
          [] {
            Sobogus sob(SobogusSolverType::Balls2D);
            std::vector<double> m{1.0}, v0{0.0}, bases, CoR, mu, alpha, beta, v2, f;
            std::vector<int32_t> ia, ib;
            double err = 0.0;
            unsigned its = 0;
            sob.solve(m, v0, ia, ib, bases, CoR, mu, 10, 1e-6, alpha, beta, v2, f, err, its);
          },
          SG_BAD_INPUT))
    return fail("Sobogus::solve sizes");
  return EXIT_SUCCESS;
}

int test_identity() {
  Ball2DSim a(two_balls());
  Ball2DSim b(a);
  if (a.uid() == b.uid() || a.uid() == 0) return fail("a copy has its own identity");
  const uint64_t before = b.uid();
  b = a;
  if (b.uid() == before || b.uid() == a.uid()) return fail("assignment renews the identity");
  return EXIT_SUCCESS;
}

int test_no_device() {
  sg_config c{};
  c.integrator = SG_SYMPLECTIC_EULER;
  c.dt = 0.01;
  c.tol = 1e-6;
  c.max_iters = 10;
  c.eval_every = 1;
  sg_ctx* ctx = nullptr;
  if (sg_ctx_create(&c, &ctx) == SG_OK) {  // a usable GPU: nothing to check here
    sg_ctx_destroy(ctx);
    return EXIT_SUCCESS;
  }
  Ball2DSim sim(two_balls());
  SymplecticEulerMap umap;
  Sobogus sob(SobogusSolverType::Balls2D);
  GeometricImpactFrictionMap ifmap(1e-6, 10, ImpulsesToCache::NONE);
  if (!throws_status([&] { sim.flow(1, 0.01, umap, 0.0, 0.5, sob, ifmap); }, SG_CUDA_ERROR))
    return fail("flow without a device");
  if (ifmap.context() != nullptr) return fail("no context is kept after a failed creation");
  return EXIT_SUCCESS;
}

constexpr int kMaxSolveColors = 64;  // colour limit of the solver (SG_CAPACITY beyond it)

int test_ball2d_run(const char* scene_path, const char* out_path) {
  std::ifstream in(scene_path, std::ios::binary);
  if (!in) return fail("cannot open the scene file");
  auto rd = [&in](size_t n) {
    std::vector<double> x(n);
    in.read(reinterpret_cast<char*>(x.data()), static_cast<std::streamsize>(sizeof(double) * n));
    return x;
  };
  const std::vector<double> h = rd(9);
  const size_t n = static_cast<size_t>(h[0]), np = static_cast<size_t>(h[1]);
  const double dt = h[2], gx = h[3], gy = h[4], mu = h[5], tol = h[6];
  const unsigned max_iters = static_cast<unsigned>(h[7]), steps = static_cast<unsigned>(h[8]);
  Ball2DState s;
  s.q = rd(2 * n);
  s.v = rd(2 * n);
  s.r = rd(n);
  s.m = rd(n);
  const std::vector<double> px = rd(2 * np), pn = rd(2 * np);
  if (!in) return fail("short scene file");
  for (size_t p = 0; p < np; ++p) s.planes.push_back(StaticPlane2D{{px[2 * p], px[2 * p + 1]}, {pn[2 * p], pn[2 * p + 1]}});

  std::ofstream out(out_path, std::ios::binary);
  auto wr = [&out](const std::vector<double>& x) {
    out.write(reinterpret_cast<const char*>(x.data()), static_cast<std::streamsize>(sizeof(double) * x.size()));
  };
  VerletMap verlet;
  SymplecticEulerMap symplectic_euler;
  Sobogus sob(SobogusSolverType::Balls2D, 1);
  {  // geometric map, Verlet, warm start from normal and friction impulses, CoR 0.3
    Ball2DSim sim(s, gx, gy);
    GeometricImpactFrictionMap ifmap(tol, max_iters, ImpulsesToCache::NORMAL_AND_FRICTION);
    for (unsigned it = 1; it <= steps; ++it) sim.flow(it, dt, verlet, 0.3, mu, sob, ifmap);
    wr(sim.state().q);
    wr(sim.state().v);
  }
  {  // symplectic-Euler map with stabilisation, CoR 0
    Ball2DSim sim(s, gx, gy);
    SymplecticEulerImpactFrictionMap ifmap(tol, max_iters, ImpulsesToCache::NORMAL_AND_FRICTION, true, 1e-4);
    for (unsigned it = 1; it <= steps; ++it) sim.flow(it, dt, symplectic_euler, 0.0, mu, sob, ifmap);
    wr(sim.state().q);
    wr(sim.state().v);
  }
  {  // stabilized map, CoR 0.3
    Ball2DSim sim(s, gx, gy);
    StabilizedImpactFrictionMap ifmap(tol, max_iters);
    for (unsigned it = 1; it <= steps; ++it) sim.flow(it, dt, symplectic_euler, 0.3, mu, sob, ifmap);
    wr(sim.state().q);
    wr(sim.state().v);
  }
  if (!out) return fail("cannot write the output file");
  return EXIT_SUCCESS;
}

// Problem file (little-endian doubles): 2D block nb, nc, max_iters, tol, m, v0, ia, ib, bases, CoR,
// mu, nrel, drel, alpha, beta; then the 3D block nb, nc, max_iters, tol, m, Iw, Iinv, v0, ia, ib,
// bases, arm_a, arm_b, CoR, mu, nrel, drel, alpha, beta (sizes as the solve calls take them).
int test_solve_run(const char* problem_path, const char* out_path) {
  std::ifstream in(problem_path, std::ios::binary);
  if (!in) return fail("cannot open the problem file");
  auto rd = [&in](size_t n) {
    std::vector<double> x(n);
    in.read(reinterpret_cast<char*>(x.data()), static_cast<std::streamsize>(sizeof(double) * n));
    return x;
  };
  auto rdi = [&rd](size_t n) {
    const std::vector<double> x = rd(n);
    return std::vector<int32_t>(x.begin(), x.end());
  };
  std::ofstream out(out_path, std::ios::binary);
  auto wr = [&out](const std::vector<double>& x) {
    out.write(reinterpret_cast<const char*>(x.data()), static_cast<std::streamsize>(sizeof(double) * x.size()));
  };
  auto order_of = [](sg_ctx* ctx, size_t nc) {
    std::vector<int32_t> order(nc), off(kMaxSolveColors + 1);
    int32_t ncol = 0;
    if (sg_last_solve_order(ctx, static_cast<int64_t>(nc), order.data(), off.data(), &ncol) !=
        static_cast<int64_t>(nc))
      throw Error(SG_BAD_INPUT, "sg_last_solve_order");
    return std::vector<double>(order.begin(), order.end());
  };
  {  // Ball2D with nrel_extra, drel_extra
    const std::vector<double> h = rd(4);
    const size_t nb = static_cast<size_t>(h[0]), nc = static_cast<size_t>(h[1]);
    const std::vector<double> m = rd(nb), v0 = rd(2 * nb);
    const std::vector<int32_t> ia = rdi(nc), ib = rdi(nc);
    const std::vector<double> bases = rd(4 * nc), CoR = rd(nc), mu = rd(nc), nrel = rd(nc), drel = rd(nc);
    std::vector<double> alpha = rd(nc), beta = rd(nc), v2, f;
    if (!in) return fail("short 2D problem");
    Sobogus sob(SobogusSolverType::Balls2D, 1);
    double err = 0.0;
    unsigned its = 0;
    sob.solve(m, v0, ia, ib, bases, CoR, mu, nrel, drel, static_cast<unsigned>(h[2]), h[3], alpha, beta, v2, f, err,
              its);
    wr(alpha);
    wr(beta);
    wr(v2);
    wr(f);
    wr({err, static_cast<double>(its)});
    wr(order_of(sob.context(), nc));
  }
  {  // spheres with nrel_extra, drel_extra
    const std::vector<double> h = rd(4);
    const size_t nb = static_cast<size_t>(h[0]), nc = static_cast<size_t>(h[1]);
    const std::vector<double> m = rd(nb), Iw = rd(9 * nb), Iinv = rd(9 * nb), v0 = rd(6 * nb);
    const std::vector<int32_t> ia = rdi(nc), ib = rdi(nc);
    const std::vector<double> bases = rd(9 * nc), arm_a = rd(3 * nc), arm_b = rd(3 * nc), CoR = rd(nc), mu = rd(nc);
    const std::vector<double> nrel = rd(nc), drel = rd(2 * nc);
    std::vector<double> alpha = rd(nc), beta = rd(2 * nc), v2, f;
    if (!in) return fail("short 3D problem");
    Sobogus sob(SobogusSolverType::RigidBodies3D, 1);
    double err = 0.0;
    unsigned its = 0;
    sob.solve3D(m, Iw, Iinv, v0, ia, ib, bases, arm_a, arm_b, CoR, mu, nrel, drel, static_cast<unsigned>(h[2]),
                h[3], alpha, beta, v2, f, err, its);
    wr(alpha);
    wr(beta);
    wr(v2);
    wr(f);
    wr({err, static_cast<double>(its)});
    wr(order_of(sob.context(), nc));
  }
  if (!out) return fail("cannot write the output file");
  return EXIT_SUCCESS;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    std::cerr << "Usage: " << argv[0] << " test_name [args]" << std::endl;
    return EXIT_FAILURE;
  }
  const std::string test(argv[1]);
  try {
    if (test == "names") return test_names();
    if (test == "validation") return test_validation();
    if (test == "identity") return test_identity();
    if (test == "no_device") return test_no_device();
    if (test == "ball2d_run" && argc == 4) return test_ball2d_run(argv[2], argv[3]);
    if (test == "solve_run" && argc == 4) return test_solve_run(argv[2], argv[3]);
  } catch (const std::exception& e) {
    return fail(std::string("unexpected exception: ") + e.what());
  }
  std::cerr << "Unknown test " << test << std::endl;
  return EXIT_FAILURE;
}
