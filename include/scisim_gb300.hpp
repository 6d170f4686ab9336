// scisim_gb300.hpp -- C++ host interface of the GB300 contact-path library, over the C ABI of
// scisim_gpu.h (header only; link with libscisim_gb300.so).
//
// It mirrors SCISim's object model for the contact path with the reference's class names,
// argument meanings and error conventions, so that a driver written against SCISim's
// interfaces reads the same here:
//   unconstrained maps    SymplecticEulerMap, VerletMap (ball2d/SymplecticEulerMap.h, VerletMap.h),
//                         SplitHamMap (rigidbody3d/UnconstrainedMaps/SplitHamMap.h)
//   friction solver       Sobogus, SobogusSolverType (scisim/ConstrainedMaps/Sobogus.h)
//   impact-friction maps  GeometricImpactFrictionMap, SymplecticEulerImpactFrictionMap,
//                         StabilizedImpactFrictionMap (scisim/ConstrainedMaps/), flow() as
//                         ImpactFrictionMap::flow (scisim/ConstrainedMaps/ImpactFrictionMap.h:36)
//   systems               Ball2DState / Ball2DSim (ball2d/), RigidBody3DState / RigidBody3DSim for
//                         spheres (rigidbody3d/), flow() as Ball2DSim::flow (ball2d/Ball2DSim.cpp:305)
// Vectors are std::vector<double> in SCISim's layouts (Ball2D q, v interleaved; RigidBody3D
// q = [x (3n) | R row-major (9n)], v = [v (3n) | omega (3n)]).  Scripting callbacks, periodic
// boundaries and the other systems of SCISim are not part of this path.
//
// Errors: settings the reference rejects by printing and exiting (and invalid inputs) throw
// scisim_gb300::Error carrying the sg_status; a solve that reaches max_iters is not an error, it
// returns its best iterate and reports solve_succeeded = false in the step statistics, as
// GeometricImpactFrictionMap::flow warns and goes on (GeometricImpactFrictionMap.cpp:346-350).
// Every step runs on the GPU; there is no CPU path.
#ifndef SCISIM_GB300_HPP
#define SCISIM_GB300_HPP

#include <atomic>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "scisim_gpu.h"

namespace scisim_gb300 {

inline const char* status_name(int status) {
  switch (status) {
    case SG_OK: return "SG_OK";
    case SG_NOT_CONVERGED: return "SG_NOT_CONVERGED";
    case SG_BAD_INPUT: return "SG_BAD_INPUT";
    case SG_DEVICE_TIMEOUT: return "SG_DEVICE_TIMEOUT";
    case SG_CUDA_ERROR: return "SG_CUDA_ERROR";
    case SG_CAPACITY: return "SG_CAPACITY";
    default: return "unknown status";
  }
}

class Error : public std::runtime_error {
 public:
  Error(int status, const std::string& where)
      : std::runtime_error(where + " returned " + status_name(status) + ": " + sg_last_error_string()),
        m_status(status) {}
  int status() const { return m_status; }

 private:
  int m_status;
};

// Throws for every status but SG_OK and SG_NOT_CONVERGED; returns whether the solve converged.
inline bool check(int status, const char* where) {
  if (status != SG_OK && status != SG_NOT_CONVERGED) throw Error(status, where);
  return status == SG_OK;
}

// scisim/ConstrainedMaps/ImpulsesToCache.h
enum class ImpulsesToCache : int32_t {
  NONE = SG_CACHE_NONE,
  NORMAL = SG_CACHE_NORMAL,
  NORMAL_AND_FRICTION = SG_CACHE_NORMAL_AND_FRICTION
};

// scisim/ConstrainedMaps/Sobogus.h (SobogusSolverType); RigidBody2D is not part of this path.
enum class SobogusSolverType { Balls2D, RigidBodies3D };

// Arithmetic of the Gauss-Seidel sweeps (no counterpart: the reference sweeps in FP64).
enum class Precision : int32_t { FP64 = SG_PRECISION_FP64, FP32_REFINE = SG_PRECISION_FP32_REFINE };

// ---------------------------------------------------------------------------------------------
// Unconstrained maps (scisim/UnconstrainedMaps/UnconstrainedMap.h:13-43).  They select the
// integrator that the library's step kernels run.
class UnconstrainedMap {
 public:
  virtual ~UnconstrainedMap() = default;
  virtual std::string name() const = 0;
  virtual int32_t integrator() const = 0;  // SG_SYMPLECTIC_EULER | SG_VERLET | SG_SPLIT_HAM
};

class SymplecticEulerMap final : public UnconstrainedMap {  // ball2d/SymplecticEulerMap.cpp:21-37
 public:
  std::string name() const override { return "symplectic_euler"; }
  int32_t integrator() const override { return SG_SYMPLECTIC_EULER; }
};

class VerletMap final : public UnconstrainedMap {  // ball2d/VerletMap.cpp:15-46
 public:
  std::string name() const override { return "verlet"; }
  int32_t integrator() const override { return SG_VERLET; }
};

class SplitHamMap final : public UnconstrainedMap {  // rigidbody3d/UnconstrainedMaps/SplitHamMap.cpp:17-187
 public:
  std::string name() const override { return "split_ham"; }
  int32_t integrator() const override { return SG_SPLIT_HAM; }
};

// ---------------------------------------------------------------------------------------------
// Friction solver (scisim/ConstrainedMaps/FrictionSolver.h:16-40).
class FrictionSolver {
 public:
  virtual ~FrictionSolver() = default;
  virtual std::string name() const = 0;
  virtual unsigned numFrictionImpulsesPerNormal(unsigned ambient_space_dimensions) const = 0;
};

// Sobogus (scisim/ConstrainedMaps/Sobogus.cpp:642-645 ctor, :880-1088 solve): the block
// Gauss-Seidel Coulomb solve, evaluating the residual every eval_every sweeps.  precision and
// device have no counterpart.
class Sobogus final : public FrictionSolver {
 public:
  explicit Sobogus(SobogusSolverType solver_type, unsigned eval_every = 1, Precision precision = Precision::FP64,
                   int device = 0)
      : m_type(solver_type), m_eval_every(eval_every), m_precision(precision), m_device(device) {
    if (eval_every == 0) throw Error(SG_BAD_INPUT, "Sobogus: eval_every must be positive");
  }
  ~Sobogus() override {
    if (m_ctx) sg_ctx_destroy(m_ctx);
  }
  Sobogus(const Sobogus&) = delete;
  Sobogus& operator=(const Sobogus&) = delete;

  std::string name() const override { return "sobogus"; }
  unsigned numFrictionImpulsesPerNormal(unsigned ambient_space_dimensions) const override {
    const unsigned dim = m_type == SobogusSolverType::Balls2D ? 2u : 3u;
    if (ambient_space_dimensions != dim) throw Error(SG_BAD_INPUT, "Sobogus: wrong ambient dimension");
    return dim - 1;
  }
  SobogusSolverType solverType() const { return m_type; }
  unsigned evalEvery() const { return m_eval_every; }
  Precision precision() const { return m_precision; }
  int device() const { return m_device; }
  // The context of the last solve (null before the first): sg_last_solve_order reads its order.
  sg_ctx* context() const { return m_ctx; }

  // FrictionSolver::solve for Ball2D contacts on host buffers: masses m (nb), v0 (2nb), contact
  // bodies ia/ib (ib = -1 for a static plane), bases (4 per contact, column-major [n t]),
  // per-contact CoR and mu; the map's extra relative velocities nrel_extra and drel_extra (one
  // each per contact, or empty for zero: Sobogus::solve adds them to the kinematic relative
  // velocities, Sobogus.cpp:892-904); alpha, beta are the warm start and receive the impulses; v2
  // and f (2nb) the post-impact velocity and the generalised friction impulse.  Returns
  // solve_succeeded.
  bool solve(const std::vector<double>& m, const std::vector<double>& v0, const std::vector<int32_t>& ia,
             const std::vector<int32_t>& ib, const std::vector<double>& bases, const std::vector<double>& CoR,
             const std::vector<double>& mu, const std::vector<double>& nrel_extra,
             const std::vector<double>& drel_extra, unsigned max_iters, double tol, std::vector<double>& alpha,
             std::vector<double>& beta, std::vector<double>& v2, std::vector<double>& f, double& error,
             unsigned& iterations) {
    if (m_type != SobogusSolverType::Balls2D) throw Error(SG_BAD_INPUT, "Sobogus::solve takes Balls2D contacts");
    const size_t nb = m.size(), nc = ia.size();
    if (v0.size() != 2 * nb || ib.size() != nc || bases.size() != 4 * nc || CoR.size() != nc || mu.size() != nc ||
        alpha.size() != nc || beta.size() != nc || (!nrel_extra.empty() && nrel_extra.size() != nc) ||
        (!drel_extra.empty() && drel_extra.size() != nc))
      throw Error(SG_BAD_INPUT, "Sobogus::solve: inconsistent sizes");
    ensure_ctx(SG_SYMPLECTIC_EULER, tol, max_iters);
    v2.assign(2 * nb, 0.0);
    f.assign(2 * nb, 0.0);
    uint32_t its = 0;
    const bool ok = check(sg_sobogus_solve_2d_ex(m_ctx, static_cast<int32_t>(nb), m.data(), v0.data(),
                                                 static_cast<int32_t>(nc), ia.data(), ib.data(), bases.data(),
                                                 CoR.data(), mu.data(), nrel_extra.empty() ? nullptr : nrel_extra.data(),
                                                 drel_extra.empty() ? nullptr : drel_extra.data(), max_iters, tol,
                                                 m_eval_every, alpha.data(), beta.data(), v2.data(), f.data(), &error,
                                                 &its),
                          "sg_sobogus_solve_2d_ex");
    iterations = its;
    return ok;
  }

  // The geometric map's call: no extra relative velocities (GeometricImpactFrictionMap.cpp:344).
  bool solve(const std::vector<double>& m, const std::vector<double>& v0, const std::vector<int32_t>& ia,
             const std::vector<int32_t>& ib, const std::vector<double>& bases, const std::vector<double>& CoR,
             const std::vector<double>& mu, unsigned max_iters, double tol, std::vector<double>& alpha,
             std::vector<double>& beta, std::vector<double>& v2, std::vector<double>& f, double& error,
             unsigned& iterations) {
    return solve(m, v0, ia, ib, bases, CoR, mu, {}, {}, max_iters, tol, alpha, beta, v2, f, error, iterations);
  }

  // FrictionSolver::solve for RigidBody3D sphere contacts (SobogusSolverType::RigidBodies3D,
  // Sobogus.cpp:184-251,486-567) on host buffers: masses m (nb), world inertia Iw and its inverse
  // Iinv (9 per body, row-major: the angular blocks of M and Minv), v0 (6nb, [v | omega]);
  // contacts ia/ib, bases (9 per contact, column-major [n s t]), arms arm_a / arm_b (3 per contact:
  // Constraint::getWorldSpaceContactPoint minus the body's centre), CoR, mu, nrel_extra (nc) and
  // drel_extra (2nc) or empty; alpha (nc) and beta (2nc) in = warm start, out = impulses; v2 and f
  // (6nb).  Returns solve_succeeded.
  bool solve3D(const std::vector<double>& m, const std::vector<double>& Iw, const std::vector<double>& Iinv,
               const std::vector<double>& v0, const std::vector<int32_t>& ia, const std::vector<int32_t>& ib,
               const std::vector<double>& bases, const std::vector<double>& arm_a, const std::vector<double>& arm_b,
               const std::vector<double>& CoR, const std::vector<double>& mu, const std::vector<double>& nrel_extra,
               const std::vector<double>& drel_extra, unsigned max_iters, double tol, std::vector<double>& alpha,
               std::vector<double>& beta, std::vector<double>& v2, std::vector<double>& f, double& error,
               unsigned& iterations) {
    if (m_type != SobogusSolverType::RigidBodies3D)
      throw Error(SG_BAD_INPUT, "Sobogus::solve3D takes RigidBodies3D contacts");
    const size_t nb = m.size(), nc = ia.size();
    if (Iw.size() != 9 * nb || Iinv.size() != 9 * nb || v0.size() != 6 * nb || ib.size() != nc ||
        bases.size() != 9 * nc || arm_a.size() != 3 * nc || arm_b.size() != 3 * nc || CoR.size() != nc ||
        mu.size() != nc || alpha.size() != nc || beta.size() != 2 * nc ||
        (!nrel_extra.empty() && nrel_extra.size() != nc) || (!drel_extra.empty() && drel_extra.size() != 2 * nc))
      throw Error(SG_BAD_INPUT, "Sobogus::solve3D: inconsistent sizes");
    ensure_ctx(SG_SPLIT_HAM, tol, max_iters);
    v2.assign(6 * nb, 0.0);
    f.assign(6 * nb, 0.0);
    uint32_t its = 0;
    const bool ok = check(sg_sobogus_solve_3d(m_ctx, static_cast<int32_t>(nb), m.data(), Iw.data(), Iinv.data(),
                                              v0.data(), static_cast<int32_t>(nc), ia.data(), ib.data(),
                                              bases.data(), arm_a.data(), arm_b.data(), CoR.data(), mu.data(),
                                              nrel_extra.empty() ? nullptr : nrel_extra.data(),
                                              drel_extra.empty() ? nullptr : drel_extra.data(), max_iters, tol,
                                              m_eval_every, alpha.data(), beta.data(), v2.data(), f.data(), &error,
                                              &its),
                          "sg_sobogus_solve_3d");
    iterations = its;
    return ok;
  }

 private:
  void ensure_ctx(int32_t integrator, double tol, unsigned max_iters) {
    if (m_ctx) return;
    sg_config c{};
    c.integrator = integrator;
    c.precision = static_cast<int32_t>(m_precision);
    c.device = m_device;
    c.dt = 1.0;
    c.tol = tol;
    c.max_iters = max_iters;
    c.eval_every = m_eval_every;
    check(sg_ctx_create(&c, &m_ctx), "sg_ctx_create");
  }

 private:
  SobogusSolverType m_type;
  unsigned m_eval_every;
  Precision m_precision;
  int m_device;
  sg_ctx* m_ctx = nullptr;
};

// ---------------------------------------------------------------------------------------------
// Systems.  A system uploads its scene into a context; the impact-friction map owns the context.
// Each system has an identity of its own, renewed when it is copied or assigned, by which a map
// knows whether its context still holds this system's scene.  A map keeps the radii, masses,
// inertia and planes of the system from its first flow; after changing those in place, call the
// map's resetCachedData() (positions and velocities are passed to every flow).
class ContactSystem {
 public:
  ContactSystem() : m_uid(next_uid()) {}
  ContactSystem(const ContactSystem&) : m_uid(next_uid()) {}
  ContactSystem& operator=(const ContactSystem&) {
    m_uid = next_uid();
    return *this;
  }
  virtual ~ContactSystem() = default;
  uint64_t uid() const { return m_uid; }
  virtual unsigned nbodies() const = 0;
  virtual unsigned ambientDimension() const = 0;  // 2 (Ball2D) or 3 (spheres)
  virtual std::vector<double> gravity() const = 0;
  virtual void upload(sg_ctx* ctx) const = 0;

 private:
  static uint64_t next_uid() {
    static std::atomic<uint64_t> counter{0};
    return ++counter;
  }
  uint64_t m_uid;
};

struct StaticPlane2D {  // ball2d/StaticGeometry/StaticPlane.cpp:10-19 (x, n; n normalised)
  double x[2];
  double n[2];
};

struct StaticPlane3D {  // rigidbody3d/StaticGeometry/StaticPlane.cpp:10-15
  double x[3];
  double n[3];
};

// ball2d/Ball2DState.h: q, v interleaved (2 per ball), radii, masses, static planes.
struct Ball2DState {
  std::vector<double> q, v, r, m;
  std::vector<StaticPlane2D> planes;
  unsigned nballs() const { return static_cast<unsigned>(r.size()); }
};

// RigidBody3DState of spheres: q = [x | R row-major], v = [v | omega], radii, masses, principal
// moments I0 (3 per body; RigidBodySphere::computeMassAndInertia,
// rigidbody3d/Geometry/RigidBodySphere.cpp:10-18), static planes.
struct RigidBody3DState {
  std::vector<double> q, v, r, m, I0;
  std::vector<StaticPlane3D> planes;
  unsigned nbodies() const { return static_cast<unsigned>(r.size()); }
};

class ImpactFrictionMap;

// ball2d/Ball2DSim.h: owns the state; flow() advances one step (Ball2DSim.cpp:305-326).
class Ball2DSim final : public ContactSystem {
 public:
  explicit Ball2DSim(Ball2DState state, double gx = 0.0, double gy = -9.81)
      : m_state(std::move(state)), m_g{gx, gy} {
    const size_t n = m_state.r.size();
    if (m_state.q.size() != 2 * n || m_state.v.size() != 2 * n || m_state.m.size() != n)
      throw Error(SG_BAD_INPUT, "Ball2DSim: inconsistent state sizes");
  }
  unsigned nbodies() const override { return m_state.nballs(); }
  unsigned ambientDimension() const override { return 2; }
  std::vector<double> gravity() const override { return {m_g[0], m_g[1], 0.0}; }
  const Ball2DState& state() const { return m_state; }
  Ball2DState& state() { return m_state; }
  void upload(sg_ctx* ctx) const override {
    std::vector<double> px, pn;
    for (const StaticPlane2D& p : m_state.planes) {
      px.insert(px.end(), {p.x[0], p.x[1]});
      pn.insert(pn.end(), {p.n[0], p.n[1]});
    }
    check(sg_ball2d_upload(ctx, static_cast<int32_t>(nbodies()), m_state.q.data(), m_state.v.data(),
                           m_state.r.data(), m_state.m.data(), static_cast<int32_t>(m_state.planes.size()),
                           px.data(), pn.data()),
          "sg_ball2d_upload");
  }
  // Ball2DSim::flow(iteration, dt, umap, CoR, mu, solver, ifmap), without the scripting callback.
  inline sg_step_stats flow(unsigned iteration, double dt, UnconstrainedMap& umap, double CoR, double mu,
                            FrictionSolver& solver, ImpactFrictionMap& ifmap);

 private:
  Ball2DState m_state;
  double m_g[2];
};

// rigidbody3d/RigidBody3DSim.h for spheres: flow() as RigidBody3DSim::flow
// (rigidbody3d/RigidBody3DSim.cpp:557-630); the world inertia of the new orientations is the
// library's (sg_sphere3d_world_inertia).
class RigidBody3DSim final : public ContactSystem {
 public:
  explicit RigidBody3DSim(RigidBody3DState state, double gx = 0.0, double gy = -9.81, double gz = 0.0)
      : m_state(std::move(state)), m_g{gx, gy, gz} {
    const size_t n = m_state.r.size();
    if (m_state.q.size() != 12 * n || m_state.v.size() != 6 * n || m_state.m.size() != n || m_state.I0.size() != 3 * n)
      throw Error(SG_BAD_INPUT, "RigidBody3DSim: inconsistent state sizes");
  }
  unsigned nbodies() const override { return m_state.nbodies(); }
  unsigned ambientDimension() const override { return 3; }
  std::vector<double> gravity() const override { return {m_g[0], m_g[1], m_g[2]}; }
  const RigidBody3DState& state() const { return m_state; }
  RigidBody3DState& state() { return m_state; }
  void upload(sg_ctx* ctx) const override {
    std::vector<double> px, pn;
    for (const StaticPlane3D& p : m_state.planes) {
      px.insert(px.end(), {p.x[0], p.x[1], p.x[2]});
      pn.insert(pn.end(), {p.n[0], p.n[1], p.n[2]});
    }
    check(sg_sphere3d_upload(ctx, static_cast<int32_t>(nbodies()), m_state.q.data(), m_state.v.data(),
                             m_state.r.data(), m_state.m.data(), m_state.I0.data(),
                             static_cast<int32_t>(m_state.planes.size()), px.data(), pn.data()),
          "sg_sphere3d_upload");
  }
  inline sg_step_stats flow(unsigned iteration, double dt, UnconstrainedMap& umap, double CoR, double mu,
                            FrictionSolver& solver, ImpactFrictionMap& ifmap);

 private:
  RigidBody3DState m_state;
  double m_g[3];
};

// ---------------------------------------------------------------------------------------------
// Impact-friction maps (scisim/ConstrainedMaps/ImpactFrictionMap.h:24-63).  flow() takes the host
// state (q0, v0) and writes (q1, v1); the impulse cache lives in the map's context on the GPU, as
// SCISim's ConstraintCache lives beside the simulation.  The context is built on the first flow
// and rebuilt (with the scene uploaded afresh) when the system or a setting changes.
class ImpactFrictionMap {
 public:
  virtual ~ImpactFrictionMap() {
    if (m_ctx) sg_ctx_destroy(m_ctx);
  }
  ImpactFrictionMap(const ImpactFrictionMap&) = delete;
  ImpactFrictionMap& operator=(const ImpactFrictionMap&) = delete;

  virtual std::string name() const = 0;

  // ImpactFrictionMap::flow(fsys, csys, umap, friction_solver, iteration, dt, CoR, mu_default,
  // q0, v0, q1, v1) (ImpactFrictionMap.h:36), the system in the roles of fsys and csys.
  sg_step_stats flow(const ContactSystem& sys, UnconstrainedMap& umap, FrictionSolver& friction_solver,
                     unsigned iteration, double dt, double CoR, double mu_default, const std::vector<double>& q0,
                     const std::vector<double>& v0, std::vector<double>& q1, std::vector<double>& v1) {
    sg_ctx* ctx = context(sys, umap, friction_solver, dt, CoR, mu_default);
    const size_t nq = sys.ambientDimension() == 2 ? 2 * sys.nbodies() : 12 * sys.nbodies();
    const size_t nv = sys.ambientDimension() == 2 ? 2 * sys.nbodies() : 6 * sys.nbodies();
    if (q0.size() != nq || v0.size() != nv) throw Error(SG_BAD_INPUT, name() + "::flow: state sizes");
    q1.resize(nq);
    v1.resize(nv);
    sg_step_stats st{};
    check(sg_flow(ctx, iteration, q0.data(), v0.data(), q1.data(), v1.data(), &st), "sg_flow");
    return st;
  }

  // ImpactFrictionMap::resetCachedData: drops the impulse cache (and the context holding it).
  virtual void resetCachedData() {
    if (m_ctx) sg_ctx_destroy(m_ctx);
    m_ctx = nullptr;
    m_sys = 0;
  }

  // The context of the last flow (nullptr before the first): for sg_last_contacts and the like.
  sg_ctx* context() const { return m_ctx; }

 protected:
  ImpactFrictionMap(double abs_tol, unsigned max_iters, ImpulsesToCache cache)
      : m_abs_tol(abs_tol), m_max_iters(max_iters), m_cache(cache) {
    if (!(abs_tol >= 0.0)) throw Error(SG_BAD_INPUT, "ImpactFrictionMap: abs_tol must be non-negative");
  }
  // Called once on every new context, after the scene is uploaded.
  virtual void configure(sg_ctx*, double /*CoR*/) {}

 private:
  sg_ctx* context(const ContactSystem& sys, const UnconstrainedMap& umap, const FrictionSolver& solver, double dt,
                  double CoR, double mu) {
    const Sobogus* sob = dynamic_cast<const Sobogus*>(&solver);
    if (sob == nullptr) throw Error(SG_BAD_INPUT, "only the Sobogus friction solver is available");
    const std::vector<double> g = sys.gravity();
    const bool same = m_ctx && m_sys == sys.uid() && m_nb == sys.nbodies() && m_integrator == umap.integrator() &&
                      m_eval_every == sob->evalEvery() && m_precision == sob->precision() &&
                      m_device == sob->device() && m_dt == dt && m_CoR == CoR && m_mu == mu && m_g == g;
    if (same) return m_ctx;
    resetCachedData();
    sg_config c{};
    c.integrator = umap.integrator();
    c.cache_mode = static_cast<int32_t>(m_cache);
    c.precision = static_cast<int32_t>(sob->precision());
    c.device = sob->device();
    c.dt = dt;
    for (int k = 0; k < 3; ++k) c.gravity[k] = g[k];
    c.mu = mu;
    c.CoR = CoR;
    c.tol = m_abs_tol;
    c.max_iters = m_max_iters;
    c.eval_every = sob->evalEvery();
    check(sg_ctx_create(&c, &m_ctx), "sg_ctx_create");
    try {
      sys.upload(m_ctx);
      configure(m_ctx, CoR);
    } catch (...) {
      resetCachedData();
      throw;
    }
    m_sys = sys.uid();
    m_nb = sys.nbodies();
    m_integrator = umap.integrator();
    m_eval_every = sob->evalEvery();
    m_precision = sob->precision();
    m_device = sob->device();
    m_dt = dt;
    m_CoR = CoR;
    m_mu = mu;
    m_g = g;
    return m_ctx;
  }

  double m_abs_tol;
  unsigned m_max_iters;
  ImpulsesToCache m_cache;
  sg_ctx* m_ctx = nullptr;
  uint64_t m_sys = 0;  // uid of the system whose scene the context holds
  unsigned m_nb = 0;
  int32_t m_integrator = -1;
  unsigned m_eval_every = 0;
  Precision m_precision = Precision::FP64;
  int m_device = 0;
  double m_dt = 0.0, m_CoR = 0.0, m_mu = 0.0;
  std::vector<double> m_g;
};

// GeometricImpactFrictionMap (scisim/ConstrainedMaps/GeometricImpactFrictionMap.cpp:20-31 ctor,
// :267-442 flow).
class GeometricImpactFrictionMap : public ImpactFrictionMap {
 public:
  GeometricImpactFrictionMap(double abs_tol, unsigned max_iters, ImpulsesToCache impulses_to_cache)
      : ImpactFrictionMap(abs_tol, max_iters, impulses_to_cache) {}
  std::string name() const override { return "geometric_impact_friction_map"; }
};

// SymplecticEulerImpactFrictionMap (scisim/ConstrainedMaps/SymplecticEulerImpactFrictionMap.cpp:201-407)
// for Ball2D: the force first, the solve with N^T vdelta and D^T vdelta (and the pose
// stabilisation beyond penetration_threshold when stabilize is set), then a linear update; the
// unconstrained map passed to flow() is not used.  CoR must be 0, as the reference requires.
class SymplecticEulerImpactFrictionMap final : public ImpactFrictionMap {
 public:
  SymplecticEulerImpactFrictionMap(double abs_tol, unsigned max_iters, ImpulsesToCache impulses_to_cache,
                                   bool stabilize = false, double penetration_threshold = 0.0)
      : ImpactFrictionMap(abs_tol, max_iters, impulses_to_cache), m_stabilize(stabilize),
        m_threshold(penetration_threshold) {
    if (!(penetration_threshold >= 0.0))
      throw Error(SG_BAD_INPUT, "SymplecticEulerImpactFrictionMap: penetration_threshold must be non-negative");
  }
  std::string name() const override { return "symplectic_euler_impact_friction_map"; }

 protected:
  void configure(sg_ctx* ctx, double CoR) override {
    if (CoR != 0.0) throw Error(SG_BAD_INPUT, "SymplecticEulerImpactFrictionMap: CoR must be 0");
    check(sg_set_staggering(ctx, SG_STAGGER_SYMPLECTIC_EULER, m_stabilize ? 1 : 0, m_threshold), "sg_set_staggering");
  }

 private:
  bool m_stabilize;
  double m_threshold;
};

// StabilizedImpactFrictionMap (scisim/ConstrainedMaps/StabilizedImpactFrictionMap.cpp:48-167) for
// Ball2D: the unconstrained step, a cold solve from its velocity (no impulse cache), then
// q1 = q0 + dt v1.
class StabilizedImpactFrictionMap final : public ImpactFrictionMap {
 public:
  StabilizedImpactFrictionMap(double abs_tol, unsigned max_iters)
      : ImpactFrictionMap(abs_tol, max_iters, ImpulsesToCache::NONE) {}
  std::string name() const override { return "stabilized_impact_friction_map"; }

 protected:
  void configure(sg_ctx* ctx, double) override {
    check(sg_set_staggering(ctx, SG_STAGGER_STABILIZED, 0, 0.0), "sg_set_staggering");
  }
};

inline sg_step_stats Ball2DSim::flow(unsigned iteration, double dt, UnconstrainedMap& umap, double CoR, double mu,
                                     FrictionSolver& solver, ImpactFrictionMap& ifmap) {
  std::vector<double> q1, v1;
  const sg_step_stats st = ifmap.flow(*this, umap, solver, iteration, dt, CoR, mu, m_state.q, m_state.v, q1, v1);
  m_state.q.swap(q1);
  m_state.v.swap(v1);
  return st;
}

inline sg_step_stats RigidBody3DSim::flow(unsigned iteration, double dt, UnconstrainedMap& umap, double CoR,
                                          double mu, FrictionSolver& solver, ImpactFrictionMap& ifmap) {
  std::vector<double> q1, v1;
  const sg_step_stats st = ifmap.flow(*this, umap, solver, iteration, dt, CoR, mu, m_state.q, m_state.v, q1, v1);
  m_state.q.swap(q1);
  m_state.v.swap(v1);
  return st;
}

}  // namespace scisim_gb300

#endif  // SCISIM_GB300_HPP
