// oracle.h -- CPU oracle for the SCISim per-step contact path.
//
// TEST INFRASTRUCTURE ONLY.  This is a plain C++ restatement of the reference
// algorithm (breannansmith/scisim) that the tests compare the GPU library with,
// and the timed CPU baseline.  Product code never links, imports or
// executes anything under oracle/; only tests/, __graft_entry__.smoke() and the
// cpu_baseline / reference legs of bench.py do.
//
// Build: g++ -O2 -std=c++17 -ffp-contract=off -fopenmp (see oracle/Makefile).
// FP contraction is off so every FP64 operation rounds the way the reference's
// ISO C++ build does (CMakeLists.txt:250 disables GNU extensions).
//
// Parity status: the SCISim side (integrators, broad phase, CCD, constraints,
// forcing terms, staggering, warm-start cache) follows the reference file:line
// cited at each function and is pinned by the reference's own known-answer
// tests (AABB fixtures, CCD cases, analytic slope scenes).  The Gauss-Seidel
// solver, the local Coulomb solver and the residual live in the un-vendored
// So-bogus library; they are restated from the published method (Daviet,
// Bertails-Descoubes & Boissieux 2011) and are "parity unpinned" at the level of
// individual iterates and residual scale.
#ifndef SCISIM_ORACLE_H
#define SCISIM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

// ---------------------------------------------------------------- broad phase
// aabb: n boxes as [minx, miny, maxx, maxy].  Writes pairs (i<j) in the
// lexicographic order of std::set<std::pair<unsigned,unsigned>>.
// Returns the number of pairs, or -1 if cap is too small (count still written to *total).
int64_t or_grid_overlaps_2d(int n, const double* aabb, int64_t cap, int32_t* pairs, int64_t* total);
int64_t or_allpairs_overlaps_2d(int n, const double* aabb, int64_t cap, int32_t* pairs, int64_t* total);
// 3D boxes as [minx, miny, minz, maxx, maxy, maxz].
int64_t or_grid_overlaps_3d(int n, const double* aabb, int64_t cap, int32_t* pairs, int64_t* total);
int64_t or_allpairs_overlaps_3d(int n, const double* aabb, int64_t cap, int32_t* pairs, int64_t* total);

// ---------------------------------------------------------------- narrow phase
void or_ccd_coeffs_2d(const double* q0a, const double* q1a, double ra, const double* q0b,
                      const double* q1b, double rb, double* c3);
int or_ccd_happens(const double* c3, double* t_out);

// ---------------------------------------------------------------- friction solve
// Per-contact Fischer-Burmeister Coulomb error of (r, u) in local coordinates.
double or_fb_error(int dim, const double* r, const double* u, double mu);
// Local Coulomb solve: u = W r + b, W symmetric (2D: w00 w01 w11; 3D: w00 w01 w02 w11 w12 w22).
void or_local_solve(int dim, const double* W, const double* b, double mu, double* r);

typedef struct {
  double tol;
  uint32_t max_iters;
  uint32_t eval_every;
  const int32_t* order;   // optional sweep order (permutation of contacts) or NULL for 0..nc-1
} or_gs_params;

typedef struct {
  double error;
  uint32_t iterations;
  int32_t succeeded;
} or_gs_result;

// Ball2D FrictionSolver::solve restatement (Sobogus::solve with Balls2D).
// m: per-body mass; v0: 2nb; contacts: ia[nc] (>=0), ib[nc] (>=0 or -1 static);
// bases: 4 per contact, column-major [n t]; CoR, mu per contact.
// alpha/beta: in = warm start, out = solution.  v2, f: 2nb outputs.
void or_sobogus_solve_2d(int nb, const double* m, const double* v0, int nc, const int32_t* ia,
                         const int32_t* ib, const double* bases, const double* CoR, const double* mu,
                         const or_gs_params* p, double* alpha, double* beta, double* v2, double* f,
                         or_gs_result* res);

// As or_sobogus_solve_2d with the map's extra relative velocities per contact (nrel, drel; the
// geometric map's are zero).
void or_sobogus_solve_2d_ex(int nb, const double* m, const double* v0, int nc, const int32_t* ia,
                            const int32_t* ib, const double* bases, const double* CoR, const double* mu,
                            const double* nrel, const double* drel, const or_gs_params* p, double* alpha,
                            double* beta, double* v2, double* f, or_gs_result* res);

// Coulomb residual (the solver's error function) of given impulses (alpha, beta).
double or_residual_2d(int nb, const double* m, const double* v0, int nc, const int32_t* ia, const int32_t* ib,
                      const double* bases, const double* CoR, const double* mu, const double* alpha,
                      const double* beta);

// The same with the map's extra relative velocities (nrel, drel per contact; null = zero).
double or_residual_2d_ex(int nb, const double* m, const double* v0, int nc, const int32_t* ia, const int32_t* ib,
                         const double* bases, const double* CoR, const double* mu, const double* nrel,
                         const double* drel, const double* alpha, const double* beta);

// ---------------------------------------------------------------- Ball2D scene
typedef struct or_ball2d or_ball2d;

enum { OR_SYMPLECTIC_EULER = 0, OR_VERLET = 1 };
enum { OR_CACHE_NONE = 0, OR_CACHE_NORMAL = 1, OR_CACHE_NORMAL_AND_FRICTION = 2 };
enum { OR_STAGGER_GEOMETRIC = 0, OR_STAGGER_SYMPLECTIC_EULER = 1, OR_STAGGER_STABILIZED = 2 };

typedef struct {
  int32_t integrator;     // OR_SYMPLECTIC_EULER / OR_VERLET
  int32_t cache_mode;     // OR_CACHE_*
  double dt;
  double gravity[2];
  double mu;
  double CoR;
  double tol;
  uint32_t max_iters;
  uint32_t eval_every;
  int32_t staggering;             // OR_STAGGER_* (Geometric / SymplecticEuler / Stabilized ImpactFrictionMap)
  int32_t stabilize;              // symplectic Euler: pose stabilisation g0 / dt
  double penetration_threshold;   // symplectic Euler: gaps smaller in magnitude are ignored
} or_ball2d_params;

typedef struct {
  int64_t n_contacts;
  int64_t n_ball_ball;
  int64_t n_ball_plane;
  uint32_t iterations;
  int32_t succeeded;
  double error;
} or_step_stats;

or_ball2d* or_ball2d_create(int nb, const double* q, const double* v, const double* r, const double* m,
                            int np, const double* plane_x, const double* plane_n, const or_ball2d_params* p);
void or_ball2d_destroy(or_ball2d* s);
// One GeometricImpactFrictionMap::flow step.  order_cb: optional sweep order
// supplier (NULL = sequential order, as the reference's uncoloured GS).
int or_ball2d_step(or_ball2d* s, uint32_t iteration, or_step_stats* stats);
// Runs n_steps steps starting at iteration first_iteration; returns the number of
// steps whose solve did not converge.  stats (may be NULL) gets the last step's.
int or_ball2d_run(or_ball2d* s, uint32_t first_iteration, uint32_t n_steps, or_step_stats* stats,
                  int64_t* total_contacts);
void or_ball2d_get_state(const or_ball2d* s, double* q, double* v);
void or_ball2d_set_state(or_ball2d* s, const double* q, const double* v);
// Sweep order for the next step's solve only (a permutation of its nc contacts, e.g.
// the GPU's colour order); ignored if the contact count differs.
void or_ball2d_set_next_order(or_ball2d* s, int64_t nc, const int32_t* order);
// Replaces the impulse cache with the given contacts' impulses (ib = -1 - plane for a plane).
void or_ball2d_set_cache(or_ball2d* s, int64_t nc, const int32_t* ia, const int32_t* ib, const double* alpha,
                         const double* beta);
// New solver tolerance and iteration cap (scene and impulse cache kept).
void or_ball2d_set_solver(or_ball2d* s, double tol, uint32_t max_iters);
// Contacts of the last step: ia, ib (ib=-1-plane_idx for planes), n (2 per contact), alpha, beta.
int64_t or_ball2d_last_contacts(const or_ball2d* s, int64_t cap, int32_t* ia, int32_t* ib, double* n,
                                double* alpha, double* beta);
// Active set only (no solve) for the given (q0, q1): used for contact-set parity.
int64_t or_ball2d_active_set(const or_ball2d* s, const double* q0, const double* q1, int64_t cap,
                             int32_t* ia, int32_t* ib);
// Unconstrained map only.
void or_ball2d_umap(const or_ball2d* s, uint32_t iteration, const double* q0, const double* v0, double* q1,
                    double* v1);

// ---------------------------------------------------------------- RigidBody3D spheres
// 3D So-bogus restatement (Sobogus.cpp:184-251,486-594).  Body b: mass m[b], world inertia Iw and
// its inverse Iinv (row-major 3x3, 9 per body); v0, v2, f: [v (3nb) | omega (3nb)].  Contact k:
// bases 9 per contact, column-major [n s t]; arm_a/arm_b: contact point minus body centre
// (arm_a = -r n for plane contacts, whose ib is -1).  alpha (nc) / beta (2nc): warm start in, solution out.
void or_sobogus_solve_3d(int nb, const double* m, const double* Iinv, const double* Iw, const double* v0, int nc,
                         const int32_t* ia, const int32_t* ib, const double* bases, const double* arm_a,
                         const double* arm_b, const double* CoR, const double* mu, const or_gs_params* p,
                         double* alpha, double* beta, double* v2, double* f, or_gs_result* res);
// As or_sobogus_solve_3d with the map's extra relative velocities (nrel: 1, drel: 2 per contact).
void or_sobogus_solve_3d_ex(int nb, const double* m, const double* Iinv, const double* Iw, const double* v0,
                            int nc, const int32_t* ia, const int32_t* ib, const double* bases, const double* arm_a,
                            const double* arm_b, const double* CoR, const double* mu, const double* nrel,
                            const double* drel, const or_gs_params* p, double* alpha, double* beta, double* v2,
                            double* f, or_gs_result* res);
double or_residual_3d(int nb, const double* m, const double* Iinv, const double* Iw, const double* v0, int nc,
                      const int32_t* ia, const int32_t* ib, const double* bases, const double* arm_a,
                      const double* arm_b, const double* CoR, const double* mu, const double* alpha,
                      const double* beta);
// The same with the map's extra relative velocities (nrel: 1, drel: 2 per contact; null = zero).
double or_residual_3d_ex(int nb, const double* m, const double* Iinv, const double* Iw, const double* v0, int nc,
                         const int32_t* ia, const int32_t* ib, const double* bases, const double* arm_a,
                         const double* arm_b, const double* CoR, const double* mu, const double* nrel,
                         const double* drel, const double* alpha, const double* beta);

// RigidBodySphere::computeMassAndInertia (RigidBodySphere.cpp:10-18): mass and principal inertia.
void or_sphere_mass_inertia(double r, double density, double* M, double* I);

typedef struct or_sphere3d or_sphere3d;

typedef struct {
  double dt;
  double gravity[3];
  double mu;
  double CoR;
  double tol;
  uint32_t max_iters;
  uint32_t eval_every;
  int32_t staggering;             // OR_STAGGER_GEOMETRIC (SplitHam map) or OR_STAGGER_SYMPLECTIC_EULER
  int32_t cache_mode;             // symplectic Euler: OR_CACHE_* (the geometric 3D map keeps none)
  int32_t stabilize;              // symplectic Euler: pose stabilisation g0 / dt
  double penetration_threshold;   // symplectic Euler: gaps smaller in magnitude are ignored
} or_sphere3d_params;

// q: [x (3nb) | R row-major (9nb)], v: [v (3nb) | omega (3nb)], r, m per body, I0: 3 per body.
// Planes: x and unit n, 3 each.  Geometric staggering with the SplitHam map and no impulse cache,
// or SymplecticEulerImpactFrictionMap (exponential-Euler configuration updates, impulse cache with
// the transport of cached forces to the new normal, optional pose stabilisation).
or_sphere3d* or_sphere3d_create(int nb, const double* q, const double* v, const double* r, const double* m,
                                const double* I0, int np, const double* plane_x, const double* plane_n,
                                const or_sphere3d_params* p);
void or_sphere3d_destroy(or_sphere3d* s);
int or_sphere3d_step(or_sphere3d* s, uint32_t iteration, or_step_stats* stats);
int or_sphere3d_run(or_sphere3d* s, uint32_t first_iteration, uint32_t n_steps, or_step_stats* stats,
                    int64_t* total_contacts);
void or_sphere3d_get_state(const or_sphere3d* s, double* q, double* v);
// Sets (q, v) and recomputes the world inertia from R (updateMandMinv).
void or_sphere3d_set_state(or_sphere3d* s, const double* q, const double* v);
void or_sphere3d_world_inertia(const or_sphere3d* s, double* Iw, double* Iinv);
void or_sphere3d_umap(const or_sphere3d* s, const double* q0, const double* v0, double* q1, double* v1);
void or_sphere3d_set_solver(or_sphere3d* s, double tol, uint32_t max_iters);
void or_sphere3d_set_next_order(or_sphere3d* s, int64_t nc, const int32_t* order);
int64_t or_sphere3d_active_set(const or_sphere3d* s, const double* q0, const double* q1, int64_t cap,
                               int32_t* ia, int32_t* ib);
// Contacts of the last step (ib = -1 - plane for planes); any output pointer may be NULL.
int64_t or_sphere3d_last_contacts(const or_sphere3d* s, int64_t cap, int32_t* ia, int32_t* ib, double* bases,
                                  double* arm_a, double* arm_b, double* alpha, double* beta);

// ---------------------------------------------------------------- RigidBody2D circles
// q = [x y theta] per body, v = [vx vy omega] per body (RigidBody2DState's layout); r, m, I per
// body (CircleGeometry::computeMassAndInertia gives m = rho pi r^2, I = m r^2 / 2); planes 2 each.
typedef struct or_rb2d or_rb2d;

typedef struct {
  int32_t integrator;  // OR_SYMPLECTIC_EULER / OR_VERLET (rigidbody2d/SymplecticEulerMap.cpp, VerletMap.cpp)
  int32_t cache_mode;  // OR_CACHE_*
  double dt;
  double gravity[2];
  double mu;
  double CoR;
  double tol;
  uint32_t max_iters;
  uint32_t eval_every;
  int32_t staggering;  // OR_STAGGER_GEOMETRIC or OR_STAGGER_STABILIZED
} or_rb2d_params;

or_rb2d* or_rb2d_create(int nb, const double* q, const double* v, const double* r, const double* m,
                        const double* I, int np, const double* plane_x, const double* plane_n,
                        const or_rb2d_params* p);
void or_rb2d_destroy(or_rb2d* s);
// One GeometricImpactFrictionMap::flow step of RigidBody2DSim with Sobogus(RigidBody2D).
int or_rb2d_step(or_rb2d* s, uint32_t iteration, or_step_stats* stats);
int or_rb2d_run(or_rb2d* s, uint32_t first_iteration, uint32_t n_steps, or_step_stats* stats,
                int64_t* total_contacts);
void or_rb2d_get_state(const or_rb2d* s, double* q, double* v);
void or_rb2d_set_state(or_rb2d* s, const double* q, const double* v);
void or_rb2d_set_solver(or_rb2d* s, double tol, uint32_t max_iters);
void or_rb2d_set_next_order(or_rb2d* s, int64_t nc, const int32_t* order);
// Contacts of the last step (ib = -1 - plane for planes), normals (2 per contact), angular
// entries of the tangent rows (cross(arm, t) for body a and body b; 0 for a plane's b) and
// impulses; any output pointer may be NULL.
int64_t or_rb2d_last_contacts(const or_rb2d* s, int64_t cap, int32_t* ia, int32_t* ib, double* n, double* ta,
                              double* tb, double* alpha, double* beta);

// ---------------------------------------------------------------- warm-start network
// 12 -> 64 -> 64 -> 3 MLP with GELU; parameters W1 (64x12), b1, W2 (64x64), b2, W3 (3x64), b3.
int or_mlp_param_count(void);
void or_mlp_forward(const float* params, int n, const float* x, double* y);
// Mean loss over n samples and its gradient (FP64) with respect to the packed parameters.
double or_mlp_loss_grad(const float* params, int n, const float* x, const float* t, double* grad);

#ifdef __cplusplus
}
#endif

#endif
