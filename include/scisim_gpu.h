/* scisim_gpu.h -- C ABI of the GB300 (sm_103a) SCISim contact-path library.
 *
 * libscisim_gb300.so exposes SCISim's per-step contact path for Ball2D discs and
 * RigidBody3D spheres: unconstrained maps, spatial-grid broad phase, CCD / sphere
 * narrow phase, contact bases and forcing terms, Delassus diagonal blocks,
 * graph-coloured block Gauss-Seidel Coulomb solve, impulse cache, on one GPU.  All
 * arguments are plain C types and host pointers in SCISim's own layouts (Ball2D q, v
 * interleaved [x0 y0 x1 y1 ...]; RigidBody3D q = [x (3nb) | R row-major (9nb)],
 * v = [v (3nb) | omega (3nb)]; FP64).  No call throws; every entry point returns an
 * sg_status.
 *
 * Each entry point names the reference interface it replaces (file:line within
 * breannansmith/scisim).  A context is single-threaded: one host thread per
 * context, calls are stream-ordered on the context's own CUDA stream.
 */
#ifndef SCISIM_GPU_H
#define SCISIM_GPU_H

#include <stdint.h>

#if defined(__GNUC__)
#define SG_API __attribute__((visibility("default")))
#else
#define SG_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  SG_OK = 0,
  SG_NOT_CONVERGED = 1,  /* solve hit max_iters; the best iterate is returned
                            (GeometricImpactFrictionMap.cpp:346-350 warns and goes on) */
  SG_BAD_INPUT = 2,      /* invalid sizes, pointers or parameters */
  SG_DEVICE_TIMEOUT = 3, /* a bounded device-side wait expired; the context stays usable */
  SG_CUDA_ERROR = 4,     /* a CUDA runtime call failed (see sg_last_error_string) */
  SG_CAPACITY = 5        /* a fixed internal limit was exceeded (e.g. > 64 colours) */
} sg_status;

/* Unconstrained maps: ball2d/SymplecticEulerMap.cpp, ball2d/VerletMap.cpp (Ball2D) and
 * rigidbody3d/UnconstrainedMaps/SplitHamMap.cpp (RigidBody3D). */
enum { SG_SYMPLECTIC_EULER = 0, SG_VERLET = 1, SG_SPLIT_HAM = 2 };
/* ImpulsesToCache (scisim/ConstrainedMaps/ImpulsesToCache.h) */
enum { SG_CACHE_NONE = 0, SG_CACHE_NORMAL = 1, SG_CACHE_NORMAL_AND_FRICTION = 2 };
/* Staggering of a Ball2D step: GeometricImpactFrictionMap, SymplecticEulerImpactFrictionMap or
 * StabilizedImpactFrictionMap. */
enum { SG_STAGGER_GEOMETRIC = 0, SG_STAGGER_SYMPLECTIC_EULER = 1, SG_STAGGER_STABILIZED = 2 };
/* Arithmetic of the Gauss-Seidel sweeps. */
enum { SG_PRECISION_FP64 = 0, SG_PRECISION_FP32_REFINE = 1 };

typedef struct {
  int32_t integrator;  /* SG_SYMPLECTIC_EULER | SG_VERLET (Ball2D scenes), SG_SPLIT_HAM (sphere scenes) */
  int32_t cache_mode;  /* SG_CACHE_*  (GeometricImpactFrictionMap ctor, GeometricImpactFrictionMap.cpp:20) */
  int32_t precision;   /* SG_PRECISION_* */
  int32_t device;      /* CUDA device ordinal */
  double dt;
  double gravity[3];   /* Ball2DGravityForce (ball2d/Forces/Ball2DGravityForce.cpp:36-46) uses [0..1];
                          NearEarthGravityForce (rigidbody3d/Forces/NearEarthGravityForce.cpp:39-54) [0..2] */
  double mu;           /* default friction coefficient (Ball2DSim::flow argument) */
  double CoR;          /* default coefficient of restitution */
  double tol;          /* absolute Coulomb residual tolerance (GeometricImpactFrictionMap m_abs_tol) */
  uint32_t max_iters;  /* Gauss-Seidel iteration cap (m_max_iters) */
  uint32_t eval_every; /* residual evaluation period (Sobogus m_eval_every) */
} sg_config;

typedef struct {
  int64_t n_contacts;
  int64_t n_ball_ball;
  int64_t n_ball_plane;
  uint32_t iterations; /* Gauss-Seidel sweeps executed */
  int32_t succeeded;   /* error < tol */
  double error;        /* best Coulomb residual (infinity norm of per-contact FB error) */
  uint32_t n_colors;   /* colours of the contact graph */
  uint32_t reserved;
} sg_step_stats;

typedef struct sg_ctx sg_ctx;

/* Human-readable description of the last failure on this thread. */
SG_API const char* sg_last_error_string(void);

/* Creates a context on cfg->device; all device memory is owned by the context.  Replaces
 * constructing the step's objects: the impact-friction map (GeometricImpactFrictionMap ctor,
 * scisim/ConstrainedMaps/GeometricImpactFrictionMap.cpp:20-31: tol, max_iters, impulses to cache),
 * the friction solver (Sobogus ctor, scisim/ConstrainedMaps/Sobogus.cpp:642-645: eval_every) and
 * the unconstrained map (cfg->integrator); the scene is uploaded separately.  sg_ctx_destroy
 * releases the context and all its device memory. */
SG_API int sg_ctx_create(const sg_config* cfg, sg_ctx** out);
SG_API void sg_ctx_destroy(sg_ctx* ctx);

/* Replaces the solver settings (tol, max_iters, eval_every, cache mode, precision,
 * mu, CoR, dt, gravity, integrator) of a context, keeping its scene and impulse cache
 * (as rebuilding a GeometricImpactFrictionMap with new settings on the same
 * Ball2DSim would).  cfg->device must equal the context's device. */
SG_API int sg_ctx_reconfigure(sg_ctx* ctx, const sg_config* cfg);

/* Uploads a Ball2D scene (replaces Ball2DState setup: ball2d/Ball2DState.cpp:40-77,
 * StaticPlane ctor ball2d/StaticGeometry/StaticPlane.cpp:10-19).
 * q, v: 2*nb interleaved; r, m: nb; plane_x, plane_n: 2*np (normals are normalised
 * here, tangents t = (-n_y, n_x)).  Clears the impulse cache. */
SG_API int sg_ball2d_upload(sg_ctx* ctx, int32_t nb, const double* q, const double* v, const double* r,
                     const double* m, int32_t np, const double* plane_x, const double* plane_n);

/* Uploads a RigidBody3D scene of spheres (replaces RigidBody3DState setup:
 * rigidbody3d/RigidBody3DState.cpp:140-300, StaticPlane rigidbody3d/StaticGeometry/StaticPlane.cpp:10-15).
 * q: 12nb [x | R row-major], v: 6nb [v | omega]; r, m: nb; I0: 3nb principal moments
 * (RigidBodySphere::computeMassAndInertia, rigidbody3d/Geometry/RigidBodySphere.cpp:10-18, gives
 * m and I0 from r and the density); plane_x, plane_n: 3np (normals are normalised here).
 * The world inertia is formed from R as the reference's constructor does.  The context's
 * integrator must be SG_SPLIT_HAM; the 3D geometric map keeps no impulse cache
 * (rigidbody3dutils/RigidBody3DSceneParser.cpp:1877-1880). */
SG_API int sg_sphere3d_upload(sg_ctx* ctx, int32_t nb, const double* q, const double* v, const double* r,
                              const double* m, const double* I0, int32_t np, const double* plane_x,
                              const double* plane_n);

/* Uploads a RigidBody2D scene of circles (replaces RigidBody2DState setup with CircleGeometry bodies:
 * rigidbody2d/RigidBody2DState.cpp, rigidbody2d/CircleGeometry.cpp; StaticPlane as the rigidbody2d
 * scene parser stores it, rigidbody2dutils/RigidBody2DSceneParser.cpp:271-277).  q, v: 3 per body
 * ([x y theta], [vx vy omega], RigidBody2DState's layout); r, m, I: per body (mass and moment of
 * inertia; Minv = diag(1/m, 1/m, 1/I)); plane_x, plane_n: 2 per plane (normals are normalised
 * here).  sg_step and sg_flow then step it with GeometricImpactFrictionMap::flow
 * (scisim/ConstrainedMaps/GeometricImpactFrictionMap.cpp:267-442) or, after
 * sg_set_staggering(SG_STAGGER_STABILIZED), StabilizedImpactFrictionMap::flow
 * (scisim/ConstrainedMaps/StabilizedImpactFrictionMap.cpp:48-167): the context's integrator
 * (SG_SYMPLECTIC_EULER or SG_VERLET, rigidbody2d/SymplecticEulerMap.cpp, VerletMap.cpp), the
 * active set of RigidBody2DSim (rigidbody2d/RigidBody2DSim.cpp:248-312,638-714: swept-AABB grid,
 * CCD, planes on the predictor), and Sobogus with SobogusSolverType::RigidBody2D
 * (scisim/ConstrainedMaps/Sobogus.cpp:110-182,375-484) in FP64 sweeps (the context's precision
 * does not apply).  Clears the impulse cache.  Checkpoints and the autotuner do not take
 * RigidBody2D scenes. */
SG_API int sg_rigidbody2d_upload(sg_ctx* ctx, int32_t nb, const double* q, const double* v, const double* r,
                                 const double* m, const double* I, int32_t np, const double* plane_x,
                                 const double* plane_n);

/* Contacts of the last RigidBody2D step in active-set order (RigidBody2DSim::computeActiveSet,
 * rigidbody2d/RigidBody2DSim.cpp:696-714): ia, ib (ib = -1 - plane), n (2 per contact), ta, tb
 * (the tangent row's angular entries cross(arm_a, t), cross(arm_b, t) of CircleCircleConstraint /
 * StaticPlaneCircleConstraint::evalH; tb = 0 for a plane), alpha, beta (Sobogus.cpp:421-437).  Any
 * output may be NULL.  Returns the contact count, -(count+1) if cap is too small, INT64_MIN when
 * the context holds no RigidBody2D scene. */
SG_API int64_t sg_rigidbody2d_last_contacts(sg_ctx* ctx, int64_t cap, int32_t* ia, int32_t* ib, double* n,
                                            double* ta, double* tb, double* alpha, double* beta);

/* Uploads S independent sphere scenes stepped together (no counterpart in the reference, whose
 * driver steps one RigidBody3DSim).  Scene s owns bodies body_off[s] .. body_off[s+1]-1 and planes
 * plane_off[s] .. plane_off[s+1]-1 and has its own mu[s] and CoR[s]; q: [x (3N) | R (9N)],
 * v: [v (3N) | omega (3N)] over all N = body_off[S] bodies, r, m: N, I0: 3N, planes 3 each.
 * sg_step then steps every scene as sg_sphere3d_upload + sg_step would step it alone: its own
 * broad phase, its contacts in the reference's order, and its own Gauss-Seidel termination
 * (residual, best iterate, iteration count), every scene solved in one launch, in FP64 or (the
 * context's precision SG_PRECISION_FP32_REFINE) in FP32 sweeps with FP64 checks and refinement
 * decided scene by scene; sg_batch2d_scene_stats reports each scene.  The integrator must be
 * SG_SPLIT_HAM. */
SG_API int sg_sphere3d_batch_upload(sg_ctx* ctx, int32_t n_scenes, const int32_t* body_off, const double* q,
                                    const double* v, const double* r, const double* m, const double* I0,
                                    const int32_t* plane_off, const double* plane_x, const double* plane_n,
                                    const double* mu, const double* CoR);

/* Uploads n_scenes independent Ball2D scenes stepped together (no counterpart in the
 * reference, whose driver steps one Ball2DSim; each scene evolves exactly as
 * Ball2DSim::flow would step it alone, ball2d/Ball2DSim.cpp:305-326).  Scene s owns bodies
 * [body_off[s], body_off[s+1]) of q, v (interleaved, 2 per body), r, m and planes
 * [plane_off[s], plane_off[s+1]) of plane_x, plane_n (2 per plane); mu[s] and CoR[s] are
 * its coefficients.  Contacts never join bodies of different scenes; each scene's
 * Gauss-Seidel solve stops at its own tolerance (or max_iters) and keeps its own best
 * iterate.  sg_step then runs the whole batch from a CUDA graph of 8 steps with device-side
 * contact counts; a chunk whose contacts overflow the capacity is re-run from its start
 * with more capacity.  Global indices are kept (ib = -1 - global plane index). */
SG_API int sg_batch2d_upload(sg_ctx* ctx, int32_t n_scenes, const int32_t* body_off, const double* q,
                             const double* v, const double* r, const double* m, const int32_t* plane_off,
                             const double* plane_x, const double* plane_n, const double* mu, const double* CoR);

/* Contact capacity of a batched context (no counterpart; default 3 per body + 1024).  It grows by itself
 * when a step overflows it; a smaller value bounds device memory up front. */
SG_API int sg_batch2d_set_capacity(sg_ctx* ctx, int32_t contacts);

/* Per-scene results of the last batched step (Ball2D or sphere batch): contact count,
 * Gauss-Seidel sweeps, best residual and whether the scene's solve reached the tolerance, as
 * the step statistics of each scene's own GeometricImpactFrictionMap::flow would report them
 * (scisim/ConstrainedMaps/GeometricImpactFrictionMap.cpp:344-350).  Any output may be NULL. */
SG_API int sg_batch2d_scene_stats(sg_ctx* ctx, int32_t* n_contacts, uint32_t* iterations, double* error,
                                  int32_t* succeeded);

/* Advances the device-resident scene by n_steps steps of
 * GeometricImpactFrictionMap::flow (scisim/ConstrainedMaps/GeometricImpactFrictionMap.cpp:267-442)
 * as driven by Ball2DSim::flow (ball2d/Ball2DSim.cpp:305-326) or RigidBody3DSim::flow
 * (rigidbody3d/RigidBody3DSim.cpp:557-630, world inertia updated after each step).  first_iteration is
 * the step index of the first step (SCISim counts from 1).  stats (may be NULL)
 * receives the last step's counters; total_contacts (may be NULL) the sum of
 * active contacts over the n_steps steps.  Returns SG_NOT_CONVERGED if any step's
 * solve hit max_iters. */
SG_API int sg_step(sg_ctx* ctx, uint32_t first_iteration, uint32_t n_steps, sg_step_stats* stats,
            int64_t* total_contacts);

/* ImpactFrictionMap::flow with host buffers (scisim/ConstrainedMaps/ImpactFrictionMap.h:36):
 * uploads (q0, v0), runs one step and downloads (q1, v1).  The impulse cache lives
 * in the context, as SCISim's ConstraintCache lives in Ball2DSim. */
SG_API int sg_flow(sg_ctx* ctx, uint32_t iteration, const double* q0, const double* v0, double* q1, double* v1,
            sg_step_stats* stats);

/* Downloads the device-resident state (Ball2DState::q()/v(), ball2d/Ball2DState.h:34-39;
 * RigidBody3DState::q()/v(), rigidbody3d/RigidBody3DState.h:40-44; the same layouts). */
SG_API int sg_download_state(sg_ctx* ctx, double* q, double* v);

/* Contacts of the last step in active-set order (Ball2DSim::computeActiveSet,
 * ball2d/Ball2DSim.cpp:151-173): ia, ib (ib = -1 - plane for a static plane),
 * n (2 per contact), alpha, beta (Sobogus.cpp:312-347).  Any output may be NULL.
 * Returns the contact count, or -(count+1) if cap is too small; INT64_MIN on a
 * sphere-scene context. */
SG_API int64_t sg_last_contacts(sg_ctx* ctx, int64_t cap, int32_t* ia, int32_t* ib, double* n, double* alpha,
                         double* beta);

/* Contacts of the last sphere-scene step in active-set order (RigidBody3DSim::computeActiveSet,
 * rigidbody3d/RigidBody3DSim.cpp:250-262): ia, ib (ib = -1 - plane), bases (9 per contact,
 * column-major [n s t], RigidBody3DSim::computeContactBases :277-290), alpha (1) and beta (2
 * per contact, Sobogus.cpp:526-542).  Any output may be NULL.  Returns the contact count,
 * -(count+1) if cap is too small, INT64_MIN on a Ball2D context. */
SG_API int64_t sg_sphere3d_last_contacts(sg_ctx* ctx, int64_t cap, int32_t* ia, int32_t* ib, double* bases,
                                         double* alpha, double* beta);

/* World inertia and its inverse of every sphere (the angular blocks of RigidBody3DState's
 * M and Minv, rigidbody3d/RigidBody3DState.cpp:428-462), 9 per body, row-major. */
SG_API int sg_sphere3d_world_inertia(sg_ctx* ctx, double* Iw, double* Iinv);

/* The Gauss-Seidel processing order of the last step's solve (contacts of colour 0,
 * then colour 1, ...) and the colour offsets (n_colors + 1 entries).  No counterpart: the
 * reference sweeps in active-set order without colouring
 * (scisim/ConstrainedMaps/bogus/Ball2DSobogusInterface.cpp:124-133, max_threads 0); the oracle
 * replays this order to compare whole steps bit for bit.  Returns the contact count, or
 * -(count+1) if cap is too small. */
SG_API int64_t sg_last_solve_order(sg_ctx* ctx, int64_t cap, int32_t* order, int32_t* color_offsets,
                            int32_t* n_colors);

/* FrictionSolver::solve for Ball2D (scisim/ConstrainedMaps/FrictionSolver.h:28,
 * Sobogus::solve scisim/ConstrainedMaps/Sobogus.cpp:880-1088) on host buffers.
 * m: nb masses; v0: 2nb; ia/ib: contact bodies (ib = -1 static); bases: 4 per contact,
 * column-major [n t]; CoR, mu: per contact; alpha/beta: in = warm start, out = result;
 * v2, f: 2nb outputs; error/iterations: outputs.  Returns SG_NOT_CONVERGED when the
 * solve hit max_iters (solve_succeeded = false in SCISim). */
SG_API int sg_sobogus_solve_2d(sg_ctx* ctx, int32_t nb, const double* m, const double* v0, int32_t nc,
                        const int32_t* ia, const int32_t* ib, const double* bases, const double* CoR,
                        const double* mu, uint32_t max_iters, double tol, uint32_t eval_every,
                        double* alpha, double* beta, double* v2, double* f, double* error,
                        uint32_t* iterations);

/* FrictionSolver::solve for Ball2D with all of its inputs (scisim/ConstrainedMaps/FrictionSolver.h:28):
 * sg_sobogus_solve_2d plus the impact-friction map's extra relative velocities nrel_extra and
 * drel_extra (one each per contact; NULL = zero), which Sobogus::solve adds to the kinematic
 * relative velocities before forming the forcing terms (scisim/ConstrainedMaps/Sobogus.cpp:892-904;
 * SymplecticEulerImpactFrictionMap passes N^T vdelta and D^T vdelta there,
 * scisim/ConstrainedMaps/SymplecticEulerImpactFrictionMap.cpp:293-329).  With both NULL it is
 * sg_sobogus_solve_2d bit for bit. */
SG_API int sg_sobogus_solve_2d_ex(sg_ctx* ctx, int32_t nb, const double* m, const double* v0, int32_t nc,
                                  const int32_t* ia, const int32_t* ib, const double* bases, const double* CoR,
                                  const double* mu, const double* nrel_extra, const double* drel_extra,
                                  uint32_t max_iters, double tol, uint32_t eval_every, double* alpha, double* beta,
                                  double* v2, double* f, double* error, uint32_t* iterations);

/* FrictionSolver::solve for RigidBody3D spheres (Sobogus::solve with SobogusSolverType::RigidBodies3D:
 * scisim/ConstrainedMaps/Sobogus.cpp:184-251 (initialize3D), :486-567 (solve3D);
 * scisim/ConstrainedMaps/bogus/RigidBody3DSobogusInterface.cpp:31-145) on host buffers.
 * Bodies: m (nb masses), Iw and Iinv (9 per body, row-major world inertia and its inverse: the
 * angular blocks of RigidBody3DState's M and Minv), v0 (6nb, [v (3nb) | omega (3nb)]).
 * Contacts: ia, ib (ib = -1 for a static plane); bases (9 per contact, column-major [n s t],
 * right-handed orthonormal); arm_a, arm_b (3 per contact: the world contact point minus the
 * body's centre, Constraint::getWorldSpaceContactPoint; arm_b is ignored for planes); the
 * normal row carries no torque (sphere contacts: SphereSphereConstraint::evalH,
 * rigidbody3d/Constraints/SphereSphereConstraint.cpp:254-265, asserts |arm x n| <= 1e-6, as this
 * entry does); CoR, mu (per contact); nrel_extra (nc) and drel_extra (2nc, [s t] per contact),
 * NULL = zero; alpha (nc) and beta (2nc) in = warm start, out = result; v2, f (6nb) outputs
 * (f: the friction impulse and its torque, Sobogus.cpp:533-567).  Returns SG_NOT_CONVERGED when the
 * solve hit max_iters, SG_BAD_INPUT for invalid indices, bases or arms. */
SG_API int sg_sobogus_solve_3d(sg_ctx* ctx, int32_t nb, const double* m, const double* Iw, const double* Iinv,
                               const double* v0, int32_t nc, const int32_t* ia, const int32_t* ib,
                               const double* bases, const double* arm_a, const double* arm_b, const double* CoR,
                               const double* mu, const double* nrel_extra, const double* drel_extra,
                               uint32_t max_iters, double tol, uint32_t eval_every, double* alpha, double* beta,
                               double* v2, double* f, double* error, uint32_t* iterations);

/* The FrictionSolver solve above for callers that cannot allocate GPU memory: code
 * that runs inside another runtime's memory pool, in a real-time loop, or under a
 * policy that forbids device allocation after start-up.  It has no counterpart in the
 * reference.  Every array argument is a DEVICE pointer the caller owns (same meanings
 * and layouts as sg_sobogus_solve_2d); error and iterations are host pointers; stream
 * is a cudaStream_t (NULL = default stream).  No context is needed and nothing is
 * allocated: all scratch lives in one fixed static device array of about 8.1 MB that
 * every GPU loading the library keeps until the process exits.  Limits: at most
 * 16,384 bodies and 65,536 contacts; larger problems return SG_CAPACITY.  The array's
 * device address is looked up (cudaGetSymbolAddress) on the first call in each context
 * of a device -- again after the device's context was re-created, e.g. by
 * cudaDeviceReset -- so make the first call on each device before any stream capture.
 * The device is the calling thread's current device, and stream must belong to it.  The
 * call synchronises stream before it returns (it reads the device-side input check and
 * the solve statistics), so it cannot be made while stream is being captured.  All
 * calls share the array: calls that overlap on the GPU (other streams, other host
 * threads) race and must be serialised by the caller.  The solve takes no extra
 * relative velocities (those of sg_sobogus_solve_2d_ex are zero here).  Returns as
 * sg_sobogus_solve_2d; invalid contact indices or tangents give SG_BAD_INPUT before
 * any solve work. */
SG_API int sg_sobogus_solve_2d_noalloc(int32_t nb, const double* m, const double* v0, int32_t nc,
                                       const int32_t* ia, const int32_t* ib, const double* bases,
                                       const double* CoR, const double* mu, uint32_t max_iters, double tol,
                                       uint32_t eval_every, double* alpha, double* beta, double* v2, double* f,
                                       void* stream, double* error, uint32_t* iterations);

/* SpatialGridDetector::getPotentialOverlaps (ball2d/SpatialGridDetector.cpp:106-133):
 * all overlapping pairs (i<j) of n AABBs [minx miny maxx maxy], in lexicographic
 * order.  Returns SG_CAPACITY with *npairs = required count if cap is too small. */
SG_API int sg_broadphase_2d(sg_ctx* ctx, int32_t n, const double* aabb, int64_t cap, int32_t* pairs,
                     int64_t* npairs);

/* CollisionDetectionUtilities::ballBallCCDCollisionHappens
 * (scisim/CollisionDetection/CollisionDetectionUtilities.cpp:60-126) for n ball pairs;
 * q0a, q1a, q0b, q1b: 2n; ra, rb: n.  Outputs coeffs (3n), hit (n), t (n). */
SG_API int sg_ccd_2d(sg_ctx* ctx, int32_t n, const double* q0a, const double* q1a, const double* ra,
              const double* q0b, const double* q1b, const double* rb, double* coeffs, int32_t* hit,
              double* t);

/* Learned warm start for single Ball2D scenes (no counterpart in the reference, whose solve
 * starts from the impulse cache, GeometricImpactFrictionMap.cpp:174-220).  A 12 -> 64 -> 64 -> 3
 * network (GELU) maps 12 per-contact features (relative velocity, gap, mass ratio, gravity
 * direction, mu, CoR, cached impulse, coordination; scaled by |g| dt and the contact's
 * effective mass) to a start impulse for the contacts the impulse cache missed (cached
 * contacts keep their cached impulse); each step evaluates the FP64
 * Coulomb residual of the cache start and of the network start and solves from the smaller,
 * to the same tolerance as ever.  Parameters: W1 (64x12 row-major), b1 (64), W2 (64x64), b2,
 * W3 (3x64), b3 (3): sg_mlp_param_count() floats.  Inference runs on the tensor cores (BF16
 * inputs and weights, FP32 accumulation); training (FP32 forward, backward, Adam) on CUDA cores. */
SG_API int sg_mlp_param_count(void);
SG_API int sg_mlp_load(sg_ctx* ctx, const float* params, int32_t n_params);
/* warm_start: use the loaded network in every step; record: keep each step's features and
 * targets (the converged impulses, scaled) for sg_mlp_last_samples. */
SG_API int sg_mlp_enable(sg_ctx* ctx, int32_t warm_start, int32_t record);
/* Features (12 per contact) and targets (3 per contact) of the last recorded step.  Returns
 * the sample count, -(count+1) if cap is too small, INT64_MIN when recording is off. */
SG_API int64_t sg_mlp_last_samples(sg_ctx* ctx, int64_t cap, float* x, float* t);
/* Trains params (in: initial, out: trained) with Adam on n samples for `epochs` passes in
 * minibatches of `batch`; epoch_loss (may be NULL) receives the mean loss of each epoch. */
SG_API int sg_mlp_train(sg_ctx* ctx, int64_t n, const float* x, const float* t, int32_t epochs, int32_t batch,
                        float lr, uint64_t seed, float* params, double* epoch_loss);
/* Mean loss and its gradient over n samples (the training kernel's forward and backward). */
SG_API int sg_mlp_grad(sg_ctx* ctx, const float* params, int32_t n, const float* x, const float* t, float* grad,
                       double* loss);
/* Network outputs (3 per sample): tensor_cores = 1 runs the BF16 inference kernel, 0 the FP32 one. */
SG_API int sg_mlp_infer(sg_ctx* ctx, const float* params, int32_t n, const float* x, float* y,
                        int32_t tensor_cores);
/* Steps that evaluated the network start and steps that solved from it. */
SG_API int sg_mlp_stats(sg_ctx* ctx, uint64_t* steps_evaluated, uint64_t* steps_network_start);

/* Counters of the work done since the last reset (no counterpart in SCISim, which has
 * no timing instrumentation: scisim/Timer/TimeUtils.cpp only prints wall-clock strings).
 * gs_ms sums the CUDA-event durations of the Gauss-Seidel kernel (recorded only while
 * profiling is enabled); contact_sweeps / contact_evals count contact updates and
 * residual evaluations; kernel_launches counts this library's kernel launches. */
typedef struct {
  double gs_ms;
  uint64_t gs_launches;
  uint64_t contact_sweeps;
  uint64_t contact_evals;
  uint64_t kernel_launches;
  uint64_t steps;
  uint64_t contacts;
  uint64_t contact_sweeps32; /* contact updates in FP32 sweeps (SG_PRECISION_FP32_REFINE) */
  uint64_t contact_lifts;    /* contacts lifted FP32 -> FP64 before a residual evaluation */
  uint64_t body_lifts;       /* body velocities re-gathered in FP64 for those evaluations */
  uint64_t two_level_solves; /* FP32 solves that ran the two-level (patch) sweeps */
  /* Two-level sweeps as the first block sees them (summed over those solves): time in the
   * patch-interior colours, waiting at the grid barrier after them, and in the contacts
   * between patches; the contacts between patches and the colours of those swept over the
   * grid, summed per solve. */
  double patch_interior_ms;
  double patch_wait_ms;
  double patch_boundary_ms;
  uint64_t boundary_contacts;
  uint64_t boundary_colors;
  double patch_interior_max_ms; /* the slowest block's patch-interior time, summed over solves */
  int64_t patch_slowest_block;  /* that block (= its patch) in the last two-level solve */
  uint64_t patch_contacts_staged; /* per-patch contact capacity staged in shared memory, summed */
  uint64_t fp64_start_solves;  /* FP32-form solves swept in FP64 throughout: converged in the FP64
                                  probe, or within fp64_factor tol after it */
  /* Single-scene Ball2D steps: CUDA-event time of each stage, summed: [0] predictor and grid,
   * [1] pair counting (grid scan, CCD) and plane flags, [2] contact writes and assembly,
   * [3] adjacency and colouring, [4] FP64 probe, two-level partition and FP32 packing, [5] the
   * Gauss-Seidel kernel, [6] final velocity, [7] impulse extraction, cache and final map. */
  double stage_ms[8];
} sg_profile;

SG_API int sg_profile_enable(sg_ctx* ctx, int32_t on);
SG_API int sg_profile_read(sg_ctx* ctx, sg_profile* out, int32_t reset);

/* Two-level sweeps for large single-scene steps of the FP32 form: contacts inside a spatial
 * patch (one per SM) are swept on shared-memory velocities with block barriers, then the
 * contacts between patches that lie inside one tile of the patch tiling shifted by half a
 * tile, the same way; the few left over are swept over the grid.  A Gauss-Seidel order of
 * the same kind as the colour order, with three grid barriers a sweep instead of one per
 * colour.  on: 0 keeps the one-level colour sweeps; 1 (default) takes the two-level sweeps for
 * FP32 sweeps, while a solve that the FP64 probe leaves near tol goes on in up to 160 one-level
 * FP64 sweeps before the two-level ones (near tol the two-level order, which sweeps the contacts
 * between patches after the patches, can hold the residual on a plateau just above tol for
 * hundreds of sweeps that the colour order crosses in tens, while a solve that needs thousands
 * of sweeps either way is cheaper on the partition); 2 takes the two-level sweeps for those FP64
 * sweeps from the start.  SG_BAD_INPUT for other values. */
SG_API int sg_set_two_level(sg_ctx* ctx, int32_t on);

/* The FP32 form's FP64 sweeps after the probe for Ball2D discs, one-level and on the two-level
 * partition (sg_set_two_level): 1 (default) in float-float arithmetic on the FP32 pipe
 * (velocities and impulses as pairs of floats, 48 significant bits; the data split the same way;
 * each check recomputes the velocities from the impulses and evaluates the residual in FP64),
 * which GB300 issues many times faster than FP64; 0 in FP64 arithmetic.  Both iterate to the same
 * FP64 residual checks and tolerance.  SG_BAD_INPUT for other values. */
SG_API int sg_set_fp64_pairs(sg_ctx* ctx, int32_t on);

/* Selects the map a single Ball2D, sphere or RigidBody2D scene steps with (default
 * SG_STAGGER_GEOMETRIC).
 * SG_STAGGER_SYMPLECTIC_EULER is SymplecticEulerImpactFrictionMap
 * (scisim/ConstrainedMaps/SymplecticEulerImpactFrictionMap.cpp:201-407): the force acts first
 * (vdelta = dt Minv F), collisions are detected on q0 + dt (v0 + vdelta), the solve gets the
 * extra relative velocities N^T vdelta and D^T vdelta (plus min(0, gap(q0)) / dt where stabilize
 * is set and the gap exceeds penetration_threshold in magnitude), and the step ends with
 * v1 = v + vdelta, q1 = q0 + dt v1, whatever the context's integrator.  It needs CoR = 0, as the
 * reference does.  SG_STAGGER_STABILIZED is StabilizedImpactFrictionMap
 * (scisim/ConstrainedMaps/StabilizedImpactFrictionMap.cpp:48-167): the unconstrained step, then
 * a cold solve from its velocity, then q1 = q0 + dt v; it keeps no impulse cache (cache_mode NONE).
 * Sphere scenes take SG_STAGGER_SYMPLECTIC_EULER as well: exponential-Euler predictor and
 * configuration update (rigidbody3d/UnconstrainedMaps/IntegrationTools.cpp:3-47) in place of the
 * context's integrator, and with cache_mode set the 3D impulse cache of that map (cached normal
 * and force per contact, the force turned onto the new normal by the quaternion between the two
 * normals, :48-199); stabilized sphere steps return SG_BAD_INPUT.  RigidBody2D scenes take the
 * geometric and the stabilized maps.  Batched scenes step with the geometric map only. */
SG_API int sg_set_staggering(sg_ctx* ctx, int32_t staggering, int32_t stabilize, double penetration_threshold);

/* Checkpoint / resume of a context holding one Ball2D or sphere scene (replaces SCISim's binary
 * serialisation of the simulation, ball2dcli/ball2d_cli.cpp:199-316, Ball2DSim.cpp:810-822).
 * The checkpoint holds the context's settings, the scene (positions, velocities, radii, masses,
 * planes; for spheres the principal and world inertia) and the impulse cache, byte for byte,
 * so that a run resumed with sg_checkpoint_load continues bit-identically.  It does not hold
 * the learned warm start's network.  sg_checkpoint_size returns the bytes sg_checkpoint_save
 * writes (negative for a batched or empty context); sg_checkpoint_load replaces the context's
 * settings (keeping its device) and scene. */
SG_API int64_t sg_checkpoint_size(sg_ctx* ctx);
SG_API int sg_checkpoint_save(sg_ctx* ctx, void* buf, int64_t bytes);
SG_API int sg_checkpoint_load(sg_ctx* ctx, const void* buf, int64_t bytes);

/* Performance knobs that leave the solve's contract unchanged (no counterpart in the reference):
 * two_level (sg_set_two_level: 0, 1 or 2), the contact count from which a single-scene FP32 solve uses the
 * two-level sweeps (default 20,000), and the base interval in sweeps of the FP64 checks of the
 * FP32 form (default 16; the interval grows from it while the residual is far from tol). */
typedef struct {
  int32_t two_level;
  int32_t check_interval;
  int32_t two_level_min_contacts;
  int32_t fp64_factor;  /* FP32 form: a probe of eight one-level FP64 sweeps first; a solve it leaves
                           within fp64_factor tol goes on in FP64 (see sg_set_two_level for the
                           order), any other in FP32 sweeps until the first FP64 check at or
                           below fp64_factor tol (default 100; 0: no probe, FP32 sweeps until their
                           rounding floor) */
} sg_tuning;

SG_API int sg_get_tuning(sg_ctx* ctx, sg_tuning* tuning);
SG_API int sg_set_tuning(sg_ctx* ctx, const sg_tuning* tuning);

/* Autotuner: from the current state of a single-scene context, times trial_steps steps under each
 * candidate (two-level on, check interval 8 / 16 / 32; then two-level off, the same intervals),
 * one untimed run first, each from a checkpoint of that state; restores the state and keeps the
 * fastest candidate, a later candidate replacing an earlier one only when 3 % faster.  ms_per_step (6 entries, may be NULL) gets each candidate's time per step,
 * NaN for candidates that do not apply (the FP64 form has none: its one timing goes to entry 0;
 * sphere scenes have no two-level sweeps).  best (may be NULL) gets the chosen tuning.  The
 * profile counters include the trial steps. */
SG_API int sg_autotune(sg_ctx* ctx, int32_t trial_steps, uint32_t first_iteration, sg_tuning* best,
                       double* ms_per_step);

/* Layout of the last solve's two-level sweeps (diagnostics and tests).  counts[0] = patches P,
 * counts[1] = shifted tiles Pb (the patch tiling shifted by half a tile).  Per contact, in the
 * order of sg_last_contacts: its group (g < P: inside patch g; P <= g < P + Pb: between patches,
 * both bodies in shifted tile g - P; g = P + Pb: the rest, swept over the grid) and the colour
 * it is swept in.  Per body: its patch, its shifted tile and its band flag (1 for an endpoint of
 * a contact between patches).  SG_BAD_INPUT unless the last solve ran the two-level sweeps on
 * nc contacts of the scene's nb bodies. */
SG_API int sg_last_patch_layout(sg_ctx* ctx, int64_t nc, int64_t nb, int32_t* counts, int32_t* group,
                                int32_t* color, int32_t* body_patch, int32_t* body_tile, int32_t* body_band);

/* The context's CUDA stream (cudaStream_t) for stream-ordered timing by the caller (no counterpart). */
SG_API int sg_ctx_stream(sg_ctx* ctx, void** stream);

/* Sets the iteration limit of every device-side wait (grid barriers); 0 restores the
 * default (about a second).  Used to exercise the SG_DEVICE_TIMEOUT path (no counterpart: the
 * reference runs on the CPU and has no device waits). */
SG_API int sg_set_spin_limit(sg_ctx* ctx, uint64_t spins);

/* Runs a kernel that waits on a device flag nothing sets, with the context's spin
 * limit; returns SG_DEVICE_TIMEOUT and leaves the context usable. */
SG_API int sg_selftest_wait_timeout(sg_ctx* ctx);

#ifdef __cplusplus
}
#endif

#endif
