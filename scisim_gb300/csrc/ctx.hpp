// ctx.hpp -- internal state of an sg_ctx and the launchers of the kernel stages.
#pragma once

#include "../../include/scisim_gpu.h"
#include "common.cuh"

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

namespace sg {

// Uniform grid of the broad phase (device resident, written by k_grid_setup).
struct GridParams {
  unsigned long long enc_min[2];  // ordered encodings (atomics)
  unsigned long long enc_max[2];
  unsigned long long enc_ext[2];
  double origin[2];
  double h;
  int dims[2];
  int ncells;
  int pad;
};

// Counters of one Gauss-Seidel solve (device resident).
struct SolveStats {
  unsigned long long err_slot[3];  // ordered encodings of the residual, rotating slots
  int remaining[3];                // colouring: uncoloured contacts per round, rotating slots
  int n_colors;
  int status;                      // 0 ok, SG_CAPACITY / SG_DEVICE_TIMEOUT on failure
  unsigned int iterations;
  int converged;
  double error;
  int color_count[kMaxColors];
  int color_off[kMaxColors + 1];
  int color_fill[kMaxColors];
  unsigned int sweeps32;  // FP32 sweeps (mixed-precision solve)
  unsigned int sweeps64;  // FP64 sweeps
  unsigned int evals;     // FP64 residual evaluations
  unsigned int lifts;     // FP32 -> FP64 lifts (impulses + body velocity gather)
  unsigned long long mag_slot[3];  // ordered max of the FP32 rounding-floor excess per evaluation
  int ig_max[4];                   // highest colour after each iterated-greedy pass
  // Two-level sweeps, as block 0 sees them: time in the patch-interior colours, waiting at
  // the barrier after them, and in the contacts between patches (ns); the contacts between
  // patches and the colours of those swept over the grid.
  unsigned long long phase_ns[3];
  unsigned long long interior_max;  // slowest block's patch-interior time: (ns << 8) | block
  int boundary_contacts;
  int boundary_colors;
};

// A growable device buffer.
struct Buf {
  void* p = nullptr;
  size_t bytes = 0;
  template <typename T>
  T* as() const {
    return static_cast<T*>(p);
  }
};
int grow(Buf& b, size_t bytes);  // contents are not preserved
void release(Buf& b);

// Sizes and pointers of one Ball2D contact problem, as the solver sees it.
struct ContactProblem {
  int nb = 0;
  int nc = 0;
  const double* minv = nullptr;  // nb
  const double* m = nullptr;     // nb
  const double* v0 = nullptr;    // 2nb
  const int* ia = nullptr;       // nc
  const int* ib = nullptr;       // nc, -1 static (any negative value)
  const double* n = nullptr;     // 2nc (t = (-n_y, n_x))
  const double* c = nullptr;     // 2nc local forcing E^T w
  const double* W = nullptr;     // 3nc diagonal Delassus blocks
  const double* mu = nullptr;    // nc
  double* r = nullptr;           // 2nc in: warm start (local), out: solution
  double* v2 = nullptr;          // 2nb out
  // Colours carried over from the step before (nc: the contact's colour then, -1 for a new
  // contact); null: the colouring starts from nothing.
  const int* warm_color = nullptr;
};

// Per-scene solver state of a batched solve (device arrays of S entries).
struct BatchSolve {
  int S = 0;
  const int* nc_dev = nullptr;
  const int* cscene = nullptr;
  const int* sc_off = nullptr;
  unsigned long long* err_slot = nullptr;  // 3 S
  double* best = nullptr;
  int* bestbuf = nullptr;
  int* done = nullptr;
  unsigned* iters = nullptr;
  int* done_count = nullptr;
  unsigned long long* unconverged = nullptr;
  // FP32 sweeps (SG_PRECISION_FP32_REFINE)
  int* pscene = nullptr;            // scene of each packed contact (capacity)
  const int* scene_of = nullptr;    // scene of each body
  int* mode = nullptr;              // S
  unsigned* since = nullptr;        // S
  unsigned long long* exc_slot = nullptr;  // 3 S
  unsigned long long* gmax = nullptr;      // 3
  unsigned long long* work = nullptr;      // 5 counters (FP32 / FP64 updates, evaluations, lifts)
  int* n64 = nullptr;                      // scenes in FP64 mode
  // One block per scene (scene_blocks): every scene's bodies fit in a block's shared memory.
  bool scene_blocks = false;
  const int* sb_off = nullptr;      // S + 1 body offsets
  int* key_cnt = nullptr;           // S * kMaxColors + 1 (scene, colour) counts
  int* key_start = nullptr;         // their exclusive scan
  int* key_fill = nullptr;
  int* sperm = nullptr;             // contacts by (scene, colour)
  const int* order = nullptr;       // scenes, largest first
  int* next = nullptr;              // work-list counter
  int smax = 0;                     // bodies of the largest scene
};

struct SolveParams {
  double tol;
  unsigned int max_iters;
  unsigned int eval_every;
  int precision;
  bool learned = false;  // a scene step: the learned warm start and sample recording apply
};

}  // namespace sg

struct sg_ctx {
  sg_config cfg{};
  cudaStream_t stream = nullptr;
  int device = 0;
  int num_sms = 0;
  unsigned long long spin_limit = 0;
  // Kernel attributes are per device: set once per context (each context has one device).
  int patch_smem_budget = -1;   // k_gs_patch's dynamic shared memory limit, once opted in
  bool patch64_ready = false;   // k_gs_patch64's shared-memory limit set
  bool mlp_smem_set = false;    // k_mlp_fwdbwd's dynamic shared memory limit set

  // Scene: dim 2 = Ball2D (q, v: 2 per body), dim 3 = RigidBody3D spheres
  // (q: [x (3nb) | R row-major (9nb)], v: [v (3nb) | omega (3nb)], SCISim's layouts).
  int dim = 2;
  int nb = 0, np = 0;
  sg::Buf q, v, r, m, minv, q1, v1, v2;
  sg::Buf plane_x, plane_n, plane_t;
  sg::Buf I0, Iw, Iinv;  // 3D: principal inertia (3nb), world inertia and inverse (9nb, row-major)
  // RigidBody2D circles (dim 2, rb2d): q, v hold 3 per body ([x y theta], [vx vy omega]); the moments
  // of inertia and their inverses; the centres at the start and end of the predictor (the broad
  // phase's CCD and the plane test read them as Ball2D positions); per contact the tangent row's
  // angular entries cross(arm_a, t), cross(arm_b, t); running velocities (vx, vy, omega, 0).
  bool rb2d = false;
  sg::Buf rb_I, rb_Iinv, pos0, pos1, rb_ct, rb_vrun;

  // broad phase
  sg::Buf aabb, cell_of, cell_count, cell_start, cell_fill, sorted, pair_cnt, pair_off, grid;
  sg::Buf plane_flag, plane_off, scan_tmp;

  // contacts of the current step
  int64_t ccap = 0;
  sg::Buf ia, ib, n, c, W, mu, r_loc, r_cand, r_best, key, ab;
  // impulse cache of the previous step (sorted keys and (alpha, beta))
  sg::Buf prev_key, prev_ab;
  sg::Buf pair_slots;  // the pair count's first partners per box (8 each), read by the pair write
  sg::Buf aabb32, aabb32s;  // the boxes rounded outward to FP32 (the pair scans' prefilter), by body
                            // and in cell order
  // The rows of the cached step (single-scene Ball2D): pair offsets per body, plane flags and
  // their scan, and its pair count; prev_rows says they belong to the cache held.
  sg::Buf prev_pair_off, prev_plane_off, prev_plane_flag;
  int prev_npairs = 0;
  bool prev_rows = false;
  // The cached step's contact colours (prev_n of them) and each contact's colour carried over
  // (single-scene Ball2D steps with a cache): the colouring starts from them.
  sg::Buf prev_color, init_color;
  bool prev_color_valid = false;
  // Sphere scenes under the symplectic-Euler staggering: 6 doubles per contact (cached normal and
  // force), this step's and the step before's.
  sg::Buf c6, prev_c6;
  int64_t prev_n = 0;

  // solver
  sg::Buf color, perm, body_cnt, body_off, body_fill, body_adj, v_run, stats, barrier;
  // FP32 sweep data, packed in colour order (mixed-precision solve)
  sg::Buf pk_ab, pk_n, pk_c, pk_w, pk_r, v32, minv32;
  // Float-float copies of the FP64 sweep data and state for k_gs_patch_ff (by packed contact: normal,
  // forcing, mu and 1 / w, impulse; by body: velocity, 1 / m).
  sg::Buf ff_n, ff_c, ff_m, ff_r, ff_v, ff_minv;
  // 3D contacts: basis rows n s t (9), angular rows (r_a x s, r_a x t) and (r_b x s, r_b x t)
  // (6 each), forcing (3), Delassus block (6), impulse (3: current, candidate, best),
  // (alpha, beta0, beta1) out (3); running velocities (2 double4 per body: v, omega).
  int64_t ccap3 = 0;
  sg::Buf E3, Aa3, Ab3, c3, W3, r3, r3a, r3b, ab3, vrun3;
  sg::Buf pk3, Iinv32;  // 3D FP32 sweep data (colour-packed contacts, body inverse inertia)
  // Two-level sweeps (spatial patches, one per SM): 0 off, 1 for FP32 sweeps, 2 also for the
  // FP64 sweeps of a solve the probe leaves near tol (sg_set_two_level).
  int patches = 1;
  // FP64 sweeps on the two-level partition in float-float pairs for discs (sg_set_fp64_pairs).
  bool fp64_pairs = true;
  // Staggering of the single-scene Ball2D step (sg_set_staggering): SG_STAGGER_*, and the
  // symplectic Euler map's pose stabilisation and threshold; its velocity change per body.
  int staggering = 0;
  int stabilize = 0;
  double pen_thresh = 0.0;
  sg::Buf vdelta;
  // Tunables (sg_set_tuning / sg_autotune): base interval of the FP64 checks in the FP32 form,
  // and the contact count from which a single-scene FP32 solve uses the two-level sweeps.
  int check_interval = 16;
  int two_level_min_contacts = 20000;
  // FP32 form: FP64 sweeps from the start when the start's residual is below fp64_factor tol, and
  // from the first FP64 check at or below it.
  int fp64_factor = 100;
  uint64_t patched_solves = 0;
  uint64_t fp64_start_solves = 0;  // FP32-form solves swept in FP64 throughout (probe near tol)
  bool last_patched = false;  // the last FP32 solve ran the two-level sweeps
  int last_patch_P = 0, last_patch_Pb = 0;
  uint64_t patch_phase_ns[3] = {0, 0, 0};
  uint64_t patch_interior_max_ns = 0;
  uint64_t patch_staged = 0;  // patch contacts staged in shared memory per launch, summed
  int patch_slowest_block = -1;
  uint64_t patch_boundary_contacts = 0;
  uint64_t patch_boundary_colors = 0;
  sg::Buf pt_setup, pt_patch, pt_lidx, pt_body, pt_cnt, pt_start, pt_fill, pt_key, pt_kcnt, pt_kstart, pt_kfill,
      pt_order, pt_max, pt_bcolor, pt_rem;
  // Shifted tiles and band bodies: tile of each body, band flag, tile-local slot, band bodies by
  // tile; band bodies per patch and the scatter's fill counters.
  sg::Buf pt_qpatch, pt_band, pt_lidxq, pt_qbody, pt_bcnt, pt_nfill, pt_qcnt, pt_qstart, pt_qfill;
  // Bodies of the remaining contacts: flag, slot (exclusive scan of the flags), compacted list.
  sg::Buf pt_cflag, pt_cpos, pt_cbody;
  // Contact-balanced cuts: per-column/row contact histograms, their prefix sums, the cuts, and
  // the cell column/row -> patch and shifted-tile maps.
  sg::Buf pt_hist, pt_pref, pt_cuts, pt_maps;
  // Batched Ball2D scenes (sg_batch2d_upload).  Scene s owns bodies [sb_off[s], sb_off[s+1]),
  // planes [sp_off[s], sp_off[s+1]) and plane flags [sf_off[s], sf_off[s+1]); its contacts of a
  // step are [sc_off[s], sc_off[s+1]).  Counts live on the device (b_ctl: contact count,
  // overflow); the step loop is replayed from a CUDA graph of kGraphSteps steps.
  int n_scenes = 0;  // 0: not a batched context
  long bcells = 0, bflags = 0;
  int bcap = 0;
  sg::Buf sb_off, sp_off, sf_off, scene_of, s_mu, s_CoR, s_grid, s_cells, s_cell_off, s_nc, s_npairs;
  sg::Buf sc_off, prev_sc_off, cscene, b_ctl, b_sums;
  sg::Buf s_err, s_best, s_bestbuf, s_done, s_iters, s_mode, s_since, s_exc, s_gmax, b_work, pk_scene;
  // One block per scene: (scene, colour) counts, their scan and fill, the contacts in that order,
  // the scenes largest first and the work-list counter; s_smax = bodies of the largest scene
  // (0: a scene exceeds a block's shared memory, grid-wide sweeps instead).
  sg::Buf s_kcnt, s_kstart, s_kfill, s_sperm, s_order, s_next;
  int s_smax = 0;
  sg::Buf snap_q, snap_v, snap_key, snap_ab, snap_off;
  cudaGraphExec_t graph = nullptr;
  uint64_t graph_launches = 0;  // kernel launches per graph replay
  // Learned warm start (mlp_kernels.cu): network parameters, per-contact features and
  // targets of the last step, training samples, start-selection slots and counter.
  bool mlp_loaded = false, mlp_on = false, mlp_record = false;
  int64_t mlp_last_n = 0;
  uint64_t mlp_evals = 0;
  sg::Buf mlp_p, mlp_feat, mlp_tgt, mlp_x, mlp_t, mlp_slots, mlp_choice;
  // buffers of the standalone FrictionSolver entry (kept apart from the scene)
  sg::Buf fs_m, fs_minv, fs_v0, fs_v2;
  sg::Buf fs_I, fs_in;  // sphere entry: world inertia and its inverse; packed per-contact inputs

  // host mirrors of the last step
  int64_t last_nc = 0, last_nbb = 0;
  sg::SolveStats h_stats{};

  // profiling counters (sg_profile_read)
  bool profile = false;
  cudaEvent_t ev_gs0 = nullptr, ev_gs1 = nullptr;
  // Stage timers of the single-scene Ball2D step while profiling: marks 0..8 recorded on the stream
  // (start, after predictor + grid, after pair counting + plane flags, after contact writes and
  // assembly, after colouring, before and after the Gauss-Seidel kernel, after the final velocity,
  // end of step); stage_ms[k] sums the time between mark k and the next recorded mark.
  static constexpr int kStageMarks = 9;
  cudaEvent_t ev_stage[kStageMarks] = {};
  bool stage_timing = false;
  unsigned stage_mask = 0;
  double stage_ms[kStageMarks - 1] = {};
  double gs_ms = 0.0;
  uint64_t gs_launches = 0, contact_sweeps = 0, contact_evals = 0, kernel_launches = 0, steps = 0;
  uint64_t contact_sweeps32 = 0, contact_lifts = 0, body_lifts = 0;
  uint64_t contacts_total = 0;

  // pinned staging
  void* pinned = nullptr;
  size_t pinned_bytes = 0;
};

namespace sg {

// Stage launchers (kernels in ball2d_kernels.cu / solver_kernels.cu / scan.cu).
int scan_exclusive(sg_ctx* ctx, const int* in, int* out, int n);  // out[0..n], out[n] = total
int scan_tile_count(int n);
int scan_exclusive_raw(const int* in, int* out, int n, int* tiles, cudaStream_t stream);

int ball2d_predict_and_bounds(sg_ctx* ctx);
int broadphase_build_grid(sg_ctx* ctx, const double* aabb, int n);
int broadphase_count_pairs(sg_ctx* ctx, const double* aabb, int n, bool ccd);
int broadphase_write_pairs(sg_ctx* ctx, const double* aabb, int n, bool ccd, int* out_a, int* out_b);
int plane_flags(sg_ctx* ctx);
int plane_write(sg_ctx* ctx, int npairs);
int assemble_contacts(sg_ctx* ctx, int nc);
int extract_and_cache(sg_ctx* ctx, int nc);
int ball2d_final_map(sg_ctx* ctx, const double* vin);
int ccd_batch(sg_ctx* ctx, int n, const double* q0a, const double* q1a, const double* ra, const double* q0b,
              const double* q1b, const double* rb, double* coeffs, int* hit, double* t);

// Solver pipeline on a ContactProblem living in ctx buffers.
int solve_contacts(sg_ctx* ctx, const ContactProblem& P, const SolveParams& sp);
// Batched scenes, launches sized to the capacity P.nc, count and scene data on the
// device, no host synchronisation (capturable).
int solve_contacts_batch(sg_ctx* ctx, const ContactProblem& P, const SolveParams& sp, const BatchSolve& X);
int ensure_solver_capacity(sg_ctx* ctx, int nb, int nc);
// Per-contact buffers of a single-scene 2D step for nc contacts (grown with slack).
int ensure_contact_capacity(sg_ctx* ctx, int64_t nc);
// Body -> contact adjacency (ctx->body_off / body_adj, ascending contact order), the
// solve counters cleared, and the contact colouring with its processing permutation
// (ctx->perm, colour offsets in ctx->stats).  Shared by the 2D and 3D solvers.
// nc is the host-side count (or, with nc_dev, the capacity the launches are sized to).
// With warm_color, the colouring starts from those colours (a valid colouring of the contacts that
// carry one) and colours the rest.
int prepare_contact_graph(sg_ctx* ctx, int nb, int nc, const int* ia, const int* ib, const int* nc_dev = nullptr,
                          const int* warm_color = nullptr);

// Cooperative launch through cudaLaunchKernelEx (capturable in a CUDA graph).
inline cudaError_t launch_cooperative(const void* kernel, int grid, int block, void** args, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelExC(&cfg, kernel, args);
}

// Grid size of a cooperative launch: all blocks resident (at most max_per_sm per SM),
// no more than the work needs.
template <typename K>
int coop_grid(sg_ctx* ctx, K kernel, long work, int block, int max_per_sm = 64) {
  int bps = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kernel, block, 0) != cudaSuccess || bps < 1) bps = 1;
  long g = (long)(bps < max_per_sm ? bps : max_per_sm) * ctx->num_sms;
  const long need = (work + block - 1) / block > 1 ? (work + block - 1) / block : 1;
  return (int)(g < need ? g : need);
}

// Batched Ball2D scenes (ball2d_kernels.cu): capacity for `cap` contacts (outside any
// capture) and one step enqueued without host synchronisation.
int batch2d_reserve(sg_ctx* ctx, int cap);
int batch2d_step_enqueue(sg_ctx* ctx);
// One block per scene: Ball2D scenes of at most this many discs (24 B of shared memory each) are
// swept by one block; the per-scene kernels' shared-memory limits are set by scene_blocks_prepare
// (once per context, outside any capture).
constexpr int kSceneBlockMaxBodies = 8192;
int scene_blocks_prepare(int smax);

// Learned warm start (mlp_kernels.cu).
int mlp_param_count();
int mlp_features(sg_ctx* ctx, const ContactProblem& P);
int mlp_predict(sg_ctx* ctx, const ContactProblem& P, double* r_alt);
int mlp_targets(sg_ctx* ctx, const ContactProblem& P);

// RigidBody3D sphere scenes (sphere3d_kernels.cu).
int sphere3d_update_inertia(sg_ctx* ctx, bool construction);
int sphere3d_step(sg_ctx* ctx, sg_step_stats* out);
int sphere3d_batch_setup(sg_ctx* ctx, long flags, long cells);
int sphere3d_batch_step(sg_ctx* ctx, sg_step_stats* out);
// RigidBody2D circles (rigidbody2d_kernels.cu): one step of the geometric or stabilized map.
int rb2d_step(sg_ctx* ctx, sg_step_stats* out);
int sobogus_solve_3d(sg_ctx* ctx, int nb, const double* m, const double* Iw, const double* Iinv, const double* v0,
                     int nc, const int* ia, const int* ib, const double* bases, const double* arm_a,
                     const double* arm_b, const double* CoR, const double* mu, const double* nrel_extra,
                     const double* drel_extra, unsigned max_iters, double tol, unsigned eval_every, double* alpha,
                     double* beta, double* v2, double* f, double* error, unsigned* iterations);

int wait_timeout_selftest(sg_ctx* ctx);

// Records stage mark k of the step being profiled (no-op outside a profiled single-scene step).
inline void stage_mark(sg_ctx* ctx, int k) {
  if (ctx->stage_timing && ctx->ev_stage[k] && cudaEventRecord(ctx->ev_stage[k], ctx->stream) == cudaSuccess)
    ctx->stage_mask |= 1u << k;
}

}  // namespace sg
