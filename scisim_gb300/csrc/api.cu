// api.cu -- the C ABI (include/scisim_gpu.h): contexts, scene upload, the
// per-step pipeline of GeometricImpactFrictionMap::flow, and standalone entry
// points for the FrictionSolver, the broad phase and the CCD narrow phase.
#include "ctx.hpp"

#include <algorithm>
#include <chrono>
#include <limits>
#include <cmath>
#include <cstring>
#include <string>
#include <utility>

namespace sg {

static thread_local std::string g_last_error;
void set_error(const std::string& msg) { g_last_error = msg; }

int grow(Buf& b, size_t bytes) {
  if (bytes <= b.bytes && b.p) return SG_OK;
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.bytes = 0;
  const size_t want = std::max<size_t>(bytes + bytes / 4, 256);
  SG_CUDA_TRY(cudaMalloc(&b.p, want));
  b.bytes = want;
  return SG_OK;
}

void release(Buf& b) {
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.bytes = 0;
}

static constexpr unsigned long long kDefaultSpin = 1ull << 22;  // ~1 s of L2 polls

int ensure_contact_capacity(sg_ctx* ctx, int64_t nc) {
  if (nc <= ctx->ccap && ctx->ia.p) return SG_OK;
  const int64_t cap = std::max<int64_t>(nc + nc / 4 + 64, 1024);
  const size_t c = (size_t)cap;
  if (int r = grow(ctx->ia, sizeof(int) * c)) return r;
  if (int r = grow(ctx->ib, sizeof(int) * c)) return r;
  if (int r = grow(ctx->n, sizeof(double) * 2 * c)) return r;
  if (int r = grow(ctx->c, sizeof(double) * 2 * c)) return r;
  if (int r = grow(ctx->W, sizeof(double) * 3 * c)) return r;
  if (int r = grow(ctx->mu, sizeof(double) * c)) return r;
  if (int r = grow(ctx->r_loc, sizeof(double) * 2 * c)) return r;
  if (int r = grow(ctx->key, sizeof(unsigned long long) * c)) return r;
  if (int r = grow(ctx->ab, sizeof(double) * 2 * c)) return r;
  ctx->ccap = cap;
  return SG_OK;
}

static int upload(sg_ctx* ctx, Buf& b, const void* host, size_t bytes) {
  if (int r = grow(b, bytes)) return r;
  if (bytes) SG_CUDA_TRY(cudaMemcpyAsync(b.p, host, bytes, cudaMemcpyHostToDevice, ctx->stream));
  return SG_OK;
}

// One block per scene when every scene's bodies fit in a block's shared memory (max_bodies): the
// work list takes the scenes largest first (ties in scene order); s_smax = 0 selects the grid-wide
// batched sweeps instead.
static int scene_work_order(sg_ctx* ctx, int S, const int32_t* body_off, int max_bodies) {
  std::vector<int> order(S);
  int smax = 0;
  for (int k = 0; k < S; ++k) {
    order[k] = k;
    smax = std::max(smax, body_off[k + 1] - body_off[k]);
  }
  std::stable_sort(order.begin(), order.end(), [body_off](int x, int y) {
    return body_off[x + 1] - body_off[x] > body_off[y + 1] - body_off[y];
  });
  ctx->s_smax = smax <= max_bodies ? std::max(smax, 1) : 0;
  return upload(ctx, ctx->s_order, order.data(), sizeof(int) * (size_t)S);
}

static int validate_config(const sg_config* c) {
  if (!c) return SG_BAD_INPUT;
  if (c->integrator != SG_SYMPLECTIC_EULER && c->integrator != SG_VERLET && c->integrator != SG_SPLIT_HAM)
    return SG_BAD_INPUT;
  if (c->cache_mode < SG_CACHE_NONE || c->cache_mode > SG_CACHE_NORMAL_AND_FRICTION) return SG_BAD_INPUT;
  if (c->precision != SG_PRECISION_FP64 && c->precision != SG_PRECISION_FP32_REFINE) return SG_BAD_INPUT;
  if (!(c->dt > 0.0) || !(c->tol >= 0.0) || !(c->mu >= 0.0) || !(c->CoR >= 0.0 && c->CoR <= 1.0)) return SG_BAD_INPUT;
  return SG_OK;
}

// One geometric impact-friction step on the device-resident scene.
// Closes the stage timing of a profiled step: the end mark, then each recorded mark's interval to
// the next recorded one into stage_ms.
static int finish_stage_timing(sg_ctx* ctx) {
  if (!ctx->stage_timing) return SG_OK;
  stage_mark(ctx, sg_ctx::kStageMarks - 1);
  ctx->stage_timing = false;
  SG_CUDA_TRY(cudaEventSynchronize(ctx->ev_stage[sg_ctx::kStageMarks - 1]));
  int prev = -1;
  for (int k = 0; k < sg_ctx::kStageMarks; ++k) {
    if (!(ctx->stage_mask & (1u << k))) continue;
    if (prev >= 0) {
      float ms = 0.f;
      SG_CUDA_TRY(cudaEventElapsedTime(&ms, ctx->ev_stage[prev], ctx->ev_stage[k]));
      ctx->stage_ms[prev] += ms;
    }
    prev = k;
  }
  return SG_OK;
}

static int step_once(sg_ctx* ctx, sg_step_stats* out) {
  const int nb = ctx->nb;
  cudaStream_t s = ctx->stream;
  sg_step_stats st{};
  if (ctx->staggering == SG_STAGGER_SYMPLECTIC_EULER && ctx->cfg.CoR != 0.0) {
    set_error("the symplectic Euler staggering needs CoR = 0");
    return SG_BAD_INPUT;
  }
  if (ctx->staggering == SG_STAGGER_STABILIZED && ctx->cfg.cache_mode != SG_CACHE_NONE) {
    set_error("the stabilized staggering keeps no impulse cache");
    return SG_BAD_INPUT;
  }
  if (nb == 0) {
    if (out) *out = st;
    return SG_OK;
  }
  ctx->stage_timing = ctx->profile && ctx->ev_stage[0];
  ctx->stage_mask = 0;
  stage_mark(ctx, 0);
  // Predictor + swept AABBs (GeometricImpactFrictionMap.cpp:279, Ball2DSim.cpp:566-572).
  if (int r = ball2d_predict_and_bounds(ctx)) return r;
  const double* aabb = ctx->aabb.as<double>();
  if (int r = broadphase_build_grid(ctx, aabb, nb)) return r;
  stage_mark(ctx, 1);
  if (int r = broadphase_count_pairs(ctx, aabb, nb, true)) return r;
  if (int r = plane_flags(ctx)) return r;
  stage_mark(ctx, 2);
  int totals[2] = {0, 0};
  SG_CUDA_TRY(cudaMemcpyAsync(&totals[0], ctx->pair_off.as<int>() + nb, sizeof(int), cudaMemcpyDeviceToHost, s));
  SG_CUDA_TRY(cudaMemcpyAsync(&totals[1], ctx->plane_off.as<int>() + (long)nb * ctx->np, sizeof(int),
                              cudaMemcpyDeviceToHost, s));
  SG_CUDA_TRY(cudaStreamSynchronize(s));
  const int npairs = totals[0], nplanes = totals[1];
  const int nc = npairs + nplanes;
  // predictor 1, grid 8 (bounds init/reduce/setup, count, 3-kernel scan, scatter),
  // pair count + scan 4, plane flags + scan 4
  ctx->kernel_launches += 1 + 8 + 4 + (ctx->np > 0 ? 4 : 0);
  ctx->steps += 1;
  ctx->contacts_total += (uint64_t)nc;
  st.n_contacts = nc;
  st.n_ball_ball = npairs;
  st.n_ball_plane = nplanes;
  ctx->last_nc = nc;
  ctx->last_nbb = npairs;
  if (nc == 0) {
    ctx->mlp_last_n = 0;
    // No active constraints: keep the predictor and clear the cache (:286-298).
    std::swap(ctx->q, ctx->q1);
    std::swap(ctx->v, ctx->v1);
    ctx->prev_n = 0;
    ctx->prev_rows = false;
    ctx->prev_color_valid = false;
    st.succeeded = 1;
    if (int r = finish_stage_timing(ctx)) return r;
    if (out) *out = st;
    return SG_OK;
  }
  if (int r = ensure_contact_capacity(ctx, nc)) return r;
  if (int r = broadphase_write_pairs(ctx, aabb, nb, true, ctx->ia.as<int>(), ctx->ib.as<int>())) return r;
  if (int r = plane_write(ctx, npairs)) return r;
  // Colours carried over from the cached step (assemble_contacts writes them beside the warm start).
  const bool warm_colors = ctx->prev_color_valid && ctx->prev_n > 0 && ctx->n_scenes == 0 && !ctx->rb2d &&
                           ctx->cfg.cache_mode != SG_CACHE_NONE;
  if (int r = assemble_contacts(ctx, nc)) return r;
  stage_mark(ctx, 3);
  if (int r = grow(ctx->v2, sizeof(double) * 2 * (size_t)nb)) return r;
  ContactProblem P;
  P.nb = nb;
  P.nc = nc;
  P.minv = ctx->minv.as<double>();
  P.m = ctx->m.as<double>();
  // The stabilized map solves from the unconstrained step's velocity (StabilizedImpactFrictionMap.cpp:127).
  P.v0 = ctx->staggering == SG_STAGGER_STABILIZED ? ctx->v1.as<double>() : ctx->v.as<double>();
  P.ia = ctx->ia.as<int>();
  P.ib = ctx->ib.as<int>();
  P.n = ctx->n.as<double>();
  P.c = ctx->c.as<double>();
  P.W = ctx->W.as<double>();
  P.mu = ctx->mu.as<double>();
  P.r = ctx->r_loc.as<double>();
  P.v2 = ctx->v2.as<double>();
  P.warm_color = warm_colors ? ctx->init_color.as<int>() : nullptr;
  SolveParams sp{ctx->cfg.tol, ctx->cfg.max_iters, ctx->cfg.eval_every, ctx->cfg.precision, true};
  const int sr = solve_contacts(ctx, P, sp);
  if (sr != SG_OK && sr != SG_NOT_CONVERGED) return sr;
  st.iterations = ctx->h_stats.iterations;
  st.succeeded = ctx->h_stats.converged;
  st.error = ctx->h_stats.error;
  st.n_colors = (uint32_t)ctx->h_stats.n_colors;
  // Impulses and cache (Sobogus.cpp:312-347, GeometricImpactFrictionMap.cpp:428).
  if (int r = extract_and_cache(ctx, nc)) return r;
  if (ctx->cfg.cache_mode != SG_CACHE_NONE) {
    std::swap(ctx->key, ctx->prev_key);
    std::swap(ctx->ab, ctx->prev_ab);
    ctx->prev_n = nc;
    // This step's rows (pair offsets, plane flags and their scan) locate next step's cache entries.
    std::swap(ctx->pair_off, ctx->prev_pair_off);
    std::swap(ctx->plane_off, ctx->prev_plane_off);
    std::swap(ctx->plane_flag, ctx->prev_plane_flag);
    ctx->prev_npairs = npairs;
    ctx->prev_rows = true;
    // This step's colouring seeds the next one's.
    if (int r = grow(ctx->prev_color, sizeof(int) * (size_t)nc)) return r;
    SG_CUDA_TRY(cudaMemcpyAsync(ctx->prev_color.p, ctx->color.p, sizeof(int) * (size_t)nc, cudaMemcpyDeviceToDevice, s));
    ctx->prev_color_valid = true;
    // keep ccap consistent with the smaller of the swapped buffers
    const int64_t kcap = (int64_t)std::min(ctx->key.bytes / sizeof(unsigned long long), ctx->ab.bytes / (2 * sizeof(double)));
    ctx->ccap = std::min<int64_t>(ctx->ccap, kcap);
  } else {
    ctx->prev_n = 0;
    ctx->prev_rows = false;
    ctx->prev_color_valid = false;
  }
  // Final map with the post-impact velocity (:441).
  if (int r = ball2d_final_map(ctx, ctx->v2.as<double>())) return r;
  ctx->kernel_launches += 2 + (ctx->np > 0 ? 1 : 0) + 1 + 1;  // write pairs, assemble, plane write, extract, final map
  std::swap(ctx->q, ctx->q1);
  std::swap(ctx->v, ctx->v1);
  if (int r = finish_stage_timing(ctx)) return r;
  if (out) *out = st;
  return sr;
}

}  // namespace sg

using namespace sg;

extern "C" {

const char* sg_last_error_string(void) { return g_last_error.c_str(); }

int sg_ctx_create(const sg_config* cfg, sg_ctx** out) {
  if (!out) return SG_BAD_INPUT;
  *out = nullptr;
  if (validate_config(cfg) != SG_OK) {
    set_error("invalid sg_config");
    return SG_BAD_INPUT;
  }
  int ndev = 0;
  SG_CUDA_TRY(cudaGetDeviceCount(&ndev));
  if (cfg->device < 0 || cfg->device >= ndev) {
    set_error("invalid CUDA device ordinal");
    return SG_BAD_INPUT;
  }
  SG_CUDA_TRY(cudaSetDevice(cfg->device));
  auto* ctx = new sg_ctx;
  ctx->cfg = *cfg;
  ctx->device = cfg->device;
  ctx->spin_limit = kDefaultSpin;
  cudaError_t e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, cfg->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    set_error(std::string("context setup failed: ") + cudaGetErrorString(e));
    delete ctx;
    return SG_CUDA_ERROR;
  }
  *out = ctx;
  return SG_OK;
}

void sg_ctx_destroy(sg_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  Buf* bufs3[] = {&ctx->I0, &ctx->Iw, &ctx->Iinv, &ctx->E3, &ctx->Aa3, &ctx->Ab3, &ctx->c3, &ctx->W3,
                  &ctx->r3, &ctx->r3a, &ctx->r3b, &ctx->ab3, &ctx->vrun3, &ctx->pk_ab, &ctx->pk_n, &ctx->pk_c,
                  &ctx->pk_w, &ctx->pk_r, &ctx->v32, &ctx->minv32, &ctx->pk3, &ctx->Iinv32, &ctx->pt_setup,
                  &ctx->pt_patch, &ctx->pt_lidx, &ctx->pt_body, &ctx->pt_cnt, &ctx->pt_start, &ctx->pt_fill,
                  &ctx->pt_key, &ctx->pt_kcnt, &ctx->pt_kstart, &ctx->pt_kfill, &ctx->pt_order, &ctx->pt_max,
                  &ctx->pt_bcolor, &ctx->pt_rem, &ctx->pt_qpatch, &ctx->pt_band, &ctx->pt_lidxq,
                  &ctx->pt_qbody, &ctx->pt_bcnt, &ctx->pt_nfill, &ctx->pt_qcnt, &ctx->pt_qstart, &ctx->pt_qfill,
                  &ctx->pt_cflag, &ctx->pt_cpos, &ctx->pt_cbody, &ctx->pt_hist, &ctx->pt_pref,
                  &ctx->pt_cuts, &ctx->pt_maps, &ctx->ff_n, &ctx->ff_c, &ctx->ff_m, &ctx->ff_r, &ctx->ff_v,
                  &ctx->ff_minv};
  for (Buf* b : bufs3) release(*b);
  Buf* bufsm[] = {&ctx->mlp_p, &ctx->mlp_feat, &ctx->mlp_tgt, &ctx->mlp_x, &ctx->mlp_t, &ctx->mlp_slots,
                  &ctx->mlp_choice};
  for (Buf* b : bufsm) release(*b);
  Buf* bufsb[] = {&ctx->sb_off,  &ctx->sp_off,   &ctx->sf_off,      &ctx->scene_of, &ctx->s_mu,    &ctx->s_CoR,
                  &ctx->s_grid,  &ctx->s_cells,  &ctx->s_cell_off,  &ctx->s_nc,     &ctx->s_npairs, &ctx->sc_off,
                  &ctx->prev_sc_off, &ctx->cscene, &ctx->b_ctl,     &ctx->b_sums,   &ctx->s_err,   &ctx->s_best,
                  &ctx->s_bestbuf, &ctx->s_done, &ctx->s_iters,     &ctx->snap_q,   &ctx->snap_v,  &ctx->snap_key,
                  &ctx->snap_ab, &ctx->snap_off, &ctx->s_mode, &ctx->s_since, &ctx->s_exc, &ctx->s_gmax,
                  &ctx->b_work, &ctx->pk_scene, &ctx->s_kcnt, &ctx->s_kstart, &ctx->s_kfill, &ctx->s_sperm,
                  &ctx->s_order, &ctx->s_next};
  for (Buf* b : bufsb) release(*b);
  if (ctx->graph) cudaGraphExecDestroy(ctx->graph);
  Buf* bufs[] = {&ctx->q, &ctx->v, &ctx->r, &ctx->m, &ctx->minv, &ctx->q1, &ctx->v1, &ctx->v2, &ctx->plane_x,
                 &ctx->plane_n, &ctx->plane_t, &ctx->aabb, &ctx->cell_of, &ctx->cell_count, &ctx->cell_start,
                 &ctx->cell_fill, &ctx->sorted, &ctx->pair_cnt, &ctx->pair_off, &ctx->grid, &ctx->plane_flag,
                 &ctx->plane_off, &ctx->scan_tmp, &ctx->ia, &ctx->ib, &ctx->n, &ctx->c, &ctx->W, &ctx->mu,
                 &ctx->r_loc, &ctx->r_cand, &ctx->r_best, &ctx->key, &ctx->ab, &ctx->prev_key, &ctx->prev_ab,
                 &ctx->color, &ctx->perm, &ctx->body_cnt, &ctx->body_off, &ctx->body_fill, &ctx->body_adj,
                 &ctx->v_run, &ctx->stats, &ctx->barrier, &ctx->fs_m, &ctx->fs_minv, &ctx->fs_v0, &ctx->fs_v2,
                 &ctx->fs_I, &ctx->fs_in, &ctx->c6, &ctx->prev_c6, &ctx->pair_slots, &ctx->aabb32, &ctx->aabb32s, &ctx->prev_pair_off, &ctx->prev_plane_off,
                 &ctx->prev_plane_flag, &ctx->prev_color, &ctx->init_color, &ctx->vdelta, &ctx->rb_I, &ctx->rb_Iinv,
                 &ctx->pos0, &ctx->pos1, &ctx->rb_ct, &ctx->rb_vrun};
  for (Buf* b : bufs) release(*b);
  if (ctx->pinned) cudaFreeHost(ctx->pinned);
  if (ctx->ev_gs0) cudaEventDestroy(ctx->ev_gs0);
  if (ctx->ev_gs1) cudaEventDestroy(ctx->ev_gs1);
  for (cudaEvent_t e : ctx->ev_stage)
    if (e) cudaEventDestroy(e);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
}

int sg_ctx_reconfigure(sg_ctx* ctx, const sg_config* cfg) {
  if (!ctx || validate_config(cfg) != SG_OK || cfg->device != ctx->device) {
    set_error("sg_ctx_reconfigure: invalid sg_config");
    return SG_BAD_INPUT;
  }
  ctx->cfg = *cfg;
  if (ctx->graph) {
    cudaGraphExecDestroy(ctx->graph);  // kernel arguments carry the old settings
    ctx->graph = nullptr;
  }
  return SG_OK;
}

int sg_ball2d_upload(sg_ctx* ctx, int32_t nb, const double* q, const double* v, const double* r, const double* m,
                     int32_t np, const double* plane_x, const double* plane_n) {
  if (!ctx || nb < 0 || np < 0 || (nb > 0 && (!q || !v || !r || !m)) || (np > 0 && (!plane_x || !plane_n))) {
    set_error("sg_ball2d_upload: invalid arguments");
    return SG_BAD_INPUT;
  }
  for (int i = 0; i < nb; ++i)
    if (!(r[i] > 0.0) || !(m[i] > 0.0)) {
      set_error("sg_ball2d_upload: radii and masses must be positive");
      return SG_BAD_INPUT;
    }
  SG_CUDA_TRY(cudaSetDevice(ctx->device));
  ctx->dim = 2;
  ctx->rb2d = false;
  ctx->n_scenes = 0;
  if (ctx->graph) {
    cudaGraphExecDestroy(ctx->graph);
    ctx->graph = nullptr;
  }
  ctx->nb = nb;
  ctx->np = np;
  const size_t b2 = sizeof(double) * 2 * (size_t)std::max(nb, 1), b1 = sizeof(double) * (size_t)std::max(nb, 1);
  std::vector<double> minv(nb);
  for (int i = 0; i < nb; ++i) minv[i] = 1.0 / m[i];  // Ball2DState createMinv (Ball2DState.cpp:55-67)
  std::vector<double> pn(2 * (size_t)np), pt(2 * (size_t)np);
  for (int p = 0; p < np; ++p) {
    // StaticPlane: n = normalized(n), t = (-n_y, n_x) (StaticPlane.cpp:10-19)
    double nx = plane_n[2 * p], ny = plane_n[2 * p + 1];
    const double z = nx * nx + ny * ny;
    if (!(z > 0.0)) {
      set_error("sg_ball2d_upload: zero plane normal");
      return SG_BAD_INPUT;
    }
    const double sq = std::sqrt(z);
    nx = nx / sq;
    ny = ny / sq;
    pn[2 * p] = nx;
    pn[2 * p + 1] = ny;
    pt[2 * p] = -ny;
    pt[2 * p + 1] = nx;
  }
  if (int e = upload(ctx, ctx->q, q, sizeof(double) * 2 * nb)) return e;
  if (int e = upload(ctx, ctx->v, v, sizeof(double) * 2 * nb)) return e;
  if (int e = upload(ctx, ctx->r, r, sizeof(double) * nb)) return e;
  if (int e = upload(ctx, ctx->m, m, sizeof(double) * nb)) return e;
  if (int e = upload(ctx, ctx->minv, minv.data(), sizeof(double) * nb)) return e;
  if (int e = grow(ctx->q1, b2)) return e;
  if (int e = grow(ctx->v1, b2)) return e;
  if (int e = grow(ctx->v2, b2)) return e;
  if (int e = grow(ctx->aabb, 2 * b2)) return e;
  (void)b1;
  if (int e = upload(ctx, ctx->plane_x, plane_x, sizeof(double) * 2 * np)) return e;
  if (int e = upload(ctx, ctx->plane_n, pn.data(), sizeof(double) * 2 * np)) return e;
  if (int e = upload(ctx, ctx->plane_t, pt.data(), sizeof(double) * 2 * np)) return e;
  if (int e = grow(ctx->plane_x, 16)) return e;
  if (int e = grow(ctx->plane_n, 16)) return e;
  if (int e = grow(ctx->plane_t, 16)) return e;
  ctx->prev_n = 0;
  ctx->prev_rows = false;
  ctx->prev_color_valid = false;
  ctx->last_nc = 0;
  SG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SG_OK;
}

int sg_rigidbody2d_upload(sg_ctx* ctx, int32_t nb, const double* q, const double* v, const double* r, const double* m,
                          const double* I, int32_t np, const double* plane_x, const double* plane_n) {
  if (!ctx || nb < 0 || np < 0 || (nb > 0 && (!q || !v || !r || !m || !I)) || (np > 0 && (!plane_x || !plane_n))) {
    set_error("sg_rigidbody2d_upload: invalid arguments");
    return SG_BAD_INPUT;
  }
  for (int i = 0; i < nb; ++i)
    if (!(r[i] > 0.0) || !(m[i] > 0.0) || !(I[i] > 0.0)) {
      set_error("sg_rigidbody2d_upload: radii, masses and moments of inertia must be positive");
      return SG_BAD_INPUT;
    }
  if (ctx->cfg.integrator == SG_SPLIT_HAM) {
    set_error("sg_rigidbody2d_upload: RigidBody2D scenes step with SG_SYMPLECTIC_EULER or SG_VERLET");
    return SG_BAD_INPUT;
  }
  SG_CUDA_TRY(cudaSetDevice(ctx->device));
  ctx->dim = 2;
  ctx->rb2d = true;
  ctx->n_scenes = 0;
  if (ctx->graph) {
    cudaGraphExecDestroy(ctx->graph);
    ctx->graph = nullptr;
  }
  ctx->nb = nb;
  ctx->np = np;
  const size_t n1 = (size_t)std::max(nb, 1);
  // RigidBody2DState's Minv: 1 / m (x, y), 1 / I (theta).
  std::vector<double> minv(nb), Iinv(nb);
  for (int i = 0; i < nb; ++i) {
    minv[i] = 1.0 / m[i];
    Iinv[i] = 1.0 / I[i];
  }
  std::vector<double> pn(2 * (size_t)np), pt(2 * (size_t)np);
  for (int p = 0; p < np; ++p) {
    // The scene parser stores n.normalized() (rigidbody2dutils/RigidBody2DSceneParser.cpp:271-277); t = (-n_y, n_x).
    double nx = plane_n[2 * p], ny = plane_n[2 * p + 1];
    const double z = nx * nx + ny * ny;
    if (!(z > 0.0)) {
      set_error("sg_rigidbody2d_upload: zero plane normal");
      return SG_BAD_INPUT;
    }
    const double sq = std::sqrt(z);
    nx = nx / sq;
    ny = ny / sq;
    pn[2 * p] = nx;
    pn[2 * p + 1] = ny;
    pt[2 * p] = -ny;
    pt[2 * p + 1] = nx;
  }
  if (int e = upload(ctx, ctx->q, q, sizeof(double) * 3 * nb)) return e;
  if (int e = upload(ctx, ctx->v, v, sizeof(double) * 3 * nb)) return e;
  if (int e = upload(ctx, ctx->r, r, sizeof(double) * nb)) return e;
  if (int e = upload(ctx, ctx->m, m, sizeof(double) * nb)) return e;
  if (int e = upload(ctx, ctx->minv, minv.data(), sizeof(double) * nb)) return e;
  if (int e = upload(ctx, ctx->rb_I, I, sizeof(double) * nb)) return e;
  if (int e = upload(ctx, ctx->rb_Iinv, Iinv.data(), sizeof(double) * nb)) return e;
  if (int e = grow(ctx->q1, sizeof(double) * 3 * n1)) return e;
  if (int e = grow(ctx->v1, sizeof(double) * 3 * n1)) return e;
  if (int e = grow(ctx->v2, sizeof(double) * 3 * n1)) return e;
  if (int e = grow(ctx->pos0, sizeof(double) * 2 * n1)) return e;
  if (int e = grow(ctx->pos1, sizeof(double) * 2 * n1)) return e;
  if (int e = grow(ctx->aabb, sizeof(double) * 4 * n1)) return e;
  if (int e = upload(ctx, ctx->plane_x, plane_x, sizeof(double) * 2 * np)) return e;
  if (int e = upload(ctx, ctx->plane_n, pn.data(), sizeof(double) * 2 * np)) return e;
  if (int e = upload(ctx, ctx->plane_t, pt.data(), sizeof(double) * 2 * np)) return e;
  if (int e = grow(ctx->plane_x, 16)) return e;
  if (int e = grow(ctx->plane_n, 16)) return e;
  if (int e = grow(ctx->plane_t, 16)) return e;
  ctx->prev_n = 0;
  ctx->prev_rows = false;
  ctx->prev_color_valid = false;
  ctx->last_nc = 0;
  SG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SG_OK;
}

int64_t sg_rigidbody2d_last_contacts(sg_ctx* ctx, int64_t cap, int32_t* ia, int32_t* ib, double* n, double* ta,
                                     double* tb, double* alpha, double* beta) {
  if (!ctx) return SG_BAD_INPUT;
  if (!ctx->rb2d) {
    set_error("sg_rigidbody2d_last_contacts: the context holds no RigidBody2D scene");
    return INT64_MIN;
  }
  const int64_t nc = sg_last_contacts(ctx, cap, ia, ib, n, alpha, beta);
  if (nc <= 0 || (!ta && !tb)) return nc;
  std::vector<double> ct(2 * (size_t)nc);
  if (cudaMemcpyAsync(ct.data(), ctx->rb_ct.p, sizeof(double) * 2 * (size_t)nc, cudaMemcpyDeviceToHost, ctx->stream) !=
          cudaSuccess ||
      cudaStreamSynchronize(ctx->stream) != cudaSuccess)
    return -1;
  for (int64_t k = 0; k < nc; ++k) {
    if (ta) ta[k] = ct[2 * k];
    if (tb) tb[k] = ct[2 * k + 1];
  }
  return nc;
}

static int sphere3d_upload_impl(sg_ctx* ctx, int32_t nb, const double* q, const double* v, const double* r, const double* m,
                         const double* I0, int32_t np, const double* plane_x, const double* plane_n) {
  if (!ctx || nb < 0 || np < 0 || (nb > 0 && (!q || !v || !r || !m || !I0)) || (np > 0 && (!plane_x || !plane_n))) {
    set_error("sg_sphere3d_upload: invalid arguments");
    return SG_BAD_INPUT;
  }
  for (int i = 0; i < nb; ++i)
    if (!(r[i] > 0.0) || !(m[i] > 0.0) || !(I0[3 * i] > 0.0) || !(I0[3 * i + 1] > 0.0) || !(I0[3 * i + 2] > 0.0)) {
      set_error("sg_sphere3d_upload: radii, masses and inertias must be positive");
      return SG_BAD_INPUT;
    }
  std::vector<double> pn(3 * (size_t)np);
  for (int p = 0; p < np; ++p) {
    // StaticPlane: n = n.normalized() (rigidbody3d/StaticGeometry/StaticPlane.cpp:10-15)
    const double* n = plane_n + 3 * p;
    const double z = (n[0] * n[0] + n[1] * n[1]) + n[2] * n[2];
    if (!(z > 0.0)) {
      set_error("sg_sphere3d_upload: zero plane normal");
      return SG_BAD_INPUT;
    }
    const double sq = std::sqrt(z);
    for (int j = 0; j < 3; ++j) pn[3 * p + j] = n[j] / sq;
  }
  SG_CUDA_TRY(cudaSetDevice(ctx->device));
  ctx->dim = 3;
  ctx->rb2d = false;
  ctx->n_scenes = 0;
  ctx->nb = nb;
  ctx->np = np;
  const size_t nbs = (size_t)std::max(nb, 1);
  std::vector<double> minv(nb);
  for (int i = 0; i < nb; ++i) minv[i] = 1.0 / m[i];  // formWorldSpaceInverseMassMatrix (RigidBody3DState.cpp:208-214)
  if (int e = upload(ctx, ctx->q, q, sizeof(double) * 12 * nb)) return e;
  if (int e = upload(ctx, ctx->v, v, sizeof(double) * 6 * nb)) return e;
  if (int e = upload(ctx, ctx->r, r, sizeof(double) * nb)) return e;
  if (int e = upload(ctx, ctx->m, m, sizeof(double) * nb)) return e;
  if (int e = upload(ctx, ctx->minv, minv.data(), sizeof(double) * nb)) return e;
  if (int e = upload(ctx, ctx->I0, I0, sizeof(double) * 3 * nb)) return e;
  if (int e = grow(ctx->Iw, sizeof(double) * 9 * nbs)) return e;
  if (int e = grow(ctx->Iinv, sizeof(double) * 9 * nbs)) return e;
  if (int e = grow(ctx->q1, sizeof(double) * 12 * nbs)) return e;
  if (int e = grow(ctx->v1, sizeof(double) * 6 * nbs)) return e;
  if (int e = grow(ctx->v2, sizeof(double) * 6 * nbs)) return e;
  if (int e = grow(ctx->aabb, sizeof(double) * 6 * nbs)) return e;
  if (int e = upload(ctx, ctx->plane_x, plane_x, sizeof(double) * 3 * np)) return e;
  if (int e = upload(ctx, ctx->plane_n, pn.data(), sizeof(double) * 3 * np)) return e;
  if (int e = grow(ctx->plane_x, 16)) return e;
  if (int e = grow(ctx->plane_n, 16)) return e;
  // World inertia at construction (RigidBody3DState.cpp:140-230).
  if (int e = sphere3d_update_inertia(ctx, true)) return e;
  ctx->prev_n = 0;
  ctx->prev_rows = false;
  ctx->prev_color_valid = false;
  ctx->last_nc = 0;
  SG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SG_OK;
}

// ---------------------------------------------------------------------------
// Batched Ball2D scenes.
static constexpr int kGraphSteps = 8;  // steps per captured graph (even: pointer swaps cancel)

static int batch_upload(sg_ctx* ctx, int32_t S, const int32_t* body_off, const double* q, const double* v,
                        const double* r, const double* m, const int32_t* plane_off, const double* plane_x,
                        const double* plane_n, const double* mu, const double* CoR) {
  if (!ctx || S < 1 || !body_off || !plane_off || !mu || !CoR || body_off[0] != 0 || plane_off[0] != 0) {
    set_error("sg_batch2d_upload: invalid arguments");
    return SG_BAD_INPUT;
  }
  std::vector<int> sf(S + 1, 0), scene_of;
  long cells = 0;
  for (int s = 0; s < S; ++s) {
    const int ns = body_off[s + 1] - body_off[s], np = plane_off[s + 1] - plane_off[s];
    if (ns < 0 || np < 0 || !(mu[s] >= 0.0) || !(CoR[s] >= 0.0 && CoR[s] <= 1.0)) {
      set_error("sg_batch2d_upload: offsets must not decrease; mu >= 0, 0 <= CoR <= 1 per scene");
      return SG_BAD_INPUT;
    }
    const long f = (long)sf[s] + (long)ns * np;
    cells += 4L * ns + 64;
    if (f > (1L << 30) || cells > (1L << 30)) {
      set_error("sg_batch2d_upload: batch too large");
      return SG_CAPACITY;
    }
    sf[s + 1] = (int)f;
    scene_of.insert(scene_of.end(), (size_t)ns, s);
  }
  const int N = body_off[S], NP = plane_off[S];
  if (int e = sg_ball2d_upload(ctx, N, q, v, r, m, NP, plane_x, plane_n)) return e;
  ctx->n_scenes = S;
  ctx->bcells = cells;
  ctx->bflags = sf[S];
  const size_t s1 = sizeof(int) * (size_t)(S + 1);
  if (int e = upload(ctx, ctx->sb_off, body_off, s1)) return e;
  if (int e = upload(ctx, ctx->sp_off, plane_off, s1)) return e;
  if (int e = upload(ctx, ctx->sf_off, sf.data(), s1)) return e;
  if (int e = upload(ctx, ctx->scene_of, scene_of.data(), sizeof(int) * (size_t)N)) return e;
  if (int e = upload(ctx, ctx->s_mu, mu, sizeof(double) * (size_t)S)) return e;
  if (int e = upload(ctx, ctx->s_CoR, CoR, sizeof(double) * (size_t)S)) return e;
  const size_t nbs = (size_t)std::max(N, 1);
  Buf* ints_s1[] = {&ctx->s_cells, &ctx->s_cell_off, &ctx->s_nc, &ctx->s_npairs, &ctx->sc_off, &ctx->prev_sc_off,
                    &ctx->snap_off, &ctx->s_bestbuf, &ctx->s_done, &ctx->s_iters};
  for (Buf* b : ints_s1)
    if (int e = grow(*b, s1)) return e;
  if (int e = grow(ctx->s_grid, 48 * (size_t)S)) return e;
  if (int e = grow(ctx->s_best, sizeof(double) * (size_t)S)) return e;
  if (int e = grow(ctx->s_err, sizeof(unsigned long long) * 3 * (size_t)S)) return e;
  if (int e = grow(ctx->b_ctl, 4 * sizeof(int))) return e;
  if (int e = grow(ctx->b_sums, 4 * sizeof(unsigned long long))) return e;
  if (int e = grow(ctx->cell_count, sizeof(int) * (size_t)(cells + 1))) return e;
  if (int e = grow(ctx->cell_start, sizeof(int) * (size_t)(cells + 1))) return e;
  if (int e = grow(ctx->cell_fill, sizeof(int) * (size_t)(cells + 1))) return e;
  if (int e = grow(ctx->cell_of, sizeof(int) * nbs)) return e;
  if (int e = grow(ctx->sorted, sizeof(int) * nbs)) return e;
  if (int e = grow(ctx->pair_cnt, sizeof(int) * (nbs + 1))) return e;
  if (int e = grow(ctx->pair_off, sizeof(int) * (nbs + 1))) return e;
  if (int e = grow(ctx->plane_flag, sizeof(int) * (size_t)(sf[S] + 1))) return e;
  if (int e = grow(ctx->plane_off, sizeof(int) * (size_t)(sf[S] + 1))) return e;
  if (int e = grow(ctx->snap_q, sizeof(double) * 2 * nbs)) return e;
  if (int e = grow(ctx->snap_v, sizeof(double) * 2 * nbs)) return e;
  SG_CUDA_TRY(cudaMemsetAsync(ctx->prev_sc_off.p, 0, s1, ctx->stream));
  SG_CUDA_TRY(cudaMemsetAsync(ctx->sc_off.p, 0, s1, ctx->stream));
  SG_CUDA_TRY(cudaMemsetAsync(ctx->b_ctl.p, 0, 4 * sizeof(int), ctx->stream));
  if (int e = scene_work_order(ctx, S, body_off, kSceneBlockMaxBodies)) return e;
  if (int e = batch2d_reserve(ctx, std::max(3 * N + 1024, ctx->bcap))) return e;
  SG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SG_OK;
}

// State a chunk of steps starts from (positions, velocities, impulse cache, counters).
static int batch_snapshot(sg_ctx* ctx, bool restore) {
  cudaStream_t s = ctx->stream;
  const size_t b2 = sizeof(double) * 2 * (size_t)ctx->nb;
  const size_t s1 = sizeof(int) * (size_t)(ctx->n_scenes + 1);
  const size_t kb = sizeof(unsigned long long) * (size_t)ctx->bcap, ab = sizeof(double) * 2 * (size_t)ctx->bcap;
  auto cp = [&](Buf& live, Buf& snap, size_t bytes) -> cudaError_t {
    if (!bytes) return cudaSuccess;
    return restore ? cudaMemcpyAsync(live.p, snap.p, bytes, cudaMemcpyDeviceToDevice, s)
                   : cudaMemcpyAsync(snap.p, live.p, bytes, cudaMemcpyDeviceToDevice, s);
  };
  SG_CUDA_TRY(cp(ctx->q, ctx->snap_q, b2));
  SG_CUDA_TRY(cp(ctx->v, ctx->snap_v, b2));
  if (ctx->cfg.cache_mode != SG_CACHE_NONE) {
    SG_CUDA_TRY(cp(ctx->prev_key, ctx->snap_key, kb));
    SG_CUDA_TRY(cp(ctx->prev_ab, ctx->snap_ab, ab));
    SG_CUDA_TRY(cp(ctx->prev_sc_off, ctx->snap_off, s1));
  }
  return SG_OK;
}

static int batch_build_graph(sg_ctx* ctx) {
  cudaStream_t s = ctx->stream;
  const uint64_t l0 = ctx->kernel_launches, st0 = ctx->steps;
  Buf saved[8] = {ctx->q, ctx->q1, ctx->v, ctx->v1, ctx->key, ctx->prev_key, ctx->ab, ctx->prev_ab};
  Buf saved_off[2] = {ctx->sc_off, ctx->prev_sc_off};
  SG_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
  int rc = SG_OK;
  for (int k = 0; k < kGraphSteps && rc == SG_OK; ++k) rc = batch2d_step_enqueue(ctx);
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(s, &g);
  ctx->q = saved[0], ctx->q1 = saved[1], ctx->v = saved[2], ctx->v1 = saved[3];
  ctx->key = saved[4], ctx->prev_key = saved[5], ctx->ab = saved[6], ctx->prev_ab = saved[7];
  ctx->sc_off = saved_off[0], ctx->prev_sc_off = saved_off[1];
  ctx->graph_launches = ctx->kernel_launches - l0;
  ctx->kernel_launches = l0;
  ctx->steps = st0;
  if (rc != SG_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  SG_CUDA_TRY(ce);
  const cudaError_t ie = cudaGraphInstantiate(&ctx->graph, g, 0);
  cudaGraphDestroy(g);
  SG_CUDA_TRY(ie);
  return SG_OK;
}

static int batch_step(sg_ctx* ctx, uint32_t n_steps, sg_step_stats* out, int64_t* total) {
  cudaStream_t s = ctx->stream;
  const int S = ctx->n_scenes;
  SG_CUDA_TRY(cudaMemsetAsync(ctx->b_sums.p, 0, 4 * sizeof(unsigned long long), s));
  SG_CUDA_TRY(cudaMemsetAsync(ctx->b_ctl.as<int>() + 1, 0, sizeof(int), s));
  SG_CUDA_TRY(cudaMemsetAsync(ctx->b_work.p, 0, 5 * sizeof(unsigned long long), s));
  uint32_t done = 0;
  unsigned long long sums_before[2] = {0, 0};
  int retries = 0;
  while (done < n_steps) {
    const uint32_t chunk = std::min<uint32_t>(kGraphSteps, n_steps - done);
    if (int e = batch_snapshot(ctx, false)) return e;
    SG_CUDA_TRY(cudaMemcpyAsync(sums_before, ctx->b_sums.p, sizeof sums_before, cudaMemcpyDeviceToHost, s));
    if (chunk == (uint32_t)kGraphSteps) {
      if (!ctx->graph)
        if (int e = batch_build_graph(ctx)) return e;
      SG_CUDA_TRY(cudaGraphLaunch(ctx->graph, s));
      ctx->kernel_launches += ctx->graph_launches;
      ctx->steps += chunk;
    } else {
      for (uint32_t k = 0; k < chunk; ++k)
        if (int e = batch2d_step_enqueue(ctx)) return e;
    }
    int overflow = 0;
    SG_CUDA_TRY(cudaMemcpyAsync(&overflow, ctx->b_ctl.as<int>() + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
    SG_CUDA_TRY(cudaStreamSynchronize(s));
    if (overflow > 0) {
      // Restore the chunk's starting state, grow the contact capacity and step again.
      if (++retries > 8) {
        set_error("batched step: contact capacity kept overflowing");
        return SG_CAPACITY;
      }
      if (int e = batch_snapshot(ctx, true)) return e;
      SG_CUDA_TRY(cudaMemcpyAsync(ctx->b_sums.p, sums_before, sizeof sums_before, cudaMemcpyHostToDevice, s));
      SG_CUDA_TRY(cudaMemsetAsync(ctx->b_ctl.as<int>() + 1, 0, sizeof(int), s));
      if (ctx->graph) {
        cudaGraphExecDestroy(ctx->graph);
        ctx->graph = nullptr;
      }
      ctx->steps -= chunk;
      if (int e = batch2d_reserve(ctx, overflow + overflow / 4 + 1024)) return e;
      continue;
    }
    done += chunk;
  }
  // Counters and the last step's per-scene results.
  unsigned long long sums[2] = {0, 0};
  int ctl[1] = {0};
  std::vector<unsigned> iters(S);
  std::vector<double> best(S);
  std::vector<int> sdone(S);
  SG_CUDA_TRY(cudaMemcpyAsync(sums, ctx->b_sums.p, sizeof sums, cudaMemcpyDeviceToHost, s));
  SG_CUDA_TRY(cudaMemcpyAsync(ctl, ctx->b_ctl.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  SG_CUDA_TRY(cudaMemcpyAsync(iters.data(), ctx->s_iters.p, sizeof(unsigned) * S, cudaMemcpyDeviceToHost, s));
  SG_CUDA_TRY(cudaMemcpyAsync(best.data(), ctx->s_best.p, sizeof(double) * S, cudaMemcpyDeviceToHost, s));
  SG_CUDA_TRY(cudaMemcpyAsync(sdone.data(), ctx->s_done.p, sizeof(int) * S, cudaMemcpyDeviceToHost, s));
  SG_CUDA_TRY(cudaMemcpyAsync(&ctx->h_stats, ctx->stats.p, sizeof(SolveStats), cudaMemcpyDeviceToHost, s));
  SG_CUDA_TRY(cudaStreamSynchronize(s));
  sg_step_stats st{};
  st.n_contacts = ctl[0];
  st.succeeded = 1;
  for (int k = 0; k < S; ++k) {
    st.iterations = std::max(st.iterations, iters[k]);
    if (!sdone[k]) st.succeeded = 0;
    if (best[k] < INFINITY && best[k] > st.error) st.error = best[k];
  }
  st.n_colors = (uint32_t)ctx->h_stats.n_colors;
  ctx->last_nc = ctl[0];
  ctx->contacts_total += sums[0];
  unsigned long long work[5] = {0, 0, 0, 0, 0};
  SG_CUDA_TRY(cudaMemcpy(work, ctx->b_work.p, sizeof work, cudaMemcpyDeviceToHost));
  ctx->contact_sweeps32 += work[0];
  ctx->contact_sweeps += work[1];
  ctx->contact_evals += work[2];
  ctx->contact_lifts += work[3];
  ctx->body_lifts += work[4];
  if (out) *out = st;
  if (total) *total = (int64_t)sums[0];
  return sums[1] ? SG_NOT_CONVERGED : SG_OK;
}

static int check_integrator(const sg_ctx* ctx) {
  const bool split = ctx->cfg.integrator == SG_SPLIT_HAM;
  if ((ctx->dim == 3) != split) {
    set_error(ctx->dim == 3 ? "sphere scenes step with SG_SPLIT_HAM"
                            : "Ball2D scenes step with SG_SYMPLECTIC_EULER or SG_VERLET");
    return SG_BAD_INPUT;
  }
  return SG_OK;
}

static size_t q_doubles(const sg_ctx* ctx) { return (size_t)ctx->nb * (ctx->dim == 3 ? 12 : ctx->rb2d ? 3 : 2); }
static size_t v_doubles(const sg_ctx* ctx) { return (size_t)ctx->nb * (ctx->dim == 3 ? 6 : ctx->rb2d ? 3 : 2); }

int sg_step(sg_ctx* ctx, uint32_t first_iteration, uint32_t n_steps, sg_step_stats* stats, int64_t* total_contacts) {
  if (!ctx) return SG_BAD_INPUT;
  (void)first_iteration;  // gravity is time independent
  if (int e = check_integrator(ctx)) return e;
  SG_CUDA_TRY(cudaSetDevice(ctx->device));
  if (ctx->n_scenes > 0 && ctx->dim == 2) return batch_step(ctx, n_steps, stats, total_contacts);
  int64_t tot = 0;
  int worst = SG_OK;
  sg_step_stats st{};
  for (uint32_t k = 0; k < n_steps; ++k) {
    const int r = ctx->dim == 3 ? (ctx->n_scenes > 0 ? sphere3d_batch_step(ctx, &st) : sphere3d_step(ctx, &st))
                                : ctx->rb2d ? rb2d_step(ctx, &st) : step_once(ctx, &st);
    if (r != SG_OK && r != SG_NOT_CONVERGED) return r;
    if (r == SG_NOT_CONVERGED) worst = r;
    tot += st.n_contacts;
  }
  if (stats) *stats = st;
  if (total_contacts) *total_contacts = tot;
  return worst;
}

int sg_flow(sg_ctx* ctx, uint32_t iteration, const double* q0, const double* v0, double* q1, double* v1,
            sg_step_stats* stats) {
  if (!ctx || (ctx->nb > 0 && (!q0 || !v0 || !q1 || !v1))) return SG_BAD_INPUT;
  if (int e = check_integrator(ctx)) return e;
  SG_CUDA_TRY(cudaSetDevice(ctx->device));
  const size_t qb = sizeof(double) * q_doubles(ctx), vb = sizeof(double) * v_doubles(ctx);
  SG_CUDA_TRY(cudaMemcpyAsync(ctx->q.p, q0, qb, cudaMemcpyHostToDevice, ctx->stream));
  SG_CUDA_TRY(cudaMemcpyAsync(ctx->v.p, v0, vb, cudaMemcpyHostToDevice, ctx->stream));
  // A 3D state carries its own orientations: the world inertia follows them (updateMandMinv).
  if (ctx->dim == 3)
    if (int e = sphere3d_update_inertia(ctx, false)) return e;
  const int r = sg_step(ctx, iteration, 1, stats, nullptr);
  if (r != SG_OK && r != SG_NOT_CONVERGED) return r;
  SG_CUDA_TRY(cudaMemcpyAsync(q1, ctx->q.p, qb, cudaMemcpyDeviceToHost, ctx->stream));
  SG_CUDA_TRY(cudaMemcpyAsync(v1, ctx->v.p, vb, cudaMemcpyDeviceToHost, ctx->stream));
  SG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return r;
}

int sg_download_state(sg_ctx* ctx, double* q, double* v) {
  if (!ctx) return SG_BAD_INPUT;
  SG_CUDA_TRY(cudaSetDevice(ctx->device));
  if (q) SG_CUDA_TRY(cudaMemcpyAsync(q, ctx->q.p, sizeof(double) * q_doubles(ctx), cudaMemcpyDeviceToHost, ctx->stream));
  if (v) SG_CUDA_TRY(cudaMemcpyAsync(v, ctx->v.p, sizeof(double) * v_doubles(ctx), cudaMemcpyDeviceToHost, ctx->stream));
  SG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SG_OK;
}

int64_t sg_last_contacts(sg_ctx* ctx, int64_t cap, int32_t* ia, int32_t* ib, double* n, double* alpha, double* beta) {
  if (!ctx) return SG_BAD_INPUT;
  if (ctx->dim != 2) {
    set_error("sg_last_contacts: sphere scenes use sg_sphere3d_last_contacts");
    return INT64_MIN;
  }
  const int64_t nc = ctx->last_nc;
  if (nc > cap) return -(nc + 1);
  if (nc == 0) return 0;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return -1;
  cudaStream_t s = ctx->stream;
  const size_t c = (size_t)nc;
  if (ia) cudaMemcpyAsync(ia, ctx->ia.p, sizeof(int) * c, cudaMemcpyDeviceToHost, s);
  if (ib) cudaMemcpyAsync(ib, ctx->ib.p, sizeof(int) * c, cudaMemcpyDeviceToHost, s);
  if (n) cudaMemcpyAsync(n, ctx->n.p, sizeof(double) * 2 * c, cudaMemcpyDeviceToHost, s);
  // (alpha, beta) were cached into prev_ab when caching is on, else into ab.
  const double* abp = (ctx->cfg.cache_mode != SG_CACHE_NONE) ? ctx->prev_ab.as<double>() : ctx->ab.as<double>();
  if (alpha || beta) {
    std::vector<double> ab(2 * c);
    cudaMemcpyAsync(ab.data(), abp, sizeof(double) * 2 * c, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    for (size_t k = 0; k < c; ++k) {
      if (alpha) alpha[k] = ab[2 * k];
      if (beta) beta[k] = ab[2 * k + 1];
    }
  }
  if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
  return nc;
}

int sg_batch2d_upload(sg_ctx* ctx, int32_t n_scenes, const int32_t* body_off, const double* q, const double* v,
                      const double* r, const double* m, const int32_t* plane_off, const double* plane_x,
                      const double* plane_n, const double* mu, const double* CoR) {
  if (!ctx) return SG_BAD_INPUT;
  SG_CUDA_TRY(cudaSetDevice(ctx->device));
  return batch_upload(ctx, n_scenes, body_off, q, v, r, m, plane_off, plane_x, plane_n, mu, CoR);
}

int sg_batch2d_set_capacity(sg_ctx* ctx, int32_t contacts) {
  if (!ctx || ctx->n_scenes == 0 || contacts < 1) return SG_BAD_INPUT;
  SG_CUDA_TRY(cudaSetDevice(ctx->device));
  if (ctx->graph) {
    cudaGraphExecDestroy(ctx->graph);
    ctx->graph = nullptr;
  }
  // Shrinking keeps the allocations but caps the pipeline at `contacts`.
  if (contacts > ctx->bcap) return batch2d_reserve(ctx, contacts);
  ctx->bcap = contacts;
  return SG_OK;
}

int sg_batch2d_scene_stats(sg_ctx* ctx, int32_t* n_contacts, uint32_t* iterations, double* error,
                           int32_t* succeeded) {
  if (!ctx || ctx->n_scenes == 0) return SG_BAD_INPUT;
  SG_CUDA_TRY(cudaSetDevice(ctx->device));
  const int S = ctx->n_scenes;
  cudaStream_t s = ctx->stream;
  // After a cached step the step's offsets were swapped into prev_sc_off.
  const Buf& off = ctx->cfg.cache_mode != SG_CACHE_NONE ? ctx->prev_sc_off : ctx->sc_off;
  std::vector<int> o(S + 1), d(S);
  SG_CUDA_TRY(cudaMemcpyAsync(o.data(), off.p, sizeof(int) * (S + 1), cudaMemcpyDeviceToHost, s));
  SG_CUDA_TRY(cudaMemcpyAsync(d.data(), ctx->s_done.p, sizeof(int) * S, cudaMemcpyDeviceToHost, s));
  if (iterations)
    SG_CUDA_TRY(cudaMemcpyAsync(iterations, ctx->s_iters.p, sizeof(unsigned) * S, cudaMemcpyDeviceToHost, s));
  if (error) SG_CUDA_TRY(cudaMemcpyAsync(error, ctx->s_best.p, sizeof(double) * S, cudaMemcpyDeviceToHost, s));
  SG_CUDA_TRY(cudaStreamSynchronize(s));
  for (int k = 0; k < S; ++k) {
    if (n_contacts) n_contacts[k] = o[k + 1] - o[k];
    if (succeeded) succeeded[k] = d[k];
    if (error && o[k + 1] == o[k]) error[k] = 0.0;
  }
  return SG_OK;
}

int sg_sphere3d_upload(sg_ctx* ctx, int32_t nb, const double* q, const double* v, const double* r, const double* m,
                       const double* I0, int32_t np, const double* plane_x, const double* plane_n) {
  return sphere3d_upload_impl(ctx, nb, q, v, r, m, I0, np, plane_x, plane_n);
}

int sg_sphere3d_batch_upload(sg_ctx* ctx, int32_t S, const int32_t* body_off, const double* q, const double* v,
                             const double* r, const double* m, const double* I0, const int32_t* plane_off,
                             const double* plane_x, const double* plane_n, const double* mu, const double* CoR) {
  if (!ctx || S < 1 || !body_off || !plane_off || !mu || !CoR || body_off[0] != 0 || plane_off[0] != 0) {
    set_error("sg_sphere3d_batch_upload: invalid arguments");
    return SG_BAD_INPUT;
  }
  std::vector<int> sf(S + 1, 0), scene_of;
  long cells = 0;
  for (int s = 0; s < S; ++s) {
    const int ns = body_off[s + 1] - body_off[s], np = plane_off[s + 1] - plane_off[s];
    if (ns < 0 || np < 0 || !(mu[s] >= 0.0) || !(CoR[s] >= 0.0 && CoR[s] <= 1.0)) {
      set_error("sg_sphere3d_batch_upload: offsets must not decrease; mu >= 0, 0 <= CoR <= 1 per scene");
      return SG_BAD_INPUT;
    }
    const long f = (long)sf[s] + (long)ns * np;
    cells += 4L * ns + 64;
    if (f > (1L << 30) || cells > (1L << 30)) {
      set_error("sg_sphere3d_batch_upload: batch too large");
      return SG_CAPACITY;
    }
    sf[s + 1] = (int)f;
    scene_of.insert(scene_of.end(), (size_t)ns, s);
  }
  const int N = body_off[S], NP = plane_off[S];
  if (int e = sphere3d_upload_impl(ctx, N, q, v, r, m, I0, NP, plane_x, plane_n)) return e;
  ctx->n_scenes = S;
  ctx->bcells = cells;
  ctx->bflags = sf[S];
  const size_t s1 = sizeof(int) * (size_t)(S + 1);
  if (int e = upload(ctx, ctx->sb_off, body_off, s1)) return e;
  if (int e = upload(ctx, ctx->sp_off, plane_off, s1)) return e;
  if (int e = upload(ctx, ctx->sf_off, sf.data(), s1)) return e;
  if (int e = upload(ctx, ctx->scene_of, scene_of.data(), sizeof(int) * (size_t)std::max(N, 1))) return e;
  if (int e = upload(ctx, ctx->s_mu, mu, sizeof(double) * (size_t)S)) return e;
  if (int e = upload(ctx, ctx->s_CoR, CoR, sizeof(double) * (size_t)S)) return e;
  if (int e = sphere3d_batch_setup(ctx, sf[S], cells)) return e;
  ctx->s_smax = 0;
  SG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SG_OK;
}

int64_t sg_sphere3d_last_contacts(sg_ctx* ctx, int64_t cap, int32_t* ia, int32_t* ib, double* bases, double* alpha,
                                  double* beta) {
  if (!ctx) return INT64_MIN;
  if (ctx->dim != 3) {
    set_error("sg_sphere3d_last_contacts: not a sphere scene");
    return INT64_MIN;
  }
  const int64_t nc = ctx->last_nc;
  if (nc > cap) return -(nc + 1);
  if (nc == 0) return 0;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return INT64_MIN;
  cudaStream_t s = ctx->stream;
  const size_t c = (size_t)nc;
  if (ia) cudaMemcpyAsync(ia, ctx->ia.p, sizeof(int) * c, cudaMemcpyDeviceToHost, s);
  if (ib) cudaMemcpyAsync(ib, ctx->ib.p, sizeof(int) * c, cudaMemcpyDeviceToHost, s);
  if (bases) {
    // Device rows n, s, t of each contact = columns of the 3x3 basis: column-major [n s t].
    cudaMemcpyAsync(bases, ctx->E3.p, sizeof(double) * 9 * c, cudaMemcpyDeviceToHost, s);
  }
  if (alpha || beta) {
    std::vector<double> ab(3 * c);
    cudaMemcpyAsync(ab.data(), ctx->ab3.p, sizeof(double) * 3 * c, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return INT64_MIN;
    for (size_t k = 0; k < c; ++k) {
      if (alpha) alpha[k] = ab[3 * k];
      if (beta) {
        beta[2 * k] = ab[3 * k + 1];
        beta[2 * k + 1] = ab[3 * k + 2];
      }
    }
  }
  if (cudaStreamSynchronize(s) != cudaSuccess) return INT64_MIN;
  return nc;
}

int sg_sphere3d_world_inertia(sg_ctx* ctx, double* Iw, double* Iinv) {
  if (!ctx || ctx->dim != 3) return SG_BAD_INPUT;
  SG_CUDA_TRY(cudaSetDevice(ctx->device));
  const size_t bytes = sizeof(double) * 9 * (size_t)ctx->nb;
  if (Iw && bytes) SG_CUDA_TRY(cudaMemcpyAsync(Iw, ctx->Iw.p, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  if (Iinv && bytes) SG_CUDA_TRY(cudaMemcpyAsync(Iinv, ctx->Iinv.p, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  SG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SG_OK;
}

int64_t sg_last_solve_order(sg_ctx* ctx, int64_t cap, int32_t* order, int32_t* color_offsets, int32_t* n_colors) {
  if (!ctx) return SG_BAD_INPUT;
  const int64_t nc = ctx->last_nc;
  if (nc > cap) return -(nc + 1);
  if (n_colors) *n_colors = ctx->h_stats.n_colors;
  if (color_offsets)
    for (int c = 0; c <= ctx->h_stats.n_colors; ++c) color_offsets[c] = ctx->h_stats.color_off[c];
  if (order && nc > 0) {
    if (cudaMemcpy(order, ctx->perm.p, sizeof(int) * (size_t)nc, cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  }
  return nc;
}

// FrictionSolver::solve for Ball2D on host buffers (sg_sobogus_solve_2d and its form with the map's extra
// relative velocities).  nrel_extra / drel_extra (one per contact, null = zero) are added to the kinematic
// relative velocities before the forcing terms are formed, as Sobogus::solve does
// (scisim/ConstrainedMaps/Sobogus.cpp:892-904, then Constraint::computeForcingTerm, Constraint.cpp:27-33).
static int sobogus_solve_2d_impl(sg_ctx* ctx, int32_t nb, const double* m, const double* v0, int32_t nc,
                                 const int32_t* ia, const int32_t* ib, const double* bases, const double* CoR,
                                 const double* mu, const double* nrel_extra, const double* drel_extra,
                                 uint32_t max_iters, double tol, uint32_t eval_every, double* alpha, double* beta,
                                 double* v2, double* f, double* error, uint32_t* iterations) {
  if (!ctx || nb < 0 || nc < 0 || (nb > 0 && (!m || !v0 || !v2 || !f)) ||
      (nc > 0 && (!ia || !ib || !bases || !CoR || !mu || !alpha || !beta))) {
    set_error("sg_sobogus_solve_2d: invalid arguments");
    return SG_BAD_INPUT;
  }
  for (int k = 0; k < nc; ++k) {
    if (ia[k] < 0 || ia[k] >= nb || ib[k] >= nb || ib[k] == ia[k] || ib[k] < -1) {
      set_error("sg_sobogus_solve_2d: contact body index out of range");
      return SG_BAD_INPUT;
    }
  }
  SG_CUDA_TRY(cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  // Host-side assembly of the per-contact data (what the step pipeline does on the device).
  std::vector<double> minv(nb), n(2 * (size_t)nc), c(2 * (size_t)nc), W(3 * (size_t)nc), rl(2 * (size_t)nc);
  for (int i = 0; i < nb; ++i) minv[i] = 1.0 / m[i];
  for (int k = 0; k < nc; ++k) {
    const double* B = bases + 4 * k;
    const double nx = B[0], ny = B[1], tx = B[2], ty = B[3];
    n[2 * k] = nx;
    n[2 * k + 1] = ny;
    const int a = ia[k], b = ib[k];
    double vrx = v0[2 * a], vry = v0[2 * a + 1];
    if (b >= 0) {
      vrx = vrx - v0[2 * b];
      vry = vry - v0[2 * b + 1];
    } else {
      vrx = vrx - 0.0;
      vry = vry - 0.0;
    }
    const double ndotv = nx * vrx + ny * vry;
    double nrel = -(0.0 * nx + 0.0 * ny);
    double drel = -(0.0 * tx + 0.0 * ty);
    if (nrel_extra) nrel = nrel + nrel_extra[k];
    if (drel_extra) drel = drel + drel_extra[k];
    const double sc = CoR[k] * ndotv + nrel;
    const double wx = (0.0 + nx * sc) + tx * drel;
    const double wy = (0.0 + ny * sc) + ty * drel;
    c[2 * k] = nx * wx + ny * wy;
    c[2 * k + 1] = tx * wx + ty * wy;
    const double nn = nx * nx + ny * ny, nt = nx * tx + ny * ty, tt = tx * tx + ty * ty;
    double w00 = minv[a] * nn, w01 = minv[a] * nt, w11 = minv[a] * tt;
    if (b >= 0) {
      w00 = w00 + minv[b] * nn;
      w01 = w01 + minv[b] * nt;
      w11 = w11 + minv[b] * tt;
    }
    W[3 * k] = w00;
    W[3 * k + 1] = w01;
    W[3 * k + 2] = w11;
    const double rwx = alpha[k] * nx + beta[k] * tx;
    const double rwy = alpha[k] * ny + beta[k] * ty;
    rl[2 * k] = nx * rwx + ny * rwy;
    rl[2 * k + 1] = tx * rwx + ty * rwy;
    if (std::fabs(tx + ny) > 0.0 || std::fabs(ty - nx) > 0.0) {
      set_error("sg_sobogus_solve_2d: tangent must be (-n_y, n_x)");
      return SG_BAD_INPUT;
    }
  }
  // Device buffers: reuse the context's scene and contact buffers.
  if (int e = upload(ctx, ctx->fs_m, m, sizeof(double) * nb)) return e;
  if (int e = upload(ctx, ctx->fs_minv, minv.data(), sizeof(double) * nb)) return e;
  if (int e = upload(ctx, ctx->fs_v0, v0, sizeof(double) * 2 * nb)) return e;
  if (int e = grow(ctx->fs_v2, sizeof(double) * 2 * (size_t)std::max(nb, 1))) return e;
  if (int e = ensure_contact_capacity(ctx, nc)) return e;
  std::vector<double> mus(mu, mu + nc);
  if (nc > 0) {
    SG_CUDA_TRY(cudaMemcpyAsync(ctx->ia.p, ia, sizeof(int) * nc, cudaMemcpyHostToDevice, s));
    SG_CUDA_TRY(cudaMemcpyAsync(ctx->ib.p, ib, sizeof(int) * nc, cudaMemcpyHostToDevice, s));
    SG_CUDA_TRY(cudaMemcpyAsync(ctx->n.p, n.data(), sizeof(double) * 2 * nc, cudaMemcpyHostToDevice, s));
    SG_CUDA_TRY(cudaMemcpyAsync(ctx->c.p, c.data(), sizeof(double) * 2 * nc, cudaMemcpyHostToDevice, s));
    SG_CUDA_TRY(cudaMemcpyAsync(ctx->W.p, W.data(), sizeof(double) * 3 * nc, cudaMemcpyHostToDevice, s));
    SG_CUDA_TRY(cudaMemcpyAsync(ctx->mu.p, mus.data(), sizeof(double) * nc, cudaMemcpyHostToDevice, s));
    SG_CUDA_TRY(cudaMemcpyAsync(ctx->r_loc.p, rl.data(), sizeof(double) * 2 * nc, cudaMemcpyHostToDevice, s));
  }
  ContactProblem P;
  P.nb = nb;
  P.nc = nc;
  P.minv = ctx->fs_minv.as<double>();
  P.m = ctx->fs_m.as<double>();
  P.v0 = ctx->fs_v0.as<double>();
  P.ia = ctx->ia.as<int>();
  P.ib = ctx->ib.as<int>();
  P.n = ctx->n.as<double>();
  P.c = ctx->c.as<double>();
  P.W = ctx->W.as<double>();
  P.mu = ctx->mu.as<double>();
  P.r = ctx->r_loc.as<double>();
  P.v2 = ctx->fs_v2.as<double>();
  SolveParams sp{tol, max_iters, eval_every, ctx->cfg.precision};
  const int sr = solve_contacts(ctx, P, sp);
  if (sr != SG_OK && sr != SG_NOT_CONVERGED) return sr;
  ctx->last_nc = nc;
  if (nb > 0) SG_CUDA_TRY(cudaMemcpyAsync(v2, ctx->fs_v2.p, sizeof(double) * 2 * nb, cudaMemcpyDeviceToHost, s));
  if (nc > 0) SG_CUDA_TRY(cudaMemcpyAsync(rl.data(), ctx->r_loc.p, sizeof(double) * 2 * nc, cudaMemcpyDeviceToHost, s));
  SG_CUDA_TRY(cudaStreamSynchronize(s));
  // r to world, alpha/beta and the friction force f (Sobogus.cpp:309-347).
  for (int i = 0; i < 2 * nb; ++i) f[i] = 0.0;
  for (int k = 0; k < nc; ++k) {
    const double nx = n[2 * k], ny = n[2 * k + 1], tx = -ny, ty = nx;
    const double rwx = nx * rl[2 * k] + tx * rl[2 * k + 1];
    const double rwy = ny * rl[2 * k] + ty * rl[2 * k + 1];
    alpha[k] = rwx * nx + rwy * ny;
    beta[k] = (mu[k] == 0.0) ? 0.0 : (rwx * tx + rwy * ty);
    const double f0x = beta[k] * tx, f0y = beta[k] * ty;
    f[2 * ia[k]] += f0x;
    f[2 * ia[k] + 1] += f0y;
    if (ib[k] >= 0) {
      f[2 * ib[k]] -= f0x;
      f[2 * ib[k] + 1] -= f0y;
    }
  }
  if (error) *error = (nc == 0) ? 0.0 : ctx->h_stats.error;
  if (iterations) *iterations = ctx->h_stats.iterations;
  return sr;
}

int sg_sobogus_solve_2d(sg_ctx* ctx, int32_t nb, const double* m, const double* v0, int32_t nc, const int32_t* ia,
                        const int32_t* ib, const double* bases, const double* CoR, const double* mu, uint32_t max_iters,
                        double tol, uint32_t eval_every, double* alpha, double* beta, double* v2, double* f,
                        double* error, uint32_t* iterations) {
  return sobogus_solve_2d_impl(ctx, nb, m, v0, nc, ia, ib, bases, CoR, mu, nullptr, nullptr, max_iters, tol,
                               eval_every, alpha, beta, v2, f, error, iterations);
}

int sg_sobogus_solve_2d_ex(sg_ctx* ctx, int32_t nb, const double* m, const double* v0, int32_t nc,
                           const int32_t* ia, const int32_t* ib, const double* bases, const double* CoR,
                           const double* mu, const double* nrel_extra, const double* drel_extra, uint32_t max_iters,
                           double tol, uint32_t eval_every, double* alpha, double* beta, double* v2, double* f,
                           double* error, uint32_t* iterations) {
  return sobogus_solve_2d_impl(ctx, nb, m, v0, nc, ia, ib, bases, CoR, mu, nrel_extra, drel_extra, max_iters, tol,
                               eval_every, alpha, beta, v2, f, error, iterations);
}

int sg_sobogus_solve_3d(sg_ctx* ctx, int32_t nb, const double* m, const double* Iw, const double* Iinv,
                        const double* v0, int32_t nc, const int32_t* ia, const int32_t* ib, const double* bases,
                        const double* arm_a, const double* arm_b, const double* CoR, const double* mu,
                        const double* nrel_extra, const double* drel_extra, uint32_t max_iters, double tol,
                        uint32_t eval_every, double* alpha, double* beta, double* v2, double* f, double* error,
                        uint32_t* iterations) {
  return sobogus_solve_3d(ctx, nb, m, Iw, Iinv, v0, nc, ia, ib, bases, arm_a, arm_b, CoR, mu, nrel_extra, drel_extra,
                          max_iters, tol, eval_every, alpha, beta, v2, f, error, iterations);
}

int sg_broadphase_2d(sg_ctx* ctx, int32_t n, const double* aabb, int64_t cap, int32_t* pairs, int64_t* npairs) {
  if (!ctx || n < 0 || (n > 0 && !aabb) || !npairs || cap < 0 || (cap > 0 && !pairs)) return SG_BAD_INPUT;
  SG_CUDA_TRY(cudaSetDevice(ctx->device));
  *npairs = 0;
  if (n == 0) return SG_OK;
  cudaStream_t s = ctx->stream;
  Buf d_aabb;
  if (int e = upload(ctx, d_aabb, aabb, sizeof(double) * 4 * (size_t)n)) return e;
  int rc = broadphase_build_grid(ctx, d_aabb.as<double>(), n);
  if (!rc) rc = broadphase_count_pairs(ctx, d_aabb.as<double>(), n, false);
  int total = 0;
  if (!rc) {
    if (cudaMemcpyAsync(&total, ctx->pair_off.as<int>() + n, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      rc = SG_CUDA_ERROR;
  }
  *npairs = total;
  if (!rc && total > cap) rc = SG_CAPACITY;
  if (!rc && total > 0) {
    Buf da, db;
    rc = grow(da, sizeof(int) * (size_t)total);
    if (!rc) rc = grow(db, sizeof(int) * (size_t)total);
    if (!rc) rc = broadphase_write_pairs(ctx, d_aabb.as<double>(), n, false, da.as<int>(), db.as<int>());
    if (!rc) {
      std::vector<int> ha(total), hb(total);
      cudaMemcpyAsync(ha.data(), da.p, sizeof(int) * total, cudaMemcpyDeviceToHost, s);
      cudaMemcpyAsync(hb.data(), db.p, sizeof(int) * total, cudaMemcpyDeviceToHost, s);
      if (cudaStreamSynchronize(s) != cudaSuccess) rc = SG_CUDA_ERROR;
      for (int k = 0; k < total && !rc; ++k) {
        pairs[2 * k] = ha[k];
        pairs[2 * k + 1] = hb[k];
      }
    }
    release(da);
    release(db);
  }
  release(d_aabb);
  return rc;
}

int sg_ccd_2d(sg_ctx* ctx, int32_t n, const double* q0a, const double* q1a, const double* ra, const double* q0b,
              const double* q1b, const double* rb, double* coeffs, int32_t* hit, double* t) {
  if (!ctx || n < 0) return SG_BAD_INPUT;
  if (n == 0) return SG_OK;
  SG_CUDA_TRY(cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  Buf b[9];
  const size_t d2 = sizeof(double) * 2 * (size_t)n, d1 = sizeof(double) * (size_t)n;
  int rc = upload(ctx, b[0], q0a, d2);
  if (!rc) rc = upload(ctx, b[1], q1a, d2);
  if (!rc) rc = upload(ctx, b[2], ra, d1);
  if (!rc) rc = upload(ctx, b[3], q0b, d2);
  if (!rc) rc = upload(ctx, b[4], q1b, d2);
  if (!rc) rc = upload(ctx, b[5], rb, d1);
  if (!rc) rc = grow(b[6], 3 * d1);
  if (!rc) rc = grow(b[7], sizeof(int) * (size_t)n);
  if (!rc) rc = grow(b[8], d1);
  if (!rc)
    rc = ccd_batch(ctx, n, b[0].as<double>(), b[1].as<double>(), b[2].as<double>(), b[3].as<double>(),
                   b[4].as<double>(), b[5].as<double>(), b[6].as<double>(), b[7].as<int>(), b[8].as<double>());
  if (!rc) {
    cudaMemcpyAsync(coeffs, b[6].p, 3 * d1, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(hit, b[7].p, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(t, b[8].p, d1, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) rc = SG_CUDA_ERROR;
  }
  for (auto& x : b) release(x);
  return rc;
}

int sg_last_patch_layout(sg_ctx* ctx, int64_t nc, int64_t nb, int32_t* counts, int32_t* group, int32_t* color,
                         int32_t* body_patch, int32_t* body_tile, int32_t* body_band) {
  if (!ctx || !counts || !group || !color || !body_patch || !body_tile || !body_band) return SG_BAD_INPUT;
  if (!ctx->last_patched || nc != ctx->last_nc || nb != (int64_t)ctx->nb) {
    set_error("sg_last_patch_layout: the last solve did not run the two-level sweeps on this many contacts/bodies");
    return SG_BAD_INPUT;
  }
  SG_CUDA_TRY(cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  const size_t c = (size_t)nc, b = (size_t)nb;
  std::vector<int32_t> key(c);
  if (c) SG_CUDA_TRY(cudaMemcpyAsync(key.data(), ctx->pt_key.p, sizeof(int32_t) * c, cudaMemcpyDeviceToHost, s));
  if (b) {
    SG_CUDA_TRY(cudaMemcpyAsync(body_patch, ctx->pt_patch.p, sizeof(int32_t) * b, cudaMemcpyDeviceToHost, s));
    SG_CUDA_TRY(cudaMemcpyAsync(body_tile, ctx->pt_qpatch.p, sizeof(int32_t) * b, cudaMemcpyDeviceToHost, s));
    SG_CUDA_TRY(cudaMemcpyAsync(body_band, ctx->pt_band.p, sizeof(int32_t) * b, cudaMemcpyDeviceToHost, s));
  }
  SG_CUDA_TRY(cudaStreamSynchronize(s));
  for (size_t k = 0; k < c; ++k) {
    group[k] = key[k] / kMaxColors;
    color[k] = key[k] % kMaxColors;
  }
  counts[0] = ctx->last_patch_P;
  counts[1] = ctx->last_patch_Pb;
  return SG_OK;
}

// ---------------------------------------------------------------------------
// Checkpoint / resume of a single-scene context (the reference serialises the whole simulation,
// ball2dcli/ball2d_cli.cpp:199-316, Ball2DSim.cpp:810-822).  Layout: CkptHeader, then the
// device arrays byte for byte (so that a resumed run is bit-identical: normalised plane normals,
// inverse masses and world inertia are restored as stored, not recomputed), then the impulse
// cache (sorted keys, (alpha, beta) per key).
namespace {
struct CkptHeader {
  char magic[8];
  int32_t version, dim, nb, np;
  int64_t prev_n;
  sg_config cfg;
  int32_t staggering, stabilize;
  double pen_thresh;
};
constexpr char kCkptMagic[8] = {'S', 'G', 'C', 'K', 'P', 'T', '1', 0};

struct CkptPart {
  Buf* buf;
  size_t bytes;
};

std::vector<CkptPart> ckpt_parts(sg_ctx* ctx, int dim, int nb, int np, int64_t prev_n) {
  const size_t d = sizeof(double), b = (size_t)nb, p = (size_t)np;
  std::vector<CkptPart> v;
  if (dim == 2) {
    v = {{&ctx->q, 2 * b * d},       {&ctx->v, 2 * b * d},       {&ctx->r, b * d},
         {&ctx->m, b * d},           {&ctx->minv, b * d},        {&ctx->plane_x, 2 * p * d},
         {&ctx->plane_n, 2 * p * d}, {&ctx->plane_t, 2 * p * d}};
  } else {
    v = {{&ctx->q, 12 * b * d},  {&ctx->v, 6 * b * d},         {&ctx->r, b * d},
         {&ctx->m, b * d},       {&ctx->minv, b * d},          {&ctx->I0, 3 * b * d},
         {&ctx->Iw, 9 * b * d},  {&ctx->Iinv, 9 * b * d},      {&ctx->plane_x, 3 * p * d},
         {&ctx->plane_n, 3 * p * d}};
  }
  // The impulse cache: (alpha, beta) per Ball2D contact; the cached normal and force (6) per
  // sphere contact (symplectic-Euler staggering; the geometric sphere map keeps none).
  v.push_back({&ctx->prev_key, (size_t)prev_n * sizeof(unsigned long long)});
  if (dim == 2) {
    v.push_back({&ctx->prev_ab, (size_t)prev_n * 2 * d});
    // The cached step's colours: the next step's colouring starts from them, so a resumed run
    // colours, and therefore sweeps, as the uninterrupted one.
    v.push_back({&ctx->prev_color, (size_t)prev_n * sizeof(int)});
  } else {
    v.push_back({&ctx->prev_c6, (size_t)prev_n * 6 * d});
  }
  return v;
}

bool ckpt_supported(const sg_ctx* ctx) { return ctx->n_scenes == 0 && !ctx->rb2d && (ctx->dim == 2 || ctx->dim == 3); }
}  // namespace

int64_t sg_checkpoint_size(sg_ctx* ctx) {
  if (!ctx || !ckpt_supported(ctx)) {
    set_error("sg_checkpoint_size: needs a context holding one Ball2D or sphere scene");
    return -1;
  }
  size_t total = sizeof(CkptHeader);
  for (const CkptPart& part : ckpt_parts(ctx, ctx->dim, ctx->nb, ctx->np, ctx->prev_n)) total += part.bytes;
  return (int64_t)total;
}

int sg_checkpoint_save(sg_ctx* ctx, void* buf, int64_t bytes) {
  const int64_t need = sg_checkpoint_size(ctx);
  if (need < 0 || !buf || bytes < need) {
    if (need >= 0) set_error("sg_checkpoint_save: buffer smaller than sg_checkpoint_size");
    return SG_BAD_INPUT;
  }
  SG_CUDA_TRY(cudaSetDevice(ctx->device));
  CkptHeader h{};
  std::memcpy(h.magic, kCkptMagic, sizeof(h.magic));
  h.version = 1;
  h.dim = ctx->dim;
  h.nb = ctx->nb;
  h.np = ctx->np;
  h.prev_n = ctx->prev_n;
  h.cfg = ctx->cfg;
  h.staggering = ctx->staggering;
  h.stabilize = ctx->stabilize;
  h.pen_thresh = ctx->pen_thresh;
  char* out = static_cast<char*>(buf);
  std::memcpy(out, &h, sizeof(h));
  size_t off = sizeof(h);
  for (const CkptPart& part : ckpt_parts(ctx, h.dim, h.nb, h.np, h.prev_n)) {
    if (part.bytes)
      SG_CUDA_TRY(cudaMemcpyAsync(out + off, part.buf->p, part.bytes, cudaMemcpyDeviceToHost, ctx->stream));
    off += part.bytes;
  }
  SG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SG_OK;
}

int sg_checkpoint_load(sg_ctx* ctx, const void* buf, int64_t bytes) {
  if (!ctx || !buf || bytes < (int64_t)sizeof(CkptHeader)) {
    set_error("sg_checkpoint_load: invalid arguments");
    return SG_BAD_INPUT;
  }
  CkptHeader h;
  std::memcpy(&h, buf, sizeof(h));
  if (std::memcmp(h.magic, kCkptMagic, sizeof(h.magic)) != 0 || h.version != 1 || (h.dim != 2 && h.dim != 3) ||
      h.nb < 0 || h.np < 0 || h.prev_n < 0) {
    set_error("sg_checkpoint_load: not a checkpoint of this library");
    return SG_BAD_INPUT;
  }
  size_t need = sizeof(h);
  for (const CkptPart& part : ckpt_parts(ctx, h.dim, h.nb, h.np, h.prev_n)) need += part.bytes;
  if ((size_t)bytes < need) {
    set_error("sg_checkpoint_load: truncated checkpoint");
    return SG_BAD_INPUT;
  }
  sg_config cfg = h.cfg;
  cfg.device = ctx->device;
  if (int r = sg_ctx_reconfigure(ctx, &cfg)) return r;
  // Upload through the normal path (allocation, validation), then overwrite every array with
  // the stored bytes.
  const char* in = static_cast<const char*>(buf) + sizeof(h);
  const size_t b = (size_t)h.nb, d = sizeof(double);
  std::vector<double> tmp;
  auto arr = [&](size_t at_doubles, size_t n) {
    tmp.resize(n);
    if (n) std::memcpy(tmp.data(), in + at_doubles * d, n * d);
    return tmp;
  };
  int rc;
  if (h.dim == 2) {
    const std::vector<double> qv = arr(0, 2 * b), vv = arr(2 * b, 2 * b), rv = arr(4 * b, b), mv = arr(5 * b, b);
    const size_t p0 = 7 * b;
    const std::vector<double> px = arr(p0, 2 * (size_t)h.np), pn = arr(p0 + 2 * (size_t)h.np, 2 * (size_t)h.np);
    rc = sg_ball2d_upload(ctx, h.nb, qv.data(), vv.data(), rv.data(), mv.data(), h.np, px.data(), pn.data());
  } else {
    const std::vector<double> qv = arr(0, 12 * b), vv = arr(12 * b, 6 * b), rv = arr(18 * b, b),
                              mv = arr(19 * b, b), iv = arr(21 * b, 3 * b);
    const size_t p0 = 42 * b;
    const std::vector<double> px = arr(p0, 3 * (size_t)h.np), pn = arr(p0 + 3 * (size_t)h.np, 3 * (size_t)h.np);
    rc = sphere3d_upload_impl(ctx, h.nb, qv.data(), vv.data(), rv.data(), mv.data(), iv.data(), h.np, px.data(),
                              pn.data());
  }
  if (rc != SG_OK) return rc;
  size_t off = 0;
  for (const CkptPart& part : ckpt_parts(ctx, h.dim, h.nb, h.np, h.prev_n)) {
    if (int r = grow(*part.buf, std::max<size_t>(part.bytes, 16))) return r;
    if (part.bytes)
      SG_CUDA_TRY(cudaMemcpyAsync(part.buf->p, in + off, part.bytes, cudaMemcpyHostToDevice, ctx->stream));
    off += part.bytes;
  }
  ctx->prev_n = h.prev_n;
  ctx->prev_rows = false;
  ctx->prev_color_valid = h.dim == 2 && h.prev_n > 0;
  ctx->last_nc = 0;
  ctx->staggering = h.staggering;
  ctx->stabilize = h.stabilize;
  ctx->pen_thresh = h.pen_thresh;
  SG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SG_OK;
}

int sg_set_staggering(sg_ctx* ctx, int32_t staggering, int32_t stabilize, double penetration_threshold) {
  if (!ctx || staggering < SG_STAGGER_GEOMETRIC || staggering > SG_STAGGER_STABILIZED ||
      !(penetration_threshold >= 0.0)) {
    set_error("sg_set_staggering: staggering SG_STAGGER_GEOMETRIC, _SYMPLECTIC_EULER or _STABILIZED, threshold >= 0");
    return SG_BAD_INPUT;
  }
  if (staggering == SG_STAGGER_STABILIZED && ctx->cfg.cache_mode != SG_CACHE_NONE) {
    set_error("sg_set_staggering: the stabilized staggering keeps no impulse cache (cache_mode NONE)");
    return SG_BAD_INPUT;
  }
  if (staggering == SG_STAGGER_SYMPLECTIC_EULER && ctx->cfg.CoR != 0.0) {
    set_error("sg_set_staggering: the symplectic Euler staggering needs CoR = 0");
    return SG_BAD_INPUT;
  }
  ctx->staggering = staggering;
  ctx->stabilize = stabilize != 0;
  ctx->pen_thresh = penetration_threshold;
  return SG_OK;
}

// ---------------------------------------------------------------------------
// Tuning of the launch-independent performance knobs (no counterpart in the reference).
int sg_get_tuning(sg_ctx* ctx, sg_tuning* t) {
  if (!ctx || !t) return SG_BAD_INPUT;
  t->two_level = ctx->patches;
  t->check_interval = ctx->check_interval;
  t->two_level_min_contacts = ctx->two_level_min_contacts;
  t->fp64_factor = ctx->fp64_factor;
  return SG_OK;
}

int sg_set_tuning(sg_ctx* ctx, const sg_tuning* t) {
  if (!ctx || !t || t->two_level < 0 || t->two_level > 2 || t->check_interval < 1 || t->check_interval > 4096 ||
      t->two_level_min_contacts < 0 || t->fp64_factor < 0) {
    set_error("sg_set_tuning: two_level in [0, 2], check_interval in [1, 4096], two_level_min_contacts >= 0, "
              "fp64_factor >= 0");
    return SG_BAD_INPUT;
  }
  ctx->patches = t->two_level;
  ctx->check_interval = t->check_interval;
  ctx->two_level_min_contacts = t->two_level_min_contacts;
  ctx->fp64_factor = t->fp64_factor;
  return SG_OK;
}

int sg_autotune(sg_ctx* ctx, int32_t trial_steps, uint32_t first_iteration, sg_tuning* best, double* ms_per_step) {
  if (!ctx || trial_steps < 1 || !ckpt_supported(ctx)) {
    set_error("sg_autotune: needs a context holding one Ball2D or sphere scene and trial_steps >= 1");
    return SG_BAD_INPUT;
  }
  const int64_t n = sg_checkpoint_size(ctx);
  if (n < 0) return SG_BAD_INPUT;
  std::vector<char> ck((size_t)n);
  if (int r = sg_checkpoint_save(ctx, ck.data(), n)) return r;
  sg_tuning cur;
  sg_get_tuning(ctx, &cur);
  // Candidates: two-level on/off x check interval 8/16/32.  The check interval acts only in
  // the FP32 form; the two-level sweeps only on single Ball2D scenes in the FP32 form.
  const bool fp32 = ctx->cfg.precision == SG_PRECISION_FP32_REFINE;
  const bool two_level_applies = fp32 && ctx->dim == 2;
  const int intervals[3] = {8, 16, 32};
  sg_tuning cand[6];
  bool use[6];
  for (int i = 0; i < 6; ++i) {
    cand[i] = cur;
    cand[i].two_level = i < 3 ? 1 : 0;
    cand[i].check_interval = intervals[i % 3];
    use[i] = fp32 && (two_level_applies || i < 3);
    if (ms_per_step) ms_per_step[i] = std::numeric_limits<double>::quiet_NaN();
  }
  if (!fp32) {  // nothing to choose: one timing of the current settings
    cand[0] = cur;
    use[0] = true;
  }
  auto run = [&](const sg_tuning& t, double* ms) -> int {
    if (int r = sg_checkpoint_load(ctx, ck.data(), n)) return r;
    sg_set_tuning(ctx, &t);
    const auto t0 = std::chrono::steady_clock::now();
    const int r = sg_step(ctx, first_iteration, (uint32_t)trial_steps, nullptr, nullptr);
    const auto t1 = std::chrono::steady_clock::now();
    if (r != SG_OK && r != SG_NOT_CONVERGED) return r;
    if (ms) *ms = std::chrono::duration<double, std::milli>(t1 - t0).count() / trial_steps;
    return SG_OK;
  };
  int rc = run(cur, nullptr);  // warm-up: first-use allocations and attributes
  int chosen = -1;
  double best_ms = std::numeric_limits<double>::infinity();
  for (int i = 0; i < 6 && rc == SG_OK; ++i) {
    if (!use[i]) continue;
    double ms = 0.0;
    rc = run(cand[i], &ms);
    if (rc != SG_OK) break;
    if (ms_per_step) ms_per_step[i] = ms;
    // A later candidate replaces an earlier one only when 3 % faster: on steps that every candidate
    // solves alike (a settled scene converging in the first FP64 sweeps) the differences are timing
    // noise, and the earlier candidates (two-level on) are the ones that pay on the hard steps.
    if (chosen < 0 || ms < 0.97 * best_ms) {
      best_ms = ms;
      chosen = i;
    }
  }
  // The state the tuning started from, with the fastest settings (or the old ones on failure).
  const int lr = sg_checkpoint_load(ctx, ck.data(), n);
  sg_set_tuning(ctx, rc == SG_OK && chosen >= 0 ? &cand[chosen] : &cur);
  if (best) sg_get_tuning(ctx, best);
  return rc != SG_OK ? rc : lr;
}

int sg_set_two_level(sg_ctx* ctx, int32_t on) {
  if (!ctx || on < 0 || on > 2) {
    set_error("sg_set_two_level: 0 (off), 1 (FP32 sweeps) or 2 (also the FP64 continuation)");
    return SG_BAD_INPUT;
  }
  ctx->patches = on;
  return SG_OK;
}

int sg_set_fp64_pairs(sg_ctx* ctx, int32_t on) {
  if (!ctx || on < 0 || on > 1) {
    set_error("sg_set_fp64_pairs: 0 (FP64 arithmetic) or 1 (float-float pairs)");
    return SG_BAD_INPUT;
  }
  ctx->fp64_pairs = on != 0;
  return SG_OK;
}

int sg_ctx_stream(sg_ctx* ctx, void** stream) {
  if (!ctx || !stream) return SG_BAD_INPUT;
  *stream = (void*)ctx->stream;
  return SG_OK;
}

int sg_profile_enable(sg_ctx* ctx, int32_t on) {
  if (!ctx) return SG_BAD_INPUT;
  SG_CUDA_TRY(cudaSetDevice(ctx->device));
  if (on && !ctx->ev_gs0) {
    SG_CUDA_TRY(cudaEventCreate(&ctx->ev_gs0));
    SG_CUDA_TRY(cudaEventCreate(&ctx->ev_gs1));
    for (cudaEvent_t& e : ctx->ev_stage) SG_CUDA_TRY(cudaEventCreate(&e));
  }
  ctx->profile = on != 0;
  return SG_OK;
}

int sg_profile_read(sg_ctx* ctx, sg_profile* out, int32_t reset) {
  if (!ctx || !out) return SG_BAD_INPUT;
  out->gs_ms = ctx->gs_ms;
  out->gs_launches = ctx->gs_launches;
  out->contact_sweeps = ctx->contact_sweeps;
  out->contact_evals = ctx->contact_evals;
  out->kernel_launches = ctx->kernel_launches;
  out->steps = ctx->steps;
  out->contacts = ctx->contacts_total;
  out->contact_sweeps32 = ctx->contact_sweeps32;
  out->contact_lifts = ctx->contact_lifts;
  out->body_lifts = ctx->body_lifts;
  out->two_level_solves = ctx->patched_solves;
  out->patch_interior_ms = 1e-6 * (double)ctx->patch_phase_ns[0];
  out->patch_wait_ms = 1e-6 * (double)ctx->patch_phase_ns[1];
  out->patch_boundary_ms = 1e-6 * (double)ctx->patch_phase_ns[2];
  out->boundary_contacts = ctx->patch_boundary_contacts;
  out->boundary_colors = ctx->patch_boundary_colors;
  out->patch_interior_max_ms = 1e-6 * (double)ctx->patch_interior_max_ns;
  out->patch_slowest_block = ctx->patch_slowest_block;
  out->patch_contacts_staged = ctx->patch_staged;
  out->fp64_start_solves = ctx->fp64_start_solves;
  for (int k = 0; k < 8; ++k) out->stage_ms[k] = ctx->stage_ms[k];
  if (reset) {
    for (double& x : ctx->stage_ms) x = 0.0;
    ctx->patched_solves = 0;
    ctx->fp64_start_solves = 0;
    ctx->patch_phase_ns[0] = ctx->patch_phase_ns[1] = ctx->patch_phase_ns[2] = 0;
    ctx->patch_boundary_contacts = ctx->patch_boundary_colors = 0;
    ctx->patch_interior_max_ns = 0;
    ctx->patch_staged = 0;
    ctx->gs_ms = 0.0;
    ctx->gs_launches = ctx->contact_sweeps = ctx->contact_evals = ctx->kernel_launches = 0;
    ctx->steps = ctx->contacts_total = 0;
    ctx->contact_sweeps32 = ctx->contact_lifts = ctx->body_lifts = 0;
  }
  return SG_OK;
}

int sg_set_spin_limit(sg_ctx* ctx, uint64_t spins) {
  if (!ctx) return SG_BAD_INPUT;
  ctx->spin_limit = spins ? (unsigned long long)spins : kDefaultSpin;
  return SG_OK;
}

int sg_selftest_wait_timeout(sg_ctx* ctx) {
  if (!ctx) return SG_BAD_INPUT;
  SG_CUDA_TRY(cudaSetDevice(ctx->device));
  return wait_timeout_selftest(ctx);
}

}  // extern "C"
