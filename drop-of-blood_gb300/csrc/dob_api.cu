// dob_api.cu — the C ABI (include/dropfluid.h): context lifetime, device
// memory, host<->device field I/O, step orchestration on one CUDA stream
// with captured CUDA graphs, statistics and timing.
//
// A step is the reference's encodePhysicsStep (BloodDropEngine.ts:1855-2111)
// minus the wave and lighting passes: advect -> centre -> [curl] -> Casson/
// forces -> divergence -> V-cycles -> project -> centre -> clear splats ->
// parcel emit -> parcel advect/splat -> dye predict -> dye resolve.  In the
// closed box nothing reads the centre velocity between advection and the
// projection (no curl), so that centre pass is left out, the projection and
// the following centre pass run as one kernel, and Casson, divergence and
// projection use the z-column kernels of k_box.cu (same bits as the general
// kernels the stage-level interface runs).  The stage sequence is
// captured once into a CUDA graph per (dye, velocity) ping-pong state and
// replayed; the per-step parameters reach the device by one 592-byte copy
// from a pinned ring before each replay.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "dob_kernels.cuh"

using namespace dob;

#include "dob_ctx.h"

static const char* g_static_err = "no error";

#define CK(call)                                                               \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess) return fail(ctx, DOB_ECUDA, #call, cudaGetErrorString(e_)); \
  } while (0)

static dob_status fail(dob_ctx* ctx, dob_status st, const char* what, const char* detail) {
  if (ctx) {
    ctx->err = std::string(what) + ": " + (detail ? detail : "");
  } else {
    static thread_local std::string msg;
    msg = std::string(what) + ": " + (detail ? detail : "");
    g_static_err = msg.c_str();
  }
  return st;
}

dob_status dob::record_error(dob_ctx* ctx, dob_status st, const char* what, const char* detail) {
  return fail(ctx, st, what, detail);
}

static size_t vs_bytes(int prec) { return prec == DOB_PREC_REFERENCE_FP16 ? 2 : 4; }
static size_t ds_bytes(int prec) { return prec == DOB_PREC_FP32 ? 4 : 2; }

static bool valid_config(const dob_config* c, std::string* why) {
  auto no = [&](const char* m) { *why = m; return false; };
  if (!c) return no("null config");
  if (c->struct_size != sizeof(dob_config)) return no("struct_size mismatch");
  if (c->nx < 4 || c->ny < 4 || c->nz < 4) return no("grid dims must be >= 4");
  if (c->nx > 2048 || c->ny > 2048 || c->nz > 2048) return no("grid dims must be <= 2048");
  if (c->nx % 2 || c->ny % 2 || c->nz % 2) return no("grid dims must be even");
  if (c->dye_refine != 1 && c->dye_refine != 2) return no("dye_refine must be 1 or 2");
  const uint64_t r3 = (uint64_t)c->dye_refine * c->dye_refine * c->dye_refine;
  if ((uint64_t)c->nx * c->ny * c->nz * r3 >= (1ull << 31)) return no("grid too large (the dye grid must have < 2^31 cells)");
  if (c->mg_levels < 1 || c->mg_levels > kMaxLevels) return no("mg_levels out of range");
  // every grid of the hierarchy has even dims (red-black split rows)
  const uint32_t m = 1u << c->mg_levels;
  if (c->nx % m || c->ny % m || c->nz % m)
    return no("dims not divisible by 2^mg_levels (every multigrid level needs even dims)");
  if (c->bc_mode != DOB_BC_REFERENCE && c->bc_mode != DOB_BC_CLOSED_BOX) return no("bad bc_mode");
  if (c->precision_mode < 0 || c->precision_mode > 2) return no("bad precision_mode");
  if (c->mg_pre < 0 || c->mg_post < 0 || c->mg_coarse_sweeps < -1 || c->mg_cycles < 0) return no("negative sweeps");
  if (c->mg_coarse_sweeps == -1) {
    const uint64_t cc = (uint64_t)(c->nx >> (c->mg_levels - 1)) * (c->ny >> (c->mg_levels - 1)) *
                        (c->nz >> (c->mg_levels - 1));
    if (cc > (uint64_t)kDenseCoarseMax)
      return no("mg_coarse_sweeps = -1 (exact coarsest solve) needs a coarsest grid of at most 4096 cells");
  }
  if (c->precision_mode == DOB_PREC_MIXED && (c->mg_max_outer < 1 || c->mg_max_outer > 32)) return no("mg_max_outer must be 1..32");
  if (c->precision_mode == DOB_PREC_MIXED && c->mg_levels < 2) return no("the mixed mode needs at least 2 grids");
  if (!(c->mg_rel_tol >= 0.0) || !(c->mg_div_tol >= 0.0) || !isfinite(c->mg_rel_tol) || !isfinite(c->mg_div_tol))
    return no("mg_rel_tol and mg_div_tol must be finite and >= 0");
  if (c->parcel_capacity < 1 || c->parcel_capacity > (1u << 26)) return no("parcel_capacity out of range");
  if (c->mg_cycles_injected < 0 || c->mg_cycles_injected > 64) return no("mg_cycles_injected must be 0..64");
  if (c->bc_mode == DOB_BC_CLOSED_BOX) {
    if (!(c->dt > 0.0f) || !isfinite(c->dt)) return no("dt must be finite and > 0");
    if (!(c->dx > 0.0f) || !isfinite(c->dx)) return no("dx must be finite and > 0");
    for (int k = 0; k < 3; ++k)
      if (!(c->domain_max[k] > c->domain_min[k])) return no("empty domain");
  }
  return true;
}

static void default_uniforms(float* U) {
  memset(U, 0, 128 * sizeof(float));
  U[36] = 1.0f; U[37] = 1.0f; U[38] = 1.0f / 60.0f;
  U[40] = 0.30f; U[41] = 1.0f; U[43] = 1.0f;
  U[44] = 1.02f; U[45] = 0.48f; U[46] = 0.9993f; U[47] = 0.995f;
  U[48] = 1.0f; U[49] = 1.0f; U[50] = 1.0f;
  U[52] = 0.48f; U[53] = -0.98f; U[54] = 0.30f; U[55] = 1.10f;
  U[57] = 0.0032f; U[58] = 1.0f; U[59] = 0.088f;
  U[60] = 0.032f; U[63] = 0.028f;
}

static dob_status dev_alloc(dob_ctx* ctx, void** p, size_t bytes) {
  *p = nullptr;
  if (bytes == 0) return DOB_OK;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, DOB_ENOMEM, "cudaMalloc", cudaGetErrorString(e));
  }
  ctx->allocs.push_back(*p);
  ctx->bytes += bytes;
  return DOB_OK;
}

// Fill the step parameters for the next step (host) from the uniform block or
// the closed-box configuration.
static void fill_params(dob_ctx* ctx, StepParams* P, uint32_t spawn) {
  const dob_config& c = ctx->cfg;
  memcpy(P->U, ctx->U, sizeof(P->U));
  if (c.bc_mode == DOB_BC_REFERENCE) {
    const float dtr = ctx->U[38];
    P->dt = dob_clampf(dtr, 0.0f, 0.025f);
    P->dmin[0] = -ctx->U[52]; P->dmin[1] = ctx->U[53]; P->dmin[2] = -ctx->U[52];
    P->dmax[0] = ctx->U[52]; P->dmax[1] = ctx->U[54]; P->dmax[2] = ctx->U[52];
    P->damp = ctx->U[46];
    P->sharp = ctx->U[47];
  } else {
    P->dt = c.dt;
    for (int k = 0; k < 3; ++k) { P->dmin[k] = c.domain_min[k]; P->dmax[k] = c.domain_max[k]; }
    P->damp = c.vel_damping;
    P->sharp = c.dye_sharpness;
  }
  for (int k = 0; k < 3; ++k) {
    P->dsize[k] = P->dmax[k] - P->dmin[k];
    P->rdsize[k] = 1.0f / P->dsize[k];
  }
  P->tau_y = c.casson_tau_y;
  P->mu_p = c.casson_mu_p;
  P->dx = c.dx;
  P->spawn_count = spawn;
  const float cur = ctx->U[61] > 0.0f ? ctx->U[61] : 0.0f;
  P->cursor = (uint32_t)cur;
  P->high_water = ctx->high_water;
  const uint64_t hw = ((uint64_t)ctx->high_water + 255u) / 256u * 256u;
  P->advect_count = (uint32_t)(hw < ctx->s.cap ? hw : ctx->s.cap);
  P->step_index = ctx->step_index;
}

static uint32_t spawn_count(const dob_ctx* ctx) {
  if (ctx->cfg.bc_mode != DOB_BC_REFERENCE) return 0u;
  const float sc = ctx->U[62] > 0.0f ? ctx->U[62] : 0.0f;
  uint32_t n = (uint32_t)sc;
  if (n > 8192u) n = 8192u;  // the emit dispatch covers at most 8192 parcels (BloodDropEngine.ts:1835)
  return n > ctx->s.cap ? ctx->s.cap : n;
}

// Copy the step parameters to the device (pinned ring slot + event guard).
static dob_status upload_params(dob_ctx* ctx, uint32_t spawn) {
  const int k = ctx->param_slot;
  ctx->param_slot = (k + 1) % kParamRing;
  CK(cudaEventSynchronize(ctx->param_ev[k]));
  fill_params(ctx, &ctx->host_params[k], spawn);
  CK(cudaMemcpyAsync(ctx->s.params, &ctx->host_params[k], sizeof(StepParams), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaEventRecord(ctx->param_ev[k], ctx->stream));
  return DOB_OK;
}

static void swap_vel(DevState& s) {
  std::swap(s.u, s.u2);
  std::swap(s.v, s.v2);
  std::swap(s.w, s.w2);
}

// Enqueue one stage on the context's stream, updating the ping-pong state.
// in_step: the stage runs inside a full step, after the projection and the
// centre pass (the dye stages may then skip clear water, see k_fluid.cu).
static void enqueue_stage(dob_ctx* ctx, DevState& s, int stage, cudaStream_t st, bool in_step = false) {
  const size_t nc = s.gc.n();
  switch (stage) {
    case DOB_STAGE_ADVECT_MAC: launch_advect_mac(s, st); swap_vel(s); break;
    case DOB_STAGE_MAC_TO_CENTER: launch_mac_to_center(s, st); break;
    case DOB_STAGE_CURL: if (s.curl) launch_curl(s, st); break;
    case DOB_STAGE_CASSON_FORCES: launch_casson(s, st); swap_vel(s); break;
    case DOB_STAGE_MAC_RHS: launch_mac_rhs(s, st); break;
    case DOB_STAGE_PRESSURE_SOLVE: launch_pressure_solve(s, st); break;
    case DOB_STAGE_PROJECT: launch_project(s, st); break;
    case DOB_STAGE_CLEAR_SPLATS: launch_clear_splats(s, st); break;
    case DOB_STAGE_PARCEL_EMIT: launch_parcel_emit(s, st); break;
    case DOB_STAGE_PARCEL_ADVECT: launch_parcel_advect(s, st); break;
    case DOB_STAGE_CONC_PREDICT: launch_conc_predict(s, st, false, in_step); break;
    case DOB_STAGE_CONC_RESOLVE: launch_conc_resolve(s, st, in_step); std::swap(s.conc, s.conc2); break;
    default: break;
  }
  (void)ctx;
}

static const int kStepOrder[] = {
    DOB_STAGE_ADVECT_MAC, DOB_STAGE_MAC_TO_CENTER, DOB_STAGE_CURL,          DOB_STAGE_CASSON_FORCES,
    DOB_STAGE_MAC_RHS,    DOB_STAGE_PRESSURE_SOLVE, DOB_STAGE_PROJECT,      DOB_STAGE_MAC_TO_CENTER,
    DOB_STAGE_CLEAR_SPLATS, DOB_STAGE_PARCEL_EMIT, DOB_STAGE_PARCEL_ADVECT, DOB_STAGE_CONC_PREDICT,
    DOB_STAGE_CONC_RESOLVE};

static void enqueue_step_body(dob_ctx* ctx, DevState& s, cudaStream_t st, float* stage_ms, bool stats_div) {
  const int n = (int)(sizeof(kStepOrder) / sizeof(kStepOrder[0]));
  // the wave substep comes first and the advection reads its result
  // (BloodDropEngine.ts:1886-1912)
  if (s.flags & DOB_PHYS_WAVE) launch_wave_step(s, st);
  bool centre_fused = false;  // reference mode: the projection has formed the centre velocity
  for (int k = 0; k < n; ++k) {
    const int stage = kStepOrder[k];
    if (centre_fused && stage == DOB_STAGE_MAC_TO_CENTER) continue;
    if (stage == DOB_STAGE_CURL && !(s.ref && (s.flags & DOB_PHYS_VORT_CONF))) continue;
    // closed box: the centre after advection has no reader, and the centre
    // after the projection comes out of the fused projection kernel
    if (!s.ref && stage == DOB_STAGE_MAC_TO_CENTER) continue;
    if (stage_ms) cudaEventRecord(ctx->stage_ev[0], st);
    if (!s.ref && stage == DOB_STAGE_PROJECT) {
      // with statistics the projection also forms max |div| (no separate
      // pass), and always the bound on the centre velocity that lets the
      // predictor skip blocks that cannot reach dye
      if (stats_div) cudaMemsetAsync(s.redu + REDU_MAXDIV, 0, sizeof(unsigned int), st);
      cudaMemsetAsync(s.redu + REDU_SPEED, 0, sizeof(unsigned int), st);
      launch_project_center_box(s, st, ctx->cfg.dt / ctx->cfg.dx, stats_div ? s.redu + REDU_MAXDIV : nullptr,
                                s.redu + REDU_SPEED);
      swap_vel(s);
    } else if (s.ref && stage == DOB_STAGE_PROJECT) {
      // the projection and the centre velocity after it in one pass
      launch_project_center_ref(s, st);
      swap_vel(s);
      centre_fused = true;
    } else if (!s.ref && stage == DOB_STAGE_MAC_RHS) {
      // with statistics the mean removal also forms ||rhs||^2
      if (stats_div) cudaMemsetAsync(s.red + RED_RHS_NORM2, 0, sizeof(double), st);
      launch_mac_rhs_box(s, st, stats_div ? s.red + RED_RHS_NORM2 : nullptr);
    } else if (stage == DOB_STAGE_CASSON_FORCES && box_casson_applies(s)) {
      launch_casson_box(s, st);
      swap_vel(s);
    } else if (!s.ref && stage == DOB_STAGE_CONC_PREDICT) {
      // closed box: the predictor brackets its taps for the resolve, which
      // then traces only the forward sample; both skip clear water
      launch_conc_predict(s, st, true, true);
    } else if (!s.ref && stage == DOB_STAGE_CONC_RESOLVE) {
      launch_dye_resolve_lim(s, st);
      std::swap(s.conc, s.conc2);
    } else {
      enqueue_stage(ctx, s, stage, st, true);
    }
    if (stage_ms) {
      cudaEventRecord(ctx->stage_ev[1], st);
      cudaEventSynchronize(ctx->stage_ev[1]);
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, ctx->stage_ev[0], ctx->stage_ev[1]);
      stage_ms[stage] += ms;
    }
    if (stats_div && stage == DOB_STAGE_MAC_RHS && s.ref) {
      cudaMemsetAsync(s.red + RED_RHS_NORM2, 0, sizeof(double), st);
      launch_sumsq(s.rhs, s.g.n(), s.red + RED_RHS_NORM2, s.num_sms, st);
    }
    if (stats_div && stage == DOB_STAGE_PRESSURE_SOLVE && (ctx->stats_mask & DOB_STATS_RESIDUAL)) {
      launch_residual_norm(s, s.red + RED_RES_NORM2, st);
    }
    if (stats_div && stage == DOB_STAGE_PROJECT && s.ref) {
      const float scale = s.ref ? 1.0f : ctx->cfg.dt / ctx->cfg.dx;
      cudaMemsetAsync(s.redu + REDU_MAXDIV, 0, sizeof(unsigned int), st);
      launch_divergence(s, nullptr, scale, s.redu + REDU_MAXDIV, st);
    }
  }
}

// Graphs are cached per (statistics on/off, dye and velocity buffers at the
// step's start).
static void pingpong_get(const DevState& s, void** out) {
  out[0] = s.u; out[1] = s.v; out[2] = s.w; out[3] = s.u2; out[4] = s.v2; out[5] = s.w2;
  out[6] = s.conc; out[7] = s.conc2;
}
static void pingpong_set(DevState& s, void* const* in) {
  s.u = in[0]; s.v = in[1]; s.w = in[2]; s.u2 = in[3]; s.v2 = in[4]; s.w2 = in[5];
  s.conc = in[6]; s.conc2 = in[7];
}

static dob_status get_graph(dob_ctx* ctx, bool stats, bool injected, dob_ctx::StepGraph** out) {
  const int nslots = (int)(sizeof(ctx->graphs) / sizeof(ctx->graphs[0]));
  int slot = -1;
  for (int k = 0; k < nslots; ++k) {
    dob_ctx::StepGraph& G = ctx->graphs[k];
    if (G.ex && G.stats == stats && G.injected == injected && G.conc == ctx->s.conc && G.u == ctx->s.u) {
      *out = &G;
      return DOB_OK;
    }
    if (!G.ex && slot < 0) slot = k;
  }
  if (slot < 0) {
    slot = ctx->graph_next;
    ctx->graph_next = (slot + 1) % nslots;
    cudaGraphExecDestroy(ctx->graphs[slot].ex);
    ctx->graphs[slot].ex = nullptr;
  }
  DevState s = ctx->s;
  if (injected) s.cycles = ctx->cfg.mg_cycles_injected;
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  enqueue_step_body(ctx, s, ctx->stream, nullptr, stats);
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
  if (e != cudaSuccess) return fail(ctx, DOB_ECUDA, "cudaStreamEndCapture", cudaGetErrorString(e));
  size_t nn = 0;
  cudaGraphGetNodes(g, nullptr, &nn);
  std::vector<cudaGraphNode_t> nodes(nn);
  if (nn) cudaGraphGetNodes(g, nodes.data(), &nn);
  int kernels = 0;
  for (size_t k = 0; k < nn; ++k) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(nodes[k], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++kernels;
  }
  if (!stats) ctx->kernels_per_step = kernels;
  cudaGraphExec_t ex = nullptr;
  e = cudaGraphInstantiate(&ex, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(ctx, DOB_ECUDA, "cudaGraphInstantiate", cudaGetErrorString(e));
  dob_ctx::StepGraph& G = ctx->graphs[slot];
  G.ex = ex;
  G.stats = stats;
  G.injected = injected;
  G.conc = ctx->s.conc;
  G.u = ctx->s.u;
  pingpong_get(s, G.after);
  *out = &G;
  return DOB_OK;
}

static void drop_graphs(dob_ctx* ctx) {
  for (auto& G : ctx->graphs) {
    if (G.ex) cudaGraphExecDestroy(G.ex);
    G = dob_ctx::StepGraph();
  }
  ctx->graph_next = 0;
}

static dob_status one_step(dob_ctx* ctx, uint32_t flags, float* stage_ms) {
  const uint32_t spawn = spawn_count(ctx);
  if (ctx->cfg.bc_mode == DOB_BC_REFERENCE) {  // BloodDropEngine.ts:1832-1840
    const uint64_t hw = (uint64_t)ctx->high_water + spawn;
    ctx->high_water = (uint32_t)(hw < ctx->s.cap ? hw : ctx->s.cap);
  }
  dob_status st = upload_params(ctx, spawn);
  if (st != DOB_OK) return st;
  const bool stats = (flags & DOB_STEP_STATS) != 0;
  // the first kInjectedSteps steps after an injection run mg_cycles_injected
  // V-cycles (the mixed loop adapts by itself)
  const bool injected = ctx->inject_pending > 0 && ctx->cfg.mg_cycles_injected > 0 &&
                        ctx->cfg.precision_mode != DOB_PREC_MIXED && ctx->cfg.mg_cycles_injected != ctx->cfg.mg_cycles;
  if (ctx->inject_pending > 0) --ctx->inject_pending;
  ctx->last_cycles = injected ? ctx->cfg.mg_cycles_injected : ctx->cfg.mg_cycles;
  if (stage_ms || (flags & DOB_STEP_NO_GRAPH)) {
    const int cycles = ctx->s.cycles;
    if (injected) ctx->s.cycles = ctx->cfg.mg_cycles_injected;
    enqueue_step_body(ctx, ctx->s, ctx->stream, stage_ms, stats);
    ctx->s.cycles = cycles;
  } else {
    dob_ctx::StepGraph* G = nullptr;
    st = get_graph(ctx, stats, injected, &G);
    if (st != DOB_OK) return st;
    CK(cudaGraphLaunch(G->ex, ctx->stream));
    pingpong_set(ctx->s, G->after);  // the buffers the captured step wrote last
  }
  CK(cudaGetLastError());
  ctx->step_index++;
  return DOB_OK;
}

static void fill_stats(dob_ctx* ctx, const double* red, const unsigned int* redu, dob_step_stats* stats, int steps,
                       int cycles) {
  stats->struct_size = sizeof(dob_step_stats);
  stats->steps_done = steps;
  if (ctx->cfg.precision_mode == DOB_PREC_MIXED) {
    stats->outer_iters = (int)redu[REDU_ITERS];
    stats->vcycles = (int)redu[REDU_VCYCLES];
  } else {
    stats->outer_iters = 0;
    stats->vcycles = cycles;  // of the last step
  }
  stats->residual_l2 = (ctx->stats_mask & DOB_STATS_RESIDUAL) ? sqrt(red[RED_RES_NORM2]) : -1.0;
  stats->rhs_l2 = sqrt(red[RED_RHS_NORM2]);
  float md;
  memcpy(&md, &redu[REDU_MAXDIV], 4);
  stats->max_div = (double)md;
  stats->parcels_alive = (ctx->stats_mask & DOB_STATS_PARCELS) ? redu[REDU_ALIVE] : 0u;
}

static dob_status finish_stats(dob_ctx* ctx, dob_step_stats* stats, int steps) {
  if (!stats) return DOB_OK;
  DevState& s = ctx->s;
  double red[RED_COUNT];
  unsigned int redu[REDU_COUNT];
  if (ctx->stats_mask & DOB_STATS_PARCELS) launch_count_alive(s, s.redu + REDU_ALIVE, ctx->stream);
  CK(cudaMemcpyAsync(red, s.red, sizeof(red), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(redu, s.redu, sizeof(redu), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  fill_stats(ctx, red, redu, stats, steps, ctx->last_cycles);
  return DOB_OK;
}

extern "C" {

int dob_abi_version(void) { return DOB_ABI_VERSION; }

const char* dob_last_error(const dob_ctx* ctx) { return ctx ? ctx->err.c_str() : g_static_err; }

dob_status dob_config_reference(dob_config* c) {
  if (!c) return DOB_EINVAL;
  memset(c, 0, sizeof(*c));
  c->struct_size = sizeof(dob_config);
  c->nx = 96; c->ny = 128; c->nz = 96;
  c->dye_refine = 2;
  c->dx = 0.01f;
  c->dt = 1.0f / 60.0f;
  c->domain_min[0] = -0.48f; c->domain_min[1] = -0.98f; c->domain_min[2] = -0.48f;
  c->domain_max[0] = 0.48f; c->domain_max[1] = 0.30f; c->domain_max[2] = 0.48f;
  c->bc_mode = DOB_BC_REFERENCE;
  c->precision_mode = DOB_PREC_FP32;
  c->mg_levels = 4; c->mg_pre = 2; c->mg_post = 2; c->mg_coarse_sweeps = 6; c->mg_cycles = 1;
  c->mg_max_outer = 1; c->mg_rel_tol = 0.0; c->mg_div_tol = 0.0; c->mg_cycles_injected = 0;
  c->physics_flags = DOB_PHYS_REFERENCE_ALL;
  c->parcel_capacity = 393216;
  c->reference_schedule = 1;
  c->vel_damping = 1.0f;
  c->dye_sharpness = 1.0f;
  return DOB_OK;
}

dob_status dob_config_closed_box(dob_config* c, uint32_t nx, uint32_t ny, uint32_t nz) {
  if (!c) return DOB_EINVAL;
  memset(c, 0, sizeof(*c));
  c->struct_size = sizeof(dob_config);
  c->nx = nx; c->ny = ny; c->nz = nz;
  c->dye_refine = 1;
  c->dx = 1.0f;
  c->dt = 0.02f;
  c->domain_max[0] = (float)nx; c->domain_max[1] = (float)ny; c->domain_max[2] = (float)nz;
  c->bc_mode = DOB_BC_CLOSED_BOX;
  c->precision_mode = DOB_PREC_FP32;
  // the hierarchy is deepened until the coarsest grid has at most
  // kDenseCoarseTarget cells, which are solved exactly (dense inverse); 2+2
  // sweeps elsewhere
  int levels = 1, coarse = 6;
  for (int L = 2; L <= kMaxLevels; ++L) {
    const uint32_t m = 1u << L;
    if (nx % m || ny % m || nz % m) break;
    const uint64_t cells = (uint64_t)(nx >> (L - 1)) * (ny >> (L - 1)) * (nz >> (L - 1));
    levels = L;
    coarse = cells <= (uint64_t)kDenseCoarseMax ? -1 : 6;
    if (cells <= (uint64_t)kDenseCoarseTarget) break;
  }
  c->mg_levels = levels; c->mg_pre = 2; c->mg_post = 2; c->mg_coarse_sweeps = coarse; c->mg_cycles = 4;
  c->mg_max_outer = 16; c->mg_rel_tol = 0.0; c->mg_div_tol = 1e-5;
  c->casson_tau_y = 0.005f; c->casson_mu_p = 1e-3f;
  c->physics_flags = 0;
  c->parcel_capacity = 8192;
  c->reference_schedule = 0;
  c->vel_damping = 1.0f;
  c->dye_sharpness = 1.0f;
  // the step after a drop's injection: with 4 cycles the projection leaves
  // max |div| dt/dx up to 7.5e-5 on box192's release steps, with 8 <= 8.1e-6
  c->mg_cycles_injected = 2 * c->mg_cycles;
  return DOB_OK;
}

dob_status dob_create(const dob_config* cfg, dob_ctx** out) {
  if (!out) return fail(nullptr, DOB_EINVAL, "dob_create", "null out pointer");
  *out = nullptr;
  std::string why;
  if (!valid_config(cfg, &why)) return fail(nullptr, DOB_EINVAL, "dob_create", why.c_str());
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(nullptr, DOB_ECUDA, "dob_create", e != cudaSuccess ? cudaGetErrorString(e) : "no CUDA device");
  }
  dob_ctx* ctx = new dob_ctx();
  ctx->cfg = *cfg;
  default_uniforms(ctx->U);
  DevState& s = ctx->s;
  memset(&s, 0, sizeof(s));
  CK(cudaGetDevice(&ctx->device));
  CK(cudaDeviceGetAttribute(&s.num_sms, cudaDevAttrMultiProcessorCount, ctx->device));
  CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&ctx->aux_stream, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&ctx->aux_stream2, cudaStreamNonBlocking));
  CK(mg_prepare());
  s.aux = ctx->aux_stream;
  s.aux2 = ctx->aux_stream2;
  s.g = make_grid((int)cfg->nx, (int)cfg->ny, (int)cfg->nz);
  s.gc = make_grid((int)(cfg->nx * cfg->dye_refine), (int)(cfg->ny * cfg->dye_refine), (int)(cfg->nz * cfg->dye_refine));
  s.prec = cfg->precision_mode;
  s.ref = cfg->bc_mode == DOB_BC_REFERENCE;
  s.flags = s.ref ? cfg->physics_flags : 0;
  s.cap = cfg->parcel_capacity;
  const size_t N = s.g.n(), Nc = s.gc.n();
  const size_t vsb = vs_bytes(s.prec), dsb = ds_bytes(s.prec);
  dob_status st = DOB_OK;
  auto A = [&](void** p, size_t b) { if (st == DOB_OK) st = dev_alloc(ctx, p, b); };
  A((void**)&s.params, sizeof(StepParams));
  A(&s.u, N * vsb); A(&s.v, N * vsb); A(&s.w, N * vsb);
  A(&s.u2, N * vsb); A(&s.v2, N * vsb); A(&s.w2, N * vsb);
  A(&s.cen, N * 4 * vsb);
  if (s.ref) A(&s.curl, N * 4 * vsb);
  A((void**)&s.p, N * 4); A((void**)&s.rhs, N * 4);
  const int nch = s.ref ? 4 : 1;
  A(&s.conc, Nc * nch * dsb); A(&s.conc2, Nc * nch * dsb); A(&s.pred, Nc * dsb);
  s.concA = s.conc;
  s.concB = s.conc2;
  {
    const size_t nb = dye_brick_count(s.gc) * sizeof(uint32_t);
    A((void**)&s.cbrickA, nb); A((void**)&s.cbrickB, nb); A((void**)&s.sbrick, nb);
    if (s.ref) A((void**)&s.pbrick, nb);
  }
  if (!s.ref) A(&s.lim, Nc * 2 * dsb);
  A((void**)&s.splatI, Nc * 4); A((void**)&s.splatL, Nc * 4);
  A((void**)&s.wave, (size_t)kWaveN * kWaveN * 16);
  if (s.flags & DOB_PHYS_WAVE) {
    A((void**)&s.wspec, (size_t)kWaveN * kWaveN * 8);
    A((void**)&s.wfilm, (size_t)kWaveN * kWaveN * 4);
  }
  A((void**)&s.parcels, (size_t)s.cap * 32);
  if (s.ref && light_dims_ok(s.g)) {
    A((void**)&s.light, N * sizeof(half4));
    A((void**)&s.brick_raw, N / 64 * sizeof(float));
    A((void**)&s.bricks, N / 64 * sizeof(float));
  }
  // the FP64 and u32 reduction slots in one block, so the statistics a
  // pipelined step reads back are one copy
  A((void**)&s.red, kStatsBytes);
  if (st == DOB_OK) s.redu = reinterpret_cast<unsigned int*>(s.red + RED_COUNT);
  A((void**)&s.part, PART_SLOTS * kSumBlocks * sizeof(double));
  s.nlev = cfg->mg_levels;
  for (int l = 0; l < s.nlev; ++l) {
    MgLevel& L = s.lv[l];
    L.d = make_grid(s.g.nx >> l, s.g.ny >> l, s.g.nz >> l);
    const float sc = (float)s.g.nx / (float)L.d.nx;
    L.h2 = sc * sc;
    if (l == 0) { L.e = s.p; L.b = s.rhs; continue; }
    if (s.prec == DOB_PREC_MIXED && l >= kMixedBF16Level) {
      A((void**)&L.eh, L.d.n() * 2); A((void**)&L.bh, L.d.n() * 2);
    } else {
      A((void**)&L.e, L.d.n() * 4); A((void**)&L.b, L.d.n() * 4);
    }
  }
  if (s.prec == DOB_PREC_MIXED) {
    A((void**)&s.plo, N * 4); A((void**)&s.e0, N * 4); A((void**)&s.r0, N * 4);
  }
  if (cfg->mg_coarse_sweeps < 0 && st == DOB_OK) {
    const MgLevel& C = s.lv[s.nlev - 1];
    const std::vector<float> inv = coarse_inverse(C.d, C.h2, s.ref);
    float* d = nullptr;
    A((void**)&d, inv.size() * sizeof(float));
    if (st == DOB_OK) {
      cudaError_t ce = cudaMemcpy(d, inv.data(), inv.size() * sizeof(float), cudaMemcpyHostToDevice);
      if (ce != cudaSuccess) st = fail(ctx, DOB_ECUDA, "coarse inverse upload", cudaGetErrorString(ce));
    }
    s.cinv = d;
    s.cn = (int)C.d.n();
  }
  s.pre0 = cfg->reference_schedule ? 1 : cfg->mg_pre;
  s.post0 = cfg->reference_schedule ? 1 : cfg->mg_post;
  s.pre = cfg->mg_pre; s.post = cfg->mg_post;
  s.coarse_sweeps = cfg->mg_coarse_sweeps;
  s.cycles = cfg->mg_cycles;
  s.max_outer = cfg->mg_max_outer;
  s.rel_tol = cfg->mg_rel_tol;
  // max |b - A p| target: the projected divergence is b - A p, reported as
  // max |div| dt/dx in the closed box and unscaled in reference mode
  s.div_tol_r = (float)(s.ref ? cfg->mg_div_tol : cfg->mg_div_tol * cfg->dx / cfg->dt);
  // the mixed solve stops at 0.9 of the divergence target: the projection
  // that follows adds its own FP32 rounding to the divergence it leaves
  if (s.prec == DOB_PREC_MIXED) s.div_tol_r *= 0.9f;
  if (st != DOB_OK) {
    *out = nullptr;
    std::string keep = ctx->err;
    dob_destroy(ctx);
    return fail(nullptr, st, "dob_create", keep.c_str());
  }
  cudaError_t eh = cudaMallocHost((void**)&ctx->host_params, sizeof(StepParams) * kParamRing);
  if (eh != cudaSuccess) {
    dob_destroy(ctx);
    return fail(nullptr, DOB_ENOMEM, "cudaMallocHost", cudaGetErrorString(eh));
  }
  for (int k = 0; k < kParamRing; ++k) CK(cudaEventCreateWithFlags(&ctx->param_ev[k], cudaEventDisableTiming));
  CK(cudaEventCreate(&ctx->ev0));
  CK(cudaEventCreate(&ctx->ev1));
  for (int k = 0; k <= DOB_STAGE_COUNT; ++k) CK(cudaEventCreate(&ctx->stage_ev[k]));
  CK(cudaMemsetAsync(s.wave, 0, (size_t)kWaveN * kWaveN * 16, ctx->stream));
  dob_status r = dob_reset(ctx);
  if (r != DOB_OK) {
    std::string keep = ctx->err;
    dob_destroy(ctx);
    return fail(nullptr, r, "dob_create/reset", keep.c_str());
  }
  *out = ctx;
  return DOB_OK;
}

void dob_destroy(dob_ctx* ctx) {
  if (!ctx) return;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  drop_graphs(ctx);
  adjoint_free(ctx);
  for (auto& sn : ctx->snaps)
    for (void* p : sn.bufs) cudaFree(p);
  for (void* p : ctx->allocs) cudaFree(p);
  if (ctx->lut) cudaFree(ctx->lut);
  if (ctx->image) cudaFree(ctx->image);
  if (ctx->host_params) cudaFreeHost(ctx->host_params);
  for (int k = 0; k < kParamRing; ++k)
    if (ctx->param_ev[k]) cudaEventDestroy(ctx->param_ev[k]);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  for (int k = 0; k <= DOB_STAGE_COUNT; ++k)
    if (ctx->stage_ev[k]) cudaEventDestroy(ctx->stage_ev[k]);
  for (auto& a : ctx->async_slots) {
    if (a.red) cudaFreeHost(a.red);  // a.redu lies in the same block
    if (a.done) cudaEventDestroy(a.done);
  }
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  if (ctx->aux_stream) cudaStreamDestroy(ctx->aux_stream);
  if (ctx->aux_stream2) cudaStreamDestroy(ctx->aux_stream2);
  delete ctx;
}

dob_status dob_reset(dob_ctx* ctx) {
  if (!ctx) return DOB_EINVAL;
  DevState& s = ctx->s;
  const size_t N = s.g.n(), Nc = s.gc.n();
  const size_t vsb = vs_bytes(s.prec), dsb = ds_bytes(s.prec);
  const int nch = s.ref ? 4 : 1;
  ctx->high_water = 0;
  ctx->inject_pending = 0;
  ctx->step_index = 0;
  dob_status st = upload_params(ctx, 0);
  if (st != DOB_OK) return st;
  for (void* p : {s.u, s.v, s.w, s.u2, s.v2, s.w2}) CK(cudaMemsetAsync(p, 0, N * vsb, ctx->stream));
  CK(cudaMemsetAsync(s.cen, 0, N * 4 * vsb, ctx->stream));
  if (s.curl) CK(cudaMemsetAsync(s.curl, 0, N * 4 * vsb, ctx->stream));
  if (s.ref) launch_init_vel(s, ctx->stream);
  CK(cudaMemsetAsync(s.p, 0, N * 4, ctx->stream));
  CK(cudaMemsetAsync(s.rhs, 0, N * 4, ctx->stream));
  for (int l = 1; l < s.nlev; ++l) {
    const size_t n = s.lv[l].d.n();
    if (s.lv[l].e) CK(cudaMemsetAsync(s.lv[l].e, 0, n * 4, ctx->stream));
    if (s.lv[l].b) CK(cudaMemsetAsync(s.lv[l].b, 0, n * 4, ctx->stream));
    if (s.lv[l].eh) CK(cudaMemsetAsync(s.lv[l].eh, 0, n * 2, ctx->stream));
    if (s.lv[l].bh) CK(cudaMemsetAsync(s.lv[l].bh, 0, n * 2, ctx->stream));
  }
  for (float* a : {s.plo, s.e0, s.r0})
    if (a) CK(cudaMemsetAsync(a, 0, N * 4, ctx->stream));
  CK(cudaMemsetAsync(s.conc, 0, Nc * nch * dsb, ctx->stream));
  CK(cudaMemsetAsync(s.conc2, 0, Nc * nch * dsb, ctx->stream));
  if (s.cbrickA) {  // clear water everywhere
    const size_t nb = dye_brick_count(s.gc) * sizeof(uint32_t);
    CK(cudaMemsetAsync(s.cbrickA, 0, nb, ctx->stream));
    CK(cudaMemsetAsync(s.cbrickB, 0, nb, ctx->stream));
    CK(cudaMemsetAsync(s.sbrick, 0, nb, ctx->stream));  // the splat accumulators are zeroed below
    if (s.pbrick) CK(cudaMemsetAsync(s.pbrick, 0, nb, ctx->stream));
  }
  CK(cudaMemsetAsync(s.pred, 0, Nc * dsb, ctx->stream));
  CK(cudaMemsetAsync(s.splatI, 0, Nc * 4, ctx->stream));
  CK(cudaMemsetAsync(s.splatL, 0, Nc * 4, ctx->stream));
  // PARTICLE_RESET (particles.ts:27-45): posAndMass = 0, stretchAndLysis = (0, -0.003, 0, 0)
  std::vector<float> empty((size_t)s.cap * 8, 0.0f);
  for (uint32_t k = 0; k < s.cap; ++k) empty[(size_t)k * 8 + 5] = -0.003f;
  CK(cudaMemcpy(s.parcels, empty.data(), empty.size() * 4, cudaMemcpyHostToDevice));
  CK(cudaMemsetAsync(s.red, 0, RED_COUNT * sizeof(double), ctx->stream));
  CK(cudaMemsetAsync(s.redu, 0, REDU_COUNT * sizeof(unsigned int), ctx->stream));
  // the reset's lighting passes (BloodDropEngine.ts:1760) on the cleared dye
  if (s.light) launch_light_volume(s, ctx->stream);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  return DOB_OK;
}

dob_status dob_set_uniforms(dob_ctx* ctx, const float* u) {
  if (!ctx || !u) return DOB_EINVAL;
  for (int k = 0; k < 128; ++k)
    if (!isfinite(u[k])) return fail(ctx, DOB_EINVAL, "dob_set_uniforms", "non-finite value in the uniform block");
  memcpy(ctx->U, u, sizeof(ctx->U));
  return DOB_OK;
}

dob_status dob_inject_sphere(dob_ctx* ctx, const float c[3], float r, float dye, const float vel[3], float sigma,
                             uint64_t seed) {
  if (!ctx || !c || !vel) return DOB_EINVAL;
  if (ctx->cfg.bc_mode != DOB_BC_CLOSED_BOX)
    return fail(ctx, DOB_ESTATE, "dob_inject_sphere", "sphere injection is a closed-box operation");
  if (!(r > 0.0f) || !isfinite(r) || !isfinite(dye) || !isfinite(sigma))
    return fail(ctx, DOB_EINVAL, "dob_inject_sphere", "bad radius/dye/sigma");
  dob_status st = upload_params(ctx, 0);
  if (st != DOB_OK) return st;
  launch_inject_sphere(ctx->s, c, r, dye, vel, sigma, seed, ctx->stream);
  launch_dye_bricks_unknown(ctx->s, ctx->stream);
  ctx->inject_pending = kInjectedSteps;
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  return DOB_OK;
}

dob_status dob_inject_sphere_soft(dob_ctx* ctx, const float c[3], float r, float edge, float dye, const float vel[3],
                                  float sigma, uint64_t seed) {
  if (!ctx || !c || !vel) return DOB_EINVAL;
  if (ctx->cfg.bc_mode != DOB_BC_CLOSED_BOX)
    return fail(ctx, DOB_ESTATE, "dob_inject_sphere_soft", "sphere injection is a closed-box operation");
  if (!(r > 0.0f) || !(edge > 0.0f) || !isfinite(r) || !isfinite(edge) || !isfinite(dye) || !isfinite(sigma) ||
      !isfinite(vel[0]) || !isfinite(vel[1]) || !isfinite(vel[2]))
    return fail(ctx, DOB_EINVAL, "dob_inject_sphere_soft", "bad radius/edge/dye/velocity/sigma");
  dob_status st = upload_params(ctx, 0);
  if (st != DOB_OK) return st;
  launch_inject_sphere_soft(ctx->s, c, r, edge, dye, vel, sigma, seed, ctx->stream);
  launch_dye_bricks_unknown(ctx->s, ctx->stream);
  ctx->inject_pending = kInjectedSteps;
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  return DOB_OK;
}

dob_status dob_set_parcels(dob_ctx* ctx, const float* p, uint32_t n, uint32_t off) {
  if (!ctx || (!p && n)) return DOB_EINVAL;
  if ((uint64_t)off + n > ctx->s.cap) return fail(ctx, DOB_EINVAL, "dob_set_parcels", "range exceeds capacity");
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaMemcpy(ctx->s.parcels + (size_t)off * 8, p, (size_t)n * 32, cudaMemcpyHostToDevice));
  if (off + n > ctx->high_water) ctx->high_water = off + n;
  return DOB_OK;
}

dob_status dob_get_parcels(dob_ctx* ctx, float* p, uint32_t n, uint32_t off) {
  if (!ctx || (!p && n)) return DOB_EINVAL;
  if ((uint64_t)off + n > ctx->s.cap) return fail(ctx, DOB_EINVAL, "dob_get_parcels", "range exceeds capacity");
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaMemcpy(p, ctx->s.parcels + (size_t)off * 8, (size_t)n * 32, cudaMemcpyDeviceToHost));
  return DOB_OK;
}

dob_status dob_set_high_water(dob_ctx* ctx, uint32_t hw) {
  if (!ctx) return DOB_EINVAL;
  ctx->high_water = hw < ctx->s.cap ? hw : ctx->s.cap;
  return DOB_OK;
}

// Dye written from outside the step (field I/O, snapshots): every dye brick
// may hold dye until the next resolve rewrites the flags.
static dob_status dye_bricks_unknown(dob_ctx* ctx) {
  launch_dye_bricks_unknown(ctx->s, ctx->stream);
  CK(cudaGetLastError());
  return DOB_OK;
}

// ---- field I/O -----------------------------------------------------------------------
__global__ void k_add_arrays(const float* __restrict__ a, const float* __restrict__ b, float* __restrict__ out,
                             size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = a[i] + b[i];
}

namespace {
struct FieldDesc {
  void* dev;
  size_t count;     // host elements
  int kind;         // 0: VS, 1: DS, 2: f32, 3: u32, 4: f32 red-black split, 5: binary16
};
}  // namespace

static bool field_desc(dob_ctx* ctx, int field, FieldDesc* f) {
  DevState& s = ctx->s;
  const size_t N = s.g.n(), Nc = s.gc.n();
  switch (field) {
    case DOB_FIELD_VEL_U: *f = {s.u, N, 0}; return true;
    case DOB_FIELD_VEL_V: *f = {s.v, N, 0}; return true;
    case DOB_FIELD_VEL_W: *f = {s.w, N, 0}; return true;
    case DOB_FIELD_VEL_CENTER: *f = {s.cen, 4 * N, 0}; return true;
    case DOB_FIELD_CURL: *f = {s.curl, 4 * N, 0}; return s.curl != nullptr;
    case DOB_FIELD_PRESSURE: *f = {s.p, N, 4}; return true;
    case DOB_FIELD_RHS: *f = {s.rhs, N, 4}; return true;
    case DOB_FIELD_CONC: *f = {s.conc, (s.ref ? 4 : 1) * Nc, 1}; return true;
    case DOB_FIELD_CONC_PRED: *f = {s.pred, Nc, 1}; return true;
    case DOB_FIELD_SPLAT_INTACT: *f = {s.splatI, Nc, 3}; return true;
    case DOB_FIELD_SPLAT_LYSED: *f = {s.splatL, Nc, 3}; return true;
    case DOB_FIELD_WAVE: *f = {s.wave, (size_t)4 * kWaveN * kWaveN, 2}; return true;
    case DOB_FIELD_LIGHT: *f = {s.light, 4 * N, 5}; return s.light != nullptr;
    case DOB_FIELD_BRICKS: *f = {s.bricks, N / 64, 2}; return s.bricks != nullptr;
    case DOB_FIELD_BRICKS_RAW: *f = {s.brick_raw, N / 64, 2}; return s.brick_raw != nullptr;
    default: break;
  }
  void* dev = nullptr;
  size_t count = 0;
  int kind = 0;
  if (!adjoint_field(ctx, field, &dev, &count, &kind)) return false;
  *f = {dev, count, kind};
  return true;
}

dob_status dob_set_field(dob_ctx* ctx, int field, const void* host, size_t bytes) {
  if (!ctx || !host) return DOB_EINVAL;
  FieldDesc f;
  const bool read_only = field == DOB_FIELD_LIGHT || field == DOB_FIELD_BRICKS || field == DOB_FIELD_BRICKS_RAW;
  if (read_only || !field_desc(ctx, field, &f))
    return fail(ctx, DOB_EINVAL, "dob_set_field", "unknown or read-only field");
  if (bytes != f.count * 4) return fail(ctx, DOB_EINVAL, "dob_set_field", "byte count does not match the field");
  if (field == DOB_FIELD_CONC) {
    dob_status bs = dye_bricks_unknown(ctx);
    if (bs != DOB_OK) return bs;
  }
  if ((field == DOB_FIELD_SPLAT_INTACT || field == DOB_FIELD_SPLAT_LYSED) && ctx->s.sbrick)
    CK(cudaMemsetAsync(ctx->s.sbrick, 1, dye_brick_count(ctx->s.gc) * sizeof(uint32_t), ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  const size_t eb = f.kind == 0 ? vs_bytes(ctx->s.prec) : f.kind == 1 ? ds_bytes(ctx->s.prec) : 4;
  if (f.kind == 4) {
    float* tmp = nullptr;
    CK(cudaMalloc(&tmp, bytes));
    cudaError_t e = cudaMemcpy(tmp, host, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
      launch_split(tmp, (float*)f.dev, ctx->s.g, true, ctx->stream);
      // a pressure set from FP32 data has no low part
      if (field == DOB_FIELD_PRESSURE && ctx->s.plo) e = cudaMemsetAsync(ctx->s.plo, 0, bytes, ctx->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    }
    cudaFree(tmp);
    if (e != cudaSuccess) return fail(ctx, DOB_ECUDA, "dob_set_field", cudaGetErrorString(e));
  } else if (eb == 4) {
    CK(cudaMemcpy(f.dev, host, bytes, cudaMemcpyHostToDevice));
  } else {
    std::vector<uint16_t> tmp(f.count);
    const float* src = (const float*)host;
    for (size_t i = 0; i < f.count; ++i) tmp[i] = dob_f32_to_f16_bits(src[i]);
    CK(cudaMemcpy(f.dev, tmp.data(), f.count * 2, cudaMemcpyHostToDevice));
  }
  return DOB_OK;
}

dob_status dob_get_field(dob_ctx* ctx, int field, void* host, size_t bytes) {
  if (!ctx || !host) return DOB_EINVAL;
  CK(cudaStreamSynchronize(ctx->stream));
  if (field == DOB_FIELD_DIVERGENCE) {
    const size_t N = ctx->s.g.n();
    if (bytes != N * 4) return fail(ctx, DOB_EINVAL, "dob_get_field", "byte count does not match the field");
    float* tmp = nullptr;
    CK(cudaMalloc(&tmp, N * 4));
    launch_divergence(ctx->s, tmp, 1.0f, nullptr, ctx->stream);
    cudaError_t e = cudaMemcpyAsync(host, tmp, N * 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(tmp);
    if (e != cudaSuccess) return fail(ctx, DOB_ECUDA, "dob_get_field(divergence)", cudaGetErrorString(e));
    return DOB_OK;
  }
  FieldDesc f;
  if (!field_desc(ctx, field, &f)) return fail(ctx, DOB_EINVAL, "dob_get_field", "unknown field");
  if (bytes != f.count * 4) return fail(ctx, DOB_EINVAL, "dob_get_field", "byte count does not match the field");
  const size_t eb = f.kind == 0 ? vs_bytes(ctx->s.prec) : f.kind == 1 ? ds_bytes(ctx->s.prec) : f.kind == 5 ? 2 : 4;
  if (f.kind == 4) {
    float* tmp = nullptr;
    CK(cudaMalloc(&tmp, bytes));
    cudaError_t e = cudaSuccess;
    if (field == DOB_FIELD_PRESSURE && ctx->s.plo) {
      // double-float pressure: read p + plo rounded to FP32
      float* sum = nullptr;
      e = cudaMalloc(&sum, bytes);
      if (e == cudaSuccess) {
        k_add_arrays<<<ctx->s.num_sms * 4, 256, 0, ctx->stream>>>(ctx->s.p, ctx->s.plo, sum, f.count);
        launch_split(sum, tmp, ctx->s.g, false, ctx->stream);
        e = cudaStreamSynchronize(ctx->stream);
        cudaFree(sum);
      }
    } else {
      launch_split((const float*)f.dev, tmp, ctx->s.g, false, ctx->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpy(host, tmp, bytes, cudaMemcpyDeviceToHost);
    cudaFree(tmp);
    if (e != cudaSuccess) return fail(ctx, DOB_ECUDA, "dob_get_field", cudaGetErrorString(e));
  } else if (eb == 4) {
    CK(cudaMemcpy(host, f.dev, bytes, cudaMemcpyDeviceToHost));
  } else {
    std::vector<uint16_t> tmp(f.count);
    CK(cudaMemcpy(tmp.data(), f.dev, f.count * 2, cudaMemcpyDeviceToHost));
    float* dst = (float*)host;
    for (size_t i = 0; i < f.count; ++i) dst[i] = dob_f16_bits_to_f32(tmp[i]);
  }
  return DOB_OK;
}

// ---- stepping ----------------------------------------------------------------------------
// `light`: end with the lighting passes (DOB_PHYS_LIGHTING), which read the
// last step's parameters.
static dob_status step_impl(dob_ctx* ctx, int nsteps, uint32_t flags, dob_step_stats* stats, bool light) {
  if (!ctx || nsteps < 0) return DOB_EINVAL;
  if (ctx->cfg.bc_mode == DOB_BC_REFERENCE && !isfinite(ctx->U[38]))
    return fail(ctx, DOB_EINVAL, "dob_step", "non-finite dt");
  float stage_ms[DOB_STAGE_COUNT] = {0};
  const bool timing = (flags & DOB_STEP_TIMING) != 0;
  for (int k = 0; k < nsteps; ++k) {
    dob_status st = one_step(ctx, flags, timing ? stage_ms : nullptr);
    if (st != DOB_OK) return st;
  }
  if (light && nsteps > 0 && ctx->s.light && (ctx->s.flags & DOB_PHYS_LIGHTING)) {
    launch_light_volume(ctx->s, ctx->stream);
    CK(cudaGetLastError());
  }
  if (stats) {
    memset(stats, 0, sizeof(*stats));
    if (flags & DOB_STEP_STATS) {
      dob_status st = finish_stats(ctx, stats, nsteps);
      if (st != DOB_OK) return st;
    } else {
      CK(cudaStreamSynchronize(ctx->stream));
      stats->struct_size = sizeof(dob_step_stats);
      stats->steps_done = nsteps;
    }
    for (int k = 0; k < DOB_STAGE_COUNT; ++k) stats->stage_ms[k] = stage_ms[k];
  }
  return DOB_OK;
}

dob_status dob_step(dob_ctx* ctx, int nsteps, uint32_t flags, dob_step_stats* stats) {
  return step_impl(ctx, nsteps, flags, stats, true);
}

dob_status dob_step_async(dob_ctx* ctx, int slot) {
  if (!ctx || slot < 0 || slot >= 8) return DOB_EINVAL;
  if (ctx->cfg.bc_mode == DOB_BC_REFERENCE && !isfinite(ctx->U[38]))
    return fail(ctx, DOB_EINVAL, "dob_step_async", "non-finite dt");
  dob_ctx::AsyncSlot& a = ctx->async_slots[slot];
  if (a.pending) return fail(ctx, DOB_ESTATE, "dob_step_async", "result slot still pending");
  if (!a.red) {
    CK(cudaMallocHost((void**)&a.red, kStatsBytes));
    a.redu = reinterpret_cast<unsigned int*>(a.red + RED_COUNT);
    CK(cudaEventCreateWithFlags(&a.done, cudaEventDisableTiming));
  }
  dob_status st = one_step(ctx, DOB_STEP_STATS, nullptr);
  if (st != DOB_OK) return st;
  DevState& s = ctx->s;
  if (ctx->stats_mask & DOB_STATS_PARCELS) launch_count_alive(s, s.redu + REDU_ALIVE, ctx->stream);
  CK(cudaMemcpyAsync(a.red, s.red, kStatsBytes, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaEventRecord(a.done, ctx->stream));
  a.cycles = ctx->last_cycles;
  a.pending = true;
  return DOB_OK;
}

dob_status dob_set_step_stats(dob_ctx* ctx, uint32_t mask) {
  if (!ctx || (mask & ~DOB_STATS_ALL)) return DOB_EINVAL;
  for (auto& a : ctx->async_slots)
    if (a.pending) return fail(ctx, DOB_ESTATE, "dob_set_step_stats", "a pipelined step is pending");
  if (mask != ctx->stats_mask) {
    CK(cudaStreamSynchronize(ctx->stream));
    drop_graphs(ctx);  // the statistics graph holds the residual pass or not
    ctx->stats_mask = mask;
  }
  return DOB_OK;
}

dob_status dob_step_result(dob_ctx* ctx, int slot, dob_step_stats* stats) {
  if (!ctx || !stats || slot < 0 || slot >= 8) return DOB_EINVAL;
  dob_ctx::AsyncSlot& a = ctx->async_slots[slot];
  if (!a.pending) return fail(ctx, DOB_ESTATE, "dob_step_result", "no step pending in this slot");
  CK(cudaEventSynchronize(a.done));
  a.pending = false;
  memset(stats, 0, sizeof(*stats));
  fill_stats(ctx, a.red, a.redu, stats, 1, a.cycles);
  return DOB_OK;
}

dob_status dob_step_uniforms(dob_ctx* ctx, const float* blocks, int nsteps, uint32_t flags, dob_step_stats* stats) {
  if (!ctx || (!blocks && nsteps) || nsteps < 0) return DOB_EINVAL;
  for (int k = 0; k < nsteps; ++k) {
    dob_status st = dob_set_uniforms(ctx, blocks + (size_t)k * 128);
    if (st != DOB_OK) return st;
    st = step_impl(ctx, 1, flags, k == nsteps - 1 ? stats : nullptr, k == nsteps - 1);
    if (st != DOB_OK) return st;
  }
  return DOB_OK;
}

dob_status dob_run_stage(dob_ctx* ctx, int stage) {
  if (!ctx) return DOB_EINVAL;
  if (stage < 0 || stage >= DOB_STAGE_COUNT) return fail(ctx, DOB_EINVAL, "dob_run_stage", "bad stage");
  const uint32_t spawn = stage == DOB_STAGE_PARCEL_EMIT ? spawn_count(ctx) : 0u;
  dob_status st = upload_params(ctx, spawn);
  if (st != DOB_OK) return st;
  if (stage == DOB_STAGE_CURL && !ctx->s.curl) return fail(ctx, DOB_ESTATE, "dob_run_stage", "no curl field in this mode");
  enqueue_stage(ctx, ctx->s, stage, ctx->stream);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  return DOB_OK;
}

dob_status dob_wave_step(dob_ctx* ctx) {
  if (!ctx) return DOB_EINVAL;
  if (!(ctx->s.flags & DOB_PHYS_WAVE))
    return fail(ctx, DOB_ESTATE, "dob_wave_step", "context created without DOB_PHYS_WAVE (reference mode)");
  dob_status st = upload_params(ctx, 0u);
  if (st != DOB_OK) return st;
  launch_wave_step(ctx->s, ctx->stream);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  return DOB_OK;
}

dob_status dob_light_volume(dob_ctx* ctx) {
  if (!ctx) return DOB_EINVAL;
  if (!ctx->s.light)
    return fail(ctx, DOB_ESTATE, "dob_light_volume", "reference mode with nx, ny, nz divisible by 4 only");
  dob_status st = upload_params(ctx, 0u);
  if (st != DOB_OK) return st;
  launch_light_volume(ctx->s, ctx->stream);
  CK(cudaGetLastError());
  return DOB_OK;
}

dob_status dob_set_spectral_lut(dob_ctx* ctx, const float* rgba, size_t bytes) {
  if (!ctx || !rgba) return DOB_EINVAL;
  const size_t want = (size_t)DOB_SPECTRAL_LUT_W * DOB_SPECTRAL_LUT_H * 4 * sizeof(float);
  if (bytes != want) return fail(ctx, DOB_EINVAL, "dob_set_spectral_lut", "need 256 x 64 x 4 floats");
  if (!ctx->lut) CK(cudaMalloc((void**)&ctx->lut, want));
  CK(cudaMemcpyAsync(ctx->lut, rgba, want, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return DOB_OK;
}

// the image buffer for a W x H render (8 halves per pixel)
static dob_status render_prepare(dob_ctx* ctx, uint32_t w, uint32_t h, const char* what) {
  if (!ctx->s.light) return fail(ctx, DOB_ESTATE, what, "reference mode with nx, ny, nz divisible by 4 only");
  if (!ctx->lut) return fail(ctx, DOB_ESTATE, what, "no spectral table (dob_set_spectral_lut)");
  if (w < 1 || h < 1 || w > 8192 || h > 8192) return fail(ctx, DOB_EINVAL, what, "image size out of 1..8192");
  const size_t need = (size_t)w * h * 8 * sizeof(__half);
  if (need > ctx->image_cap) {
    if (ctx->image) cudaFree(ctx->image);
    ctx->image = nullptr;
    ctx->image_cap = 0;
    CK(cudaMalloc((void**)&ctx->image, need));
    ctx->image_cap = need;
  }
  ctx->render_w = (int)w;
  ctx->render_h = (int)h;
  return upload_params(ctx, 0u);
}

dob_status dob_render_plume(dob_ctx* ctx, uint32_t width, uint32_t height, uint16_t* out, size_t bytes) {
  if (!ctx || !out) return DOB_EINVAL;
  if (bytes != (size_t)width * height * 8 * sizeof(uint16_t))
    return fail(ctx, DOB_EINVAL, "dob_render_plume", "byte count != width x height x 8 halves");
  dob_status st = render_prepare(ctx, width, height, "dob_render_plume");
  if (st != DOB_OK) return st;
  launch_light_volume(ctx->s, ctx->stream);
  launch_render_plume(ctx->s, ctx->lut, (int)width, (int)height, ctx->image, ctx->stream);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, ctx->image, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return DOB_OK;
}

dob_status dob_sync(dob_ctx* ctx) {
  if (!ctx) return DOB_EINVAL;
  CK(cudaStreamSynchronize(ctx->stream));
  return DOB_OK;
}

dob_status dob_launches_per_step(dob_ctx* ctx, int* n) {
  if (!ctx || !n) return DOB_EINVAL;
  if (!ctx->kernels_per_step) {
    // capture the plain step graph once (no launch) to count its kernel nodes
    dob_ctx::StepGraph* G = nullptr;
    dob_status st = get_graph(ctx, false, false, &G);
    if (st != DOB_OK) return st;
  }
  *n = ctx->kernels_per_step;
  return DOB_OK;
}

dob_status dob_io_bytes(const dob_ctx* ctx, uint64_t* h2d, uint64_t* d2h) {
  if (!ctx || !h2d || !d2h) return DOB_EINVAL;
  *h2d = sizeof(StepParams);
  *d2h = sizeof(double) * RED_COUNT + sizeof(unsigned int) * REDU_COUNT;
  return DOB_OK;
}

dob_status dob_memory_bytes(const dob_ctx* ctx, uint64_t* bytes) {
  if (!ctx || !bytes) return DOB_EINVAL;
  *bytes = ctx->bytes;
  return DOB_OK;
}

dob_status dob_time_steps(dob_ctx* ctx, int nsteps, uint32_t flags, float* ms) {
  if (!ctx || !ms || nsteps < 0) return DOB_EINVAL;
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  for (int k = 0; k < nsteps; ++k) {
    dob_status st = one_step(ctx, flags & ~(uint32_t)DOB_STEP_TIMING, nullptr);
    if (st != DOB_OK) return st;
  }
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  CK(cudaEventSynchronize(ctx->ev1));
  CK(cudaEventElapsedTime(ms, ctx->ev0, ctx->ev1));
  return DOB_OK;
}

dob_status dob_bench_kernel(dob_ctx* ctx, int which, int reps, float* avg_ms, double* bytes_per_launch) {
  if (!ctx || !avg_ms || reps < 1 || which < 0 || which > 3) return DOB_EINVAL;
  if (which == 1) {
    if (!(ctx->s.flags & DOB_PHYS_WAVE))
      return fail(ctx, DOB_ESTATE, "dob_bench_kernel", "context created without DOB_PHYS_WAVE");
    dob_status st = upload_params(ctx, 0u);
    if (st != DOB_OK) return st;
  }
  if (which == 2) {
    if (!ctx->s.light) return fail(ctx, DOB_ESTATE, "dob_bench_kernel", "no light volume in this mode");
    dob_status st = upload_params(ctx, 0u);
    if (st != DOB_OK) return st;
  }
  if (which == 3) {
    if (!ctx->render_w) return fail(ctx, DOB_ESTATE, "dob_bench_kernel", "no render yet (dob_render_plume)");
    dob_status st = render_prepare(ctx, (uint32_t)ctx->render_w, (uint32_t)ctx->render_h, "dob_bench_kernel");
    if (st != DOB_OK) return st;
  }
  CK(cudaStreamSynchronize(ctx->stream));
  double total = 0.0, bytes = 0.0;
  for (int r = 0; r < reps; ++r) {
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    if (which == 0) {
      bytes = smoother_pass(ctx->s, ctx->stream);
    } else if (which == 3) {
      // plume march: the image written once (16 B per pixel); the volumes it
      // samples stay in L2 across rays and are not counted
      launch_render_plume(ctx->s, ctx->lut, ctx->render_w, ctx->render_h, ctx->image, ctx->stream);
      bytes = 16.0 * ctx->render_w * ctx->render_h;
    } else if (which == 2) {
      // light volume: the 4-channel dye read once (every dye voxel is a tap
      // of some centre sample), the light volume written once (8 B per
      // velocity cell), the two brick maps (4 B per 64 cells each) and the
      // raw map read 125 times from L2, counted once
      launch_light_volume(ctx->s, ctx->stream);
      const size_t dsb = ctx->s.prec == DOB_PREC_FP32 ? 4 : 2;
      bytes = (double)ctx->s.gc.n() * 4 * dsb + (double)ctx->s.g.n() * 8 + (double)ctx->s.g.n() / 64 * 12;
    } else {
      // the wave substep: wave 16 B in, film 4 + spectrum 8 B out (force +
      // row FFT); spectrum 8 in + 8 out twice (columns, inverse rows);
      // spectrum 8 + film 4 in, wave 16 out (finalize): 88 B per texel
      launch_wave_step(ctx->s, ctx->stream);
      bytes = 88.0 * kWaveN * kWaveN;
    }
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    CK(cudaEventSynchronize(ctx->ev1));
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    total += ms;
  }
  *avg_ms = (float)(total / reps);
  if (bytes_per_launch) *bytes_per_launch = bytes;
  return DOB_OK;
}

dob_status dob_save_state(dob_ctx* ctx, int slot) {
  if (!ctx || slot < 0 || slot >= kSnapshots) return DOB_EINVAL;
  DevState& s = ctx->s;
  const size_t N = s.g.n(), Nc = s.gc.n();
  const size_t vsb = vs_bytes(s.prec), dsb = ds_bytes(s.prec);
  const int nch = s.ref ? 4 : 1;
  // the wave field is state only when the wave solver advances it
  void* src[] = {s.u, s.v, s.w, s.cen, s.curl, s.p, s.conc, s.parcels, s.plo, s.wave};
  const size_t sz[] = {N * vsb, N * vsb, N * vsb, N * 4 * vsb, s.curl ? N * 4 * vsb : 0, N * 4, Nc * nch * dsb,
                       (size_t)s.cap * 32, s.plo ? N * 4 : 0,
                       (s.flags & DOB_PHYS_WAVE) ? (size_t)kWaveN * kWaveN * 16 : 0};
  Snapshot& sn = ctx->snaps[slot];
  if (!sn.valid) {
    for (size_t k = 0; k < sizeof(sz) / sizeof(sz[0]); ++k) {
      void* p = nullptr;
      if (sz[k]) {
        cudaError_t e = cudaMalloc(&p, sz[k]);
        if (e != cudaSuccess) {
          cudaGetLastError();
          return fail(ctx, DOB_ENOMEM, "dob_save_state", cudaGetErrorString(e));
        }
      }
      sn.bufs.push_back(p);
      sn.sizes.push_back(sz[k]);
    }
    sn.valid = true;
  }
  for (size_t k = 0; k < sn.bufs.size(); ++k)
    if (sn.sizes[k]) CK(cudaMemcpyAsync(sn.bufs[k], src[k], sn.sizes[k], cudaMemcpyDeviceToDevice, ctx->stream));
  sn.high_water = ctx->high_water;
  sn.step_index = ctx->step_index;
  sn.inject_pending = ctx->inject_pending;
  CK(cudaStreamSynchronize(ctx->stream));
  return DOB_OK;
}

dob_status dob_load_state(dob_ctx* ctx, int slot) {
  if (!ctx || slot < 0 || slot >= kSnapshots) return DOB_EINVAL;
  Snapshot& sn = ctx->snaps[slot];
  if (!sn.valid) return fail(ctx, DOB_ESTATE, "dob_load_state", "empty snapshot slot");
  DevState& s = ctx->s;
  void* dst[] = {s.u, s.v, s.w, s.cen, s.curl, s.p, s.conc, s.parcels, s.plo, s.wave};
  for (size_t k = 0; k < sn.bufs.size(); ++k)
    if (sn.sizes[k]) CK(cudaMemcpyAsync(dst[k], sn.bufs[k], sn.sizes[k], cudaMemcpyDeviceToDevice, ctx->stream));
  ctx->high_water = sn.high_water;
  ctx->step_index = sn.step_index;
  ctx->inject_pending = sn.inject_pending;
  dob_status bs = dye_bricks_unknown(ctx);
  if (bs != DOB_OK) return bs;
  CK(cudaStreamSynchronize(ctx->stream));
  return DOB_OK;
}

dob_status dob_eval_math(int fn, const float* x, const float* y, float* out, uint32_t n) {
  if (!x || !out || fn < 0 || fn > 9 || (fn == 4 || fn == 5 || fn == 9) && !y) return DOB_EINVAL;
  if (n == 0) return DOB_OK;
  cudaError_t e = eval_math_device(fn, x, y, out, n);
  if (e != cudaSuccess) return fail(nullptr, DOB_ECUDA, "dob_eval_math", cudaGetErrorString(e));
  return DOB_OK;
}

}  // extern "C"

namespace dob {
// Context-free error record for entry points defined in other translation
// units; read back with dob_last_error(NULL).
dob_status record_static_error(dob_status st, const char* what, const char* detail) {
  return fail(nullptr, st, what, detail);
}

// A step whose body the caller enqueues itself (the adjoint tape records its
// last segment this way): the host part of one_step before the body (the
// step's parameters uploaded, the injection count), the parcel stages, and
// the step count after it.  The V-cycle count of the body is the caller's.
dob_status step_host_begin(dob_ctx* ctx) {
  dob_status st = upload_params(ctx, spawn_count(ctx));
  if (st != DOB_OK) return st;
  if (ctx->inject_pending > 0) --ctx->inject_pending;
  ctx->last_cycles = ctx->cfg.mg_cycles;
  return DOB_OK;
}
void enqueue_parcel_stages(dob_ctx* ctx, DevState& s, cudaStream_t st) {
  enqueue_stage(ctx, s, DOB_STAGE_CLEAR_SPLATS, st);
  enqueue_stage(ctx, s, DOB_STAGE_PARCEL_EMIT, st);
  enqueue_stage(ctx, s, DOB_STAGE_PARCEL_ADVECT, st);
}
void step_host_end(dob_ctx* ctx) { ctx->step_index++; }
}  // namespace dob
