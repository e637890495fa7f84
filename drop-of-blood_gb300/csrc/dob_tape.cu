// dob_tape.cu — the forward/backward pair of the discrete adjoint
// (dob_adjoint_stage, dob_tape_forward, dob_tape_backward,
// dob_adjoint_sphere_impulse) for the closed-box step in FP32 and in the
// mixed mode.
//
// Memory is bounded by checkpointing: the forward keeps (velocity, dye,
// pressure) every k steps; the backward recomputes one segment of at most k
// steps at a time, recording each step's linearisation points (the step's
// input velocity, centre velocity and dye, the advected velocity, the
// predictor, and the next centre velocity), then runs the adjoint stages of
// those steps in reverse.  The recomputation launches the forward kernels
// themselves on tape buffers, so the linearisation points are the forward's
// own values (up to the order of the FP64 atomic sums in the mean removal).
// Parcels are passive tracers in the closed box (nothing reads their splat)
// and are not recomputed.
//
// Mixed mode: the tape and the checkpoints hold the dye and the predictor
// at their binary16 storage width and the pressure as its FP32 pair (p,
// plo), so a recomputed segment is the forward's own; the backward reads
// the binary16 linearisation points and keeps its adjoint arrays in FP32.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <vector>

#include "dob_ctx.h"

using namespace dob;

#define TCK(call)                                                                         \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) return record_error(ctx, DOB_ECUDA, #call, cudaGetErrorString(e_)); \
  } while (0)

namespace dob {

struct AdjCtx {
  AdjState a;
  std::vector<void*> bufs;  // adjoint arrays
  // tape
  int k = 0;          // steps per checkpoint segment
  int nsteps = 0;     // recorded steps
  bool recorded = false;
  // the tape slots hold the last segment's linearisation points, recorded by
  // dob_tape_forward (no recomputation of that segment needed)
  bool last_in_slots = false;
  std::vector<float*> ck;   // per checkpoint: u, v, w, dye, p, plo (kCk arrays; plo in the mixed mode only)
  std::vector<void*> tbufs; // segment buffers
  std::vector<float*> Tu, Tv, Tw, Tc;  // k + 1 entries
  std::vector<float4*> Tcen;           // k + 1 entries
  std::vector<float*> Tua, Tva, Twa, Tpred;  // k entries
  float* Tp = nullptr;
  float* Tplo = nullptr;    // mixed mode: the pressure's low part
  float* Trhs = nullptr;
  float* Tsc[3] = {nullptr, nullptr, nullptr};  // Casson's output during recomputation (no adjoint reads it)
  double* dred = nullptr;   // reduction slots of the drop gradients (4 doubles)
  // captured "recompute + reverse" graph of a segment, per (length, parity of
  // the dye adjoint ping-pong at its start, recomputation or the recorded
  // last segment)
  std::vector<cudaGraphExec_t> seg_graphs;
  // captured recording step j of the forward's last segment (tape slots j
  // and j + 1; the step's parameters are uploaded before each launch)
  std::vector<cudaGraphExec_t> rec_graphs;
  void drop_graphs() {
    for (cudaGraphExec_t& g : seg_graphs)
      if (g) cudaGraphExecDestroy(g);
    seg_graphs.clear();
    for (cudaGraphExec_t& g : rec_graphs)
      if (g) cudaGraphExecDestroy(g);
    rec_graphs.clear();
  }
};

void adjoint_free(dob_ctx* ctx) {
  AdjCtx* A = ctx->adj;
  if (!A) return;
  for (void* p : A->bufs) cudaFree(p);
  for (void* p : A->tbufs) cudaFree(p);
  for (float* p : A->ck) cudaFree(p);
  A->drop_graphs();
  delete A;
  ctx->adj = nullptr;
}

}  // namespace dob

namespace {

constexpr size_t kCk = 6;  // arrays per checkpoint

dob_status need_box_fp32(dob_ctx* ctx, const char* what) {
  const int prec = ctx->cfg.precision_mode;
  if (ctx->cfg.bc_mode != DOB_BC_CLOSED_BOX || (prec != DOB_PREC_FP32 && prec != DOB_PREC_MIXED) ||
      ctx->cfg.dye_refine != 1)
    return record_error(ctx, DOB_ESTATE, what,
                        "the adjoint covers the closed-box step (FP32 or mixed precision) with dye_refine 1");
  return DOB_OK;
}
bool mixed(const dob_ctx* ctx) { return ctx->s.prec == DOB_PREC_MIXED; }
// bytes of one dye (or predictor) value as stored
size_t dye_bytes(const dob_ctx* ctx) { return mixed(ctx) ? 2 : 4; }

dob_status alloc(dob_ctx* ctx, std::vector<void*>& list, void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return record_error(ctx, DOB_ENOMEM, "adjoint allocation", cudaGetErrorString(e));
  }
  list.push_back(*p);
  e = cudaMemset(*p, 0, bytes);
  if (e != cudaSuccess) return record_error(ctx, DOB_ECUDA, "adjoint allocation", cudaGetErrorString(e));
  return DOB_OK;
}

// Adjoint arrays, allocated (zeroed) on first use.
dob_status ensure_adj(dob_ctx* ctx) {
  if (ctx->adj) return DOB_OK;
  cudaError_t pe = adj_prepare();
  if (pe != cudaSuccess) return record_error(ctx, DOB_ECUDA, "adj_prepare", cudaGetErrorString(pe));
  AdjCtx* A = new AdjCtx();
  memset(&A->a, 0, sizeof(A->a));
  ctx->adj = A;
  const DevState& s = ctx->s;
  const size_t N = s.g.n(), Nc = s.gc.n();
  AdjState& a = A->a;
  dob_status st = DOB_OK;
  auto F = [&](float** p, size_t n) {
    if (st == DOB_OK) st = alloc(ctx, A->bufs, (void**)p, n * sizeof(float));
  };
  F(&a.au, N); F(&a.av, N); F(&a.aw, N); F(&a.au2, N); F(&a.av2, N); F(&a.aw2, N);
  if (st == DOB_OK) st = alloc(ctx, A->bufs, (void**)&a.acen, N * sizeof(float4));
  F(&a.ac, Nc); F(&a.ac2, Nc); F(&a.apred, Nc);
  F(&a.ap, N); F(&a.arhs, N); F(&a.alpha, N); F(&a.gq, N);
  if (s.prec == DOB_PREC_MIXED) { F(&a.lam, N); F(&a.lamlo, N); }
  for (int l = 1; l < s.nlev; ++l) {
    F(&a.le[l], s.lv[l].d.n());
    F(&a.lb[l], s.lv[l].d.n());
  }
  if (st == DOB_OK) st = alloc(ctx, A->bufs, (void**)&a.red, 8 * sizeof(double));
  if (st == DOB_OK) st = alloc(ctx, A->bufs, (void**)&a.part, 2 * kSumBlocks * sizeof(double));
  if (st == DOB_OK) st = alloc(ctx, A->bufs, (void**)&A->dred, 4 * sizeof(double));
  if (st != DOB_OK) adjoint_free(ctx);
  return st;
}

void zero_adj(const DevState& s, const AdjState& a, cudaStream_t st) {
  const size_t N = s.g.n(), Nc = s.gc.n();
  for (float* p : {a.au, a.av, a.aw, a.au2, a.av2, a.aw2, a.ap, a.arhs}) cudaMemsetAsync(p, 0, N * 4, st);
  for (float* p : {a.ac, a.ac2, a.apred}) cudaMemsetAsync(p, 0, Nc * 4, st);
  cudaMemsetAsync(a.acen, 0, N * sizeof(float4), st);
  if (a.lam) {  // mixed mode: the adjoint pressure solve's warm start
    cudaMemsetAsync(a.lam, 0, N * 4, st);
    cudaMemsetAsync(a.lamlo, 0, N * 4, st);
  }
  for (int l = 1; l < s.nlev; ++l) {
    cudaMemsetAsync(a.le[l], 0, s.lv[l].d.n() * 4, st);
    cudaMemsetAsync(a.lb[l], 0, s.lv[l].d.n() * 4, st);
  }
}

// Tape buffers for segments of k steps.
dob_status ensure_tape(dob_ctx* ctx, int k, int nseg) {
  AdjCtx* A = ctx->adj;
  const DevState& s = ctx->s;
  const size_t N = s.g.n(), Nc = s.gc.n(), db = dye_bytes(ctx);
  if (A->k != k) {
    A->drop_graphs();
    for (void* p : A->tbufs) cudaFree(p);
    A->tbufs.clear();
    A->Tu.assign(k + 1, nullptr); A->Tv.assign(k + 1, nullptr); A->Tw.assign(k + 1, nullptr);
    A->Tc.assign(k + 1, nullptr); A->Tcen.assign(k + 1, nullptr);
    A->Tua.assign(k, nullptr); A->Tva.assign(k, nullptr); A->Twa.assign(k, nullptr); A->Tpred.assign(k, nullptr);
    A->k = 0;
    dob_status st = DOB_OK;
    auto F = [&](void** p, size_t b) {
      if (st == DOB_OK) st = alloc(ctx, A->tbufs, p, b);
    };
    for (int j = 0; j <= k; ++j) {
      F((void**)&A->Tu[j], N * 4); F((void**)&A->Tv[j], N * 4); F((void**)&A->Tw[j], N * 4);
      F((void**)&A->Tc[j], Nc * db); F((void**)&A->Tcen[j], N * sizeof(float4));
      if (j < k) {
        F((void**)&A->Tua[j], N * 4); F((void**)&A->Tva[j], N * 4); F((void**)&A->Twa[j], N * 4);
        F((void**)&A->Tpred[j], Nc * db);
      }
    }
    F((void**)&A->Tp, N * 4);
    if (mixed(ctx)) F((void**)&A->Tplo, N * 4);
    F((void**)&A->Trhs, N * 4);
    for (int c = 0; c < 3; ++c) F((void**)&A->Tsc[c], N * 4);
    if (st != DOB_OK) return st;
    A->k = k;
  }
  const size_t want = (size_t)nseg * kCk;
  while (A->ck.size() < want) {
    float* p = nullptr;
    const size_t j = A->ck.size() % kCk;
    if (j == 5 && !mixed(ctx)) {
      A->ck.push_back(nullptr);
      continue;
    }
    const size_t b = j == 3 ? Nc * db : N * 4;
    cudaError_t e = cudaMalloc(&p, b);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return record_error(ctx, DOB_ENOMEM, "dob_tape_forward", cudaGetErrorString(e));
    }
    A->ck.push_back(p);
  }
  return DOB_OK;
}

void save_checkpoint(dob_ctx* ctx, int seg) {
  AdjCtx* A = ctx->adj;
  const DevState& s = ctx->s;
  const size_t N = s.g.n(), Nc = s.gc.n();
  float** c = &A->ck[(size_t)seg * kCk];
  cudaStream_t st = ctx->stream;
  cudaMemcpyAsync(c[0], s.u, N * 4, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(c[1], s.v, N * 4, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(c[2], s.w, N * 4, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(c[3], s.conc, Nc * dye_bytes(ctx), cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(c[4], s.p, N * 4, cudaMemcpyDeviceToDevice, st);
  if (mixed(ctx)) cudaMemcpyAsync(c[5], s.plo, N * 4, cudaMemcpyDeviceToDevice, st);
}

// Recompute steps [0, len) of segment `seg` from its checkpoint, recording
// the linearisation points in the tape buffers.
void restore_checkpoint(dob_ctx* ctx, int seg) {
  AdjCtx* A = ctx->adj;
  const DevState& s = ctx->s;
  const size_t N = s.g.n(), Nc = s.gc.n();
  cudaStream_t st = ctx->stream;
  float** c = &A->ck[(size_t)seg * kCk];
  cudaMemcpyAsync(A->Tu[0], c[0], N * 4, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(A->Tv[0], c[1], N * 4, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(A->Tw[0], c[2], N * 4, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(A->Tc[0], c[3], Nc * dye_bytes(ctx), cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(A->Tp, c[4], N * 4, cudaMemcpyDeviceToDevice, st);
  if (mixed(ctx)) cudaMemcpyAsync(A->Tplo, c[5], N * 4, cudaMemcpyDeviceToDevice, st);
}
// Step j of a segment from tape slot j: the step's fluid and dye stages
// writing their linearisation points into the tape (slot j + 1 receives the
// step's result).  Casson's output (the unprojected velocity, which no
// adjoint stage reads) goes to scratch; the projection writes the next
// step's velocity and centre velocity.  The column kernels give the bits of
// the step graph's.  parcels: also the parcel stages of the step (recording
// the forward pass).
void tape_step(dob_ctx* ctx, int j, bool parcels) {
  AdjCtx* A = ctx->adj;
  const DevState& s = ctx->s;
  cudaStream_t st = ctx->stream;
  DevState t = s;
  t.p = A->Tp; t.plo = A->Tplo; t.rhs = A->Trhs;
  t.u = A->Tu[j]; t.v = A->Tv[j]; t.w = A->Tw[j]; t.cen = A->Tcen[j];
  t.u2 = A->Tua[j]; t.v2 = A->Tva[j]; t.w2 = A->Twa[j];
  launch_advect_mac(t, st);
  t.u = A->Tua[j]; t.v = A->Tva[j]; t.w = A->Twa[j]; t.conc = A->Tc[j];
  t.u2 = A->Tsc[0]; t.v2 = A->Tsc[1]; t.w2 = A->Tsc[2];
  launch_casson_box(t, st);
  t.u = A->Tsc[0]; t.v = A->Tsc[1]; t.w = A->Tsc[2];
  launch_mac_rhs_box(t, st);
  launch_pressure_solve(t, st);
  t.u2 = A->Tu[j + 1]; t.v2 = A->Tv[j + 1]; t.w2 = A->Tw[j + 1]; t.cen = A->Tcen[j + 1];
  launch_project_center_box(t, st);
  if (parcels) {
    DevState tp = s;
    tp.cen = A->Tcen[j + 1];
    enqueue_parcel_stages(ctx, tp, st);
  }
  t.conc = A->Tc[j]; t.pred = A->Tpred[j]; t.conc2 = A->Tc[j + 1];
  launch_conc_predict(t, st, true);
  launch_dye_resolve_lim(t, st);
}
// From the restored checkpoint state in the first tape slot: recompute
// `len` steps recording their linearisation points.
void replay_segment(dob_ctx* ctx, int len) {
  AdjCtx* A = ctx->adj;
  DevState t = ctx->s;
  t.u = A->Tu[0]; t.v = A->Tv[0]; t.w = A->Tw[0]; t.cen = A->Tcen[0];
  launch_mac_to_center(t, ctx->stream);  // the centre velocity at a step's start is C(u)
  for (int j = 0; j < len; ++j) tape_step(ctx, j, false);
}
// The forward pass's last segment (checkpoint `seg` just saved from the
// context): its `len` steps computed once, by the recording kernels, with
// each step's parameters and parcel stages as dob_step runs them; then the
// context takes the final state from the tape.  The backward finds this
// segment's linearisation points in the slots and does not recompute it.
dob_status record_last_segment(dob_ctx* ctx, int seg, int len) {
  AdjCtx* A = ctx->adj;
  DevState& s = ctx->s;
  cudaStream_t st = ctx->stream;
  const size_t N = s.g.n(), Nc = s.gc.n();
  restore_checkpoint(ctx, seg);
  DevState t = s;
  t.u = A->Tu[0]; t.v = A->Tv[0]; t.w = A->Tw[0]; t.cen = A->Tcen[0];
  launch_mac_to_center(t, st);
  if (A->rec_graphs.size() != (size_t)A->k) {
    for (cudaGraphExec_t& g : A->rec_graphs)
      if (g) cudaGraphExecDestroy(g);
    A->rec_graphs.assign(A->k, nullptr);
  }
  for (int j = 0; j < len; ++j) {
    dob_status e = step_host_begin(ctx);
    if (e != DOB_OK) return e;
    // one captured graph per slot: the mixed solve's loops become while-nodes
    // (uncaptured, every possible cycle would be enqueued behind flags)
    cudaGraphExec_t& ge = A->rec_graphs[j];
    if (!ge) {
      TCK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      tape_step(ctx, j, true);
      cudaGraph_t g = nullptr;
      TCK(cudaStreamEndCapture(st, &g));
      cudaError_t ce = cudaGraphInstantiate(&ge, g, 0);
      cudaGraphDestroy(g);
      if (ce != cudaSuccess) {
        ge = nullptr;
        return record_error(ctx, DOB_ECUDA, "cudaGraphInstantiate", cudaGetErrorString(ce));
      }
    }
    TCK(cudaGraphLaunch(ge, st));
    step_host_end(ctx);
  }
  cudaMemcpyAsync(s.u, A->Tu[len], N * 4, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(s.v, A->Tv[len], N * 4, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(s.w, A->Tw[len], N * 4, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(s.cen, A->Tcen[len], N * sizeof(float4), cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(s.conc, A->Tc[len], Nc * dye_bytes(ctx), cudaMemcpyDeviceToDevice, st);
  launch_dye_bricks_unknown(s, st);  // the dye came from the tape
  cudaMemcpyAsync(s.pred, A->Tpred[len - 1], Nc * dye_bytes(ctx), cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(s.p, A->Tp, N * 4, cudaMemcpyDeviceToDevice, st);
  if (mixed(ctx)) cudaMemcpyAsync(s.plo, A->Tplo, N * 4, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(s.rhs, A->Trhs, N * 4, cudaMemcpyDeviceToDevice, st);
  return DOB_OK;
}

template <class T> void swap3(T& a, T& b, T& c, T& d, T& e, T& f) {
  std::swap(a, d); std::swap(b, e); std::swap(c, f);
}

// Adjoint of recorded step j of the current segment (reverse stage order).
void backward_step(dob_ctx* ctx, int j) {
  AdjCtx* A = ctx->adj;
  AdjState& a = A->a;
  const DevState& s = ctx->s;
  const size_t N = s.g.n(), Nc = s.gc.n();
  cudaStream_t st = ctx->stream;
  DevState t = s;
  // dye: resolve then predict, linearised at (dye_j, pred_j, cen_{j+1})
  std::swap(a.ac, a.ac2);
  cudaMemsetAsync(a.ac, 0, Nc * 4, st);
  t.conc = A->Tc[j]; t.pred = A->Tpred[j]; t.cen = A->Tcen[j + 1];
  launch_adj_conc_resolve(t, a, st);
  cudaMemsetAsync(a.ac2, 0, Nc * 4, st);
  launch_adj_conc_predict(t, a, st);
  cudaMemsetAsync(a.apred, 0, Nc * 4, st);
  // centre velocity of u_{j+1}: both this step's dye stages and the next
  // step's advection read it
  launch_adj_mac_to_center(t, a, st);
  cudaMemsetAsync(a.acen, 0, N * sizeof(float4), st);
  // projection, pressure solve (warm start from p_j), divergence
  launch_adj_project(t, a, st);
  launch_adj_pressure_solve(t, a, st);
  launch_adj_mac_rhs(t, a, st);
  cudaMemsetAsync(a.arhs, 0, N * 4, st);
  // Casson viscosity, linearised at (u after advection, dye_j)
  swap3(a.au, a.av, a.aw, a.au2, a.av2, a.aw2);
  for (float* p : {a.au, a.av, a.aw}) cudaMemsetAsync(p, 0, N * 4, st);
  t.u = A->Tua[j]; t.v = A->Tva[j]; t.w = A->Twa[j]; t.conc = A->Tc[j];
  launch_adj_casson(t, a, st);
  // advection, linearised at (u_j, cen_j)
  swap3(a.au, a.av, a.aw, a.au2, a.av2, a.aw2);
  for (float* p : {a.au, a.av, a.aw}) cudaMemsetAsync(p, 0, N * 4, st);
  t.u = A->Tu[j]; t.v = A->Tv[j]; t.w = A->Tw[j]; t.cen = A->Tcen[j];
  launch_adj_advect_mac(t, a, st);
  for (float* p : {a.au2, a.av2, a.aw2}) cudaMemsetAsync(p, 0, N * 4, st);
}

}  // namespace

namespace dob {
bool adjoint_field(dob_ctx* ctx, int field, void** dev, size_t* count, int* kind) {
  if (field < DOB_FIELD_ADJ_VEL_U || field > DOB_FIELD_ADJ_RHS) return false;
  if (need_box_fp32(ctx, "adjoint field") != DOB_OK) return false;
  if (ensure_adj(ctx) != DOB_OK) return false;
  const AdjState& a = ctx->adj->a;
  const size_t N = ctx->s.g.n(), Nc = ctx->s.gc.n();
  *kind = 2;
  switch (field) {
    case DOB_FIELD_ADJ_VEL_U: *dev = a.au; *count = N; return true;
    case DOB_FIELD_ADJ_VEL_V: *dev = a.av; *count = N; return true;
    case DOB_FIELD_ADJ_VEL_W: *dev = a.aw; *count = N; return true;
    case DOB_FIELD_ADJ_VEL_U2: *dev = a.au2; *count = N; return true;
    case DOB_FIELD_ADJ_VEL_V2: *dev = a.av2; *count = N; return true;
    case DOB_FIELD_ADJ_VEL_W2: *dev = a.aw2; *count = N; return true;
    case DOB_FIELD_ADJ_CENTER: *dev = a.acen; *count = 4 * N; return true;
    case DOB_FIELD_ADJ_CONC: *dev = a.ac; *count = Nc; return true;
    case DOB_FIELD_ADJ_CONC2: *dev = a.ac2; *count = Nc; return true;
    case DOB_FIELD_ADJ_PRED: *dev = a.apred; *count = Nc; return true;
    case DOB_FIELD_ADJ_PRESSURE: *dev = a.ap; *count = N; *kind = 4; return true;
    case DOB_FIELD_ADJ_RHS: *dev = a.arhs; *count = N; *kind = 4; return true;
    default: return false;
  }
}
}  // namespace dob


extern "C" {

dob_status dob_adjoint_stage(dob_ctx* ctx, int stage) {
  if (!ctx) return DOB_EINVAL;
  dob_status st = need_box_fp32(ctx, "dob_adjoint_stage");
  if (st != DOB_OK) return st;
  if ((st = ensure_adj(ctx)) != DOB_OK) return st;
  const DevState& s = ctx->s;
  const AdjState& a = ctx->adj->a;
  cudaStream_t cs = ctx->stream;
  switch (stage) {
    case DOB_STAGE_ADVECT_MAC: launch_adj_advect_mac(s, a, cs); break;
    case DOB_STAGE_MAC_TO_CENTER: launch_adj_mac_to_center(s, a, cs); break;
    case DOB_STAGE_CASSON_FORCES: launch_adj_casson(s, a, cs); break;
    case DOB_STAGE_MAC_RHS: launch_adj_mac_rhs(s, a, cs); break;
    case DOB_STAGE_PRESSURE_SOLVE: launch_adj_pressure_solve(s, a, cs); break;
    case DOB_STAGE_PROJECT: launch_adj_project(s, a, cs); break;
    case DOB_STAGE_CONC_PREDICT: launch_adj_conc_predict(s, a, cs); break;
    case DOB_STAGE_CONC_RESOLVE: launch_adj_conc_resolve(s, a, cs); break;
    default: return record_error(ctx, DOB_EINVAL, "dob_adjoint_stage", "stage has no adjoint");
  }
  TCK(cudaGetLastError());
  TCK(cudaStreamSynchronize(cs));
  return DOB_OK;
}

dob_status dob_tape_forward(dob_ctx* ctx, int nsteps, int checkpoint_every) {
  if (!ctx) return DOB_EINVAL;
  dob_status st = need_box_fp32(ctx, "dob_tape_forward");
  if (st != DOB_OK) return st;
  if (nsteps < 1 || checkpoint_every < 1 || checkpoint_every > 4096)
    return record_error(ctx, DOB_EINVAL, "dob_tape_forward", "need nsteps >= 1 and 1 <= checkpoint_every <= 4096");
  if ((st = ensure_adj(ctx)) != DOB_OK) return st;
  const int k = checkpoint_every;
  const int nseg = (nsteps + k - 1) / k;
  if ((st = ensure_tape(ctx, k, nseg)) != DOB_OK) return st;
  AdjCtx* A = ctx->adj;
  A->recorded = false;
  A->last_in_slots = false;
  // every recorded step runs mg_cycles V-cycles, as the recomputation does
  ctx->inject_pending = 0;
  TCK(cudaStreamSynchronize(ctx->stream));
  launch_mac_to_center(ctx->s, ctx->stream);
  const int last = (nseg - 1) * k;  // first step of the last segment
  for (int n = 0; n < last; ++n) {
    if (n % k == 0) save_checkpoint(ctx, n / k);
    st = dob_step(ctx, 1, 0, nullptr);
    if (st != DOB_OK) return st;
  }
  save_checkpoint(ctx, nseg - 1);
  st = record_last_segment(ctx, nseg - 1, nsteps - last);
  if (st != DOB_OK) return st;
  TCK(cudaGetLastError());
  TCK(cudaStreamSynchronize(ctx->stream));
  A->nsteps = nsteps;
  A->recorded = true;
  A->last_in_slots = true;
  return DOB_OK;
}

dob_status dob_tape_backward(dob_ctx* ctx, const float* dye_grad, size_t bytes) {
  if (!ctx || !dye_grad) return DOB_EINVAL;
  AdjCtx* A = ctx->adj;
  if (!A || !A->recorded) return record_error(ctx, DOB_ESTATE, "dob_tape_backward", "no recorded forward");
  const DevState& s = ctx->s;
  const size_t Nc = s.gc.n();
  if (bytes != Nc * sizeof(float)) return record_error(ctx, DOB_EINVAL, "dob_tape_backward", "byte count != dye grid");
  cudaStream_t st = ctx->stream;
  zero_adj(s, A->a, st);
  TCK(cudaMemcpyAsync(A->a.ac, dye_grad, bytes, cudaMemcpyHostToDevice, st));
  const int k = A->k;
  const int nseg = (A->nsteps + k - 1) / k;
  if (A->seg_graphs.size() != (size_t)(4 * (k + 1))) {
    A->drop_graphs();
    A->seg_graphs.assign(4 * (k + 1), nullptr);
  }
  for (int seg = nseg - 1; seg >= 0; --seg) {
    const int len = (seg == nseg - 1) ? A->nsteps - seg * k : k;
    // the last segment's points are still in the slots after dob_tape_forward
    const bool recompute = !(seg == nseg - 1 && A->last_in_slots);
    if (recompute) restore_checkpoint(ctx, seg);
    // The segment's launches only depend on (len, which dye adjoint buffer is
    // current, recomputation or not): capture them once as a graph and
    // replay it.
    const int parity = A->a.ac < A->a.ac2 ? 0 : 1;
    cudaGraphExec_t& ge = A->seg_graphs[(recompute ? 0 : 2 * (k + 1)) + 2 * len + parity];
    const AdjState before = A->a;
    if (!ge) {
      TCK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      if (recompute) replay_segment(ctx, len);
      for (int j = len - 1; j >= 0; --j) backward_step(ctx, j);
      cudaGraph_t g = nullptr;
      TCK(cudaStreamEndCapture(st, &g));
      cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) {
        ge = nullptr;
        return record_error(ctx, DOB_ECUDA, "cudaGraphInstantiate", cudaGetErrorString(e));
      }
      // capturing applied the segment's buffer swaps to the host copy;
      // start from the pre-capture assignment and replay the graph
      A->a = before;
    }
    TCK(cudaGraphLaunch(ge, st));
    // the swaps the segment performs: dye adjoint ping-pong once per step,
    // velocity adjoints twice per step (net none)
    if (len & 1) std::swap(A->a.ac, A->a.ac2);
    if (recompute) A->last_in_slots = false;  // the slots now hold this segment
  }
  TCK(cudaGetLastError());
  // the trajectory starts from cen = C(u(0))
  DevState t = s;
  launch_adj_mac_to_center(t, A->a, st);
  TCK(cudaMemsetAsync(A->a.acen, 0, s.g.n() * sizeof(float4), st));
  TCK(cudaGetLastError());
  TCK(cudaStreamSynchronize(st));
  return DOB_OK;
}

dob_status dob_adjoint_sphere_impulse(dob_ctx* ctx, const float center[3], float radius, const float vel[3],
                                      double* out) {
  if (!ctx || !center || !vel || !out) return DOB_EINVAL;
  dob_status st = need_box_fp32(ctx, "dob_adjoint_sphere_impulse");
  if (st != DOB_OK) return st;
  if ((st = ensure_adj(ctx)) != DOB_OK) return st;
  const AdjState& a = ctx->adj->a;
  launch_sphere_impulse(ctx->s, a.au, a.av, a.aw, center, radius, vel, ctx->adj->dred, ctx->stream);
  TCK(cudaGetLastError());
  TCK(cudaMemcpyAsync(out, ctx->adj->dred, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  TCK(cudaStreamSynchronize(ctx->stream));
  return DOB_OK;
}

dob_status dob_adjoint_sphere_soft(dob_ctx* ctx, const float center[3], float radius, float edge, float dye,
                                   const float vel[3], float noise_sigma, uint64_t seed, double out[4]) {
  if (!ctx || !center || !vel || !out) return DOB_EINVAL;
  dob_status st = need_box_fp32(ctx, "dob_adjoint_sphere_soft");
  if (st != DOB_OK) return st;
  if (!(radius > 0.0f) || !(edge > 0.0f) || !isfinite(radius) || !isfinite(edge) || !isfinite(dye) ||
      !isfinite(noise_sigma))
    return record_error(ctx, DOB_EINVAL, "dob_adjoint_sphere_soft", "bad radius/edge/dye/sigma");
  if ((st = ensure_adj(ctx)) != DOB_OK) return st;
  const AdjState& a = ctx->adj->a;
  launch_sphere_soft_grad(ctx->s, a.au, a.av, a.aw, a.ac, center, radius, edge, dye, vel, noise_sigma, seed,
                          ctx->adj->dred, ctx->stream);
  TCK(cudaGetLastError());
  TCK(cudaMemcpyAsync(out, ctx->adj->dred, 4 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  TCK(cudaStreamSynchronize(ctx->stream));
  return DOB_OK;
}

}  // extern "C"
