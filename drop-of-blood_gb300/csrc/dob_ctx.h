// dob_ctx.h — the context behind the opaque dob_ctx handle of the C ABI
// (internal: shared by the translation units that implement the ABI).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "dob_kernels.cuh"

namespace dob {

constexpr int kParamRing = 16;
constexpr int kSnapshots = 8;
// Steps after an injection that run cfg.mg_cycles_injected V-cycles: the
// injection step itself and the next, whose right-hand side still carries
// most of the new drop's divergence (the warm start from the injection
// step's pressure leaves max |div| near 7e-5 after 4 V-cycles at 192 x 256
// x 192; the third step is back below 2e-6).
constexpr int kInjectedSteps = 2;

struct Snapshot {
  std::vector<void*> bufs;
  std::vector<size_t> sizes;
  uint32_t high_water = 0;
  int step_index = 0;
  int inject_pending = 0;
  bool valid = false;
};

struct AdjCtx;  // discrete-adjoint buffers and tape (dob_tape.cu)

}  // namespace dob

struct dob_ctx {
  dob_config cfg;
  dob::DevState s;
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t aux_stream = nullptr;   // body capture of conditional graph nodes
  cudaStream_t aux_stream2 = nullptr;  // the same, one nesting level up
  std::string err;
  float U[128];
  dob::StepParams* host_params = nullptr;  // pinned ring
  cudaEvent_t param_ev[dob::kParamRing];
  int param_slot = 0;
  uint32_t high_water = 0;
  int step_index = 0;
  std::vector<void*> allocs;
  uint64_t bytes = 0;
  // Captured step graphs, keyed by statistics on/off and the ping-pong
  // buffers current at capture (dye and velocity alternate between steps);
  // `after` holds the ping-pong pointers the captured step leaves behind.
  struct StepGraph {
    cudaGraphExec_t ex = nullptr;
    bool stats = false;
    bool injected = false;  // captured with mg_cycles_injected V-cycles
    void *conc = nullptr, *u = nullptr;
    void* after[8] = {};  // u, v, w, u2, v2, w2, conc, conc2
  } graphs[12];
  int graph_next = 0;  // round-robin replacement when all slots are taken
  // steps left that run cfg.mg_cycles_injected V-cycles (when set and the
  // pressure is FP32): an injection sets kInjectedSteps
  int inject_pending = 0;
  int last_cycles = 0;  // V-cycles of the last step (FP32 pressure)
  uint32_t stats_mask = DOB_STATS_ALL;  // statistics a DOB_STEP_STATS step forms
  int kernels_per_step = 0;
  dob::Snapshot snaps[dob::kSnapshots];
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t stage_ev[DOB_STAGE_COUNT + 1];
  dob::AdjCtx* adj = nullptr;
  // results of dob_step_async: pinned statistics slots and their events
  struct AsyncSlot {
    double* red = nullptr;        // pinned, RED_COUNT
    unsigned int* redu = nullptr; // pinned, REDU_COUNT
    cudaEvent_t done = nullptr;
    bool pending = false;
    int cycles = 0;               // V-cycles of the step (FP32 pressure)
  } async_slots[8];
  // plume render (dob_render_plume): the caller's spectral table (256 x 64
  // float4) and the image buffer (8 halves per pixel), grown on demand
  float4* lut = nullptr;
  __half* image = nullptr;
  size_t image_cap = 0;
  int render_w = 0, render_h = 0;  // the last render's size (dob_bench_kernel 3)
};

namespace dob {
// Error recording for dob_last_error (dob_api.cu).
dob_status record_error(dob_ctx* ctx, dob_status st, const char* what, const char* detail);
// Adjoint state (dob_tape.cu): release with the context; field lookup for
// dob_set_field / dob_get_field (kind 2: FP32 natural, 4: FP32 split).
void adjoint_free(dob_ctx* ctx);
bool adjoint_field(dob_ctx* ctx, int field, void** dev, size_t* count, int* kind);
// A closed-box step enqueued by its caller (dob_api.cu): step_host_begin
// (parameters, bookkeeping), the caller's body with enqueue_parcel_stages
// after the projection, then step_host_end.
dob_status step_host_begin(dob_ctx* ctx);
void enqueue_parcel_stages(dob_ctx* ctx, DevState& s, cudaStream_t st);
void step_host_end(dob_ctx* ctx);
}  // namespace dob
