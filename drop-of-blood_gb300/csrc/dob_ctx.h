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

struct Snapshot {
  std::vector<void*> bufs;
  std::vector<size_t> sizes;
  uint32_t high_water = 0;
  int step_index = 0;
  bool valid = false;
};

struct AdjCtx;  // discrete-adjoint buffers and tape (dob_tape.cu)

}  // namespace dob

struct dob_ctx {
  dob_config cfg;
  dob::DevState s;
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t aux_stream = nullptr;  // body capture of conditional graph nodes
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
    void *conc = nullptr, *u = nullptr;
    void* after[8] = {};  // u, v, w, u2, v2, w2, conc, conc2
  } graphs[8];
  int graph_next = 0;  // round-robin replacement when all slots are taken
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
  } async_slots[8];
};

namespace dob {
// Error recording for dob_last_error (dob_api.cu).
dob_status record_error(dob_ctx* ctx, dob_status st, const char* what, const char* detail);
// Adjoint state (dob_tape.cu): release with the context; field lookup for
// dob_set_field / dob_get_field (kind 2: FP32 natural, 4: FP32 split).
void adjoint_free(dob_ctx* ctx);
bool adjoint_field(dob_ctx* ctx, int field, void** dev, size_t* count, int* kind);
}  // namespace dob
