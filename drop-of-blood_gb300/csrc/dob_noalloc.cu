// dob_noalloc.cu — dob_pressure_solve_noalloc: the multigrid pressure solve
// for callers that cannot allocate device memory.
//
// Some hosts own every byte of device memory themselves: an engine whose
// allocator reserves the whole GPU up front, a plugin loaded into such an
// engine, or a frame loop that must not call cudaMalloc/cudaFree because both
// synchronise the device and can fail mid-frame.  They still want the
// library's V-cycle on buffers they already hold.  This entry point gives it
// to them: the caller passes the right-hand side and the pressure (device
// pointers, natural x-fastest layout); every other array the V-cycle needs —
// the red-black split copies of both, the correction and right-hand side of
// every coarser grid, the FP64 reduction slots — lives in one fixed
// file-scope device array below.  No call here allocates device or pinned
// memory, directly or through a library.
//
// Limits and sharing rules:
//   * at most kNoAllocMaxCells = 2^21 cells (e.g. the reference's 96x128x96
//     grid, or 128^3); larger grids are rejected with DOB_EINVAL;
//   * the array (about 40 MiB) is part of the library's device image: every
//     GPU that loads the library holds it until the process exits;
//   * every call, from any thread and on any stream, works in the same array
//     and leaves the last call's contents there.  Two calls whose work overlaps
//     on the GPU (different streams without ordering, or different host
//     threads) race and corrupt each other's results; order them on one
//     stream;
//   * the first call on each device does a one-time set-up with that device
//     current: it looks up the array's device address with
//     cudaGetSymbolAddress and raises the coarse-grid kernel's shared-memory
//     limit.  Make that first call before any stream capture;
//   * with an exact coarsest solve (mg_coarse_sweeps = -1), a call whose
//     coarsest grid differs from the one the array's inverse was made for
//     (its dims, the boundary mode, or its spacing, i.e. the number of
//     coarsenings) recomputes that inverse on the host and uploads it,
//     waiting for the caller's stream to drain; such a call blocks the host
//     and must not be made during stream capture.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <mutex>
#include <vector>

#include "dob_kernels.cuh"

namespace dob {
// Records an error for dob_last_error(NULL) (defined with the other entry
// points in dob_api.cu).
dob_status record_static_error(dob_status st, const char* what, const char* detail);
}  // namespace dob

using namespace dob;

namespace {

constexpr size_t kNoAllocMaxCells = size_t(1) << 21;
constexpr size_t kAlign = 256;
constexpr size_t kSlotBytes = 1024;  // FP64 + u32 reduction slots at the front
constexpr size_t kPartBytes = PART_SLOTS * kSumBlocks * sizeof(double);  // mean-removal partials
// Layout for n cells: slots, partials, split p (4n), split rhs (4n), then correction and
// right-hand side of every coarser grid, each rounded up to 256 bytes.  The
// coarser grids hold fewer than n/7 cells together, so 10 bytes per cell
// bounds the whole layout for every accepted grid.
// The dense inverse of an exactly solved coarsest grid (up to
// kNoAllocDenseMax cells, the closed-box configuration's target) follows the
// multigrid arrays.
constexpr int kNoAllocDenseMax = kDenseCoarseTarget;
constexpr size_t kDenseBytes = (size_t)kNoAllocDenseMax * kNoAllocDenseMax * sizeof(float);
constexpr size_t kScratchBytes = kSlotBytes + kPartBytes + 10 * kNoAllocMaxCells + kDenseBytes;

static_assert(RED_COUNT * sizeof(double) <= 512, "reduction slots exceed their area");
static_assert(REDU_COUNT * sizeof(unsigned int) <= kSlotBytes - 512, "flag slots exceed their area");

// The scratch array.  In host code this name is only a handle for
// cudaGetSymbolAddress; its device address comes from that call.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_ptr[kMaxDevices] = {};
int g_num_sms[kMaxDevices] = {};
// Which coarsest-grid inverse each device's array holds: the grid's dims, the
// boundary mode and the bits of the level's h^2 (the inverse is scaled by it,
// and h^2 depends on how many coarsenings lead to the grid: 48x64x48 with 3
// grids and 96x128x96 with 4 both end at 12x16x12, with h^2 16 and 64).
constexpr int kInvKey = 5;
int g_inv_key[kMaxDevices][kInvKey] = {};

size_t round_up(size_t b) { return (b + kAlign - 1) / kAlign * kAlign; }

dob_status bad(const char* detail) { return record_static_error(DOB_EINVAL, "dob_pressure_solve_noalloc", detail); }

dob_status cuda_fail(const char* what, cudaError_t e) {
  cudaGetLastError();
  return record_static_error(DOB_ECUDA, what, cudaGetErrorString(e));
}

bool is_device_pointer(const void* p, int device) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) && a.device == device;
}

// One-time set-up of the current device (guarded by g_setup_mutex).
dob_status setup_device(int device) {
  if (g_scratch_ptr[device]) return DOB_OK;
  void* ptr = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
  if (e != cudaSuccess) return cuda_fail("cudaGetSymbolAddress(g_noalloc_scratch)", e);
  int sms = 0;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return cuda_fail("cudaDeviceGetAttribute", e);
  e = mg_prepare();
  if (e != cudaSuccess) return cuda_fail("mg_prepare", e);
  g_num_sms[device] = sms;
  g_scratch_ptr[device] = ptr;
  return DOB_OK;
}

}  // namespace

extern "C" dob_status dob_pressure_solve_noalloc(const dob_config* cfg, const float* rhs, float* pressure,
                                                 void* stream) {
  if (!cfg) return bad("null config");
  if (cfg->struct_size != sizeof(dob_config)) return bad("struct_size mismatch");
  if (!rhs || !pressure) return bad("null buffer");
  if (((uintptr_t)rhs | (uintptr_t)pressure) & 3) return bad("buffers must be 4-byte aligned");
  const uint32_t nx = cfg->nx, ny = cfg->ny, nz = cfg->nz;
  if (nx < 4 || ny < 4 || nz < 4) return bad("grid dims must be >= 4");
  if (nx % 2 || ny % 2 || nz % 2) return bad("grid dims must be even");
  if (nx > 2048 || ny > 2048 || nz > 2048) return bad("grid dims must be <= 2048");
  const size_t n = (size_t)nx * ny * nz;
  if (n > kNoAllocMaxCells)
    return bad("grid larger than the fixed scratch array allows (at most 2^21 = 2097152 cells)");
  if (cfg->mg_levels < 1 || cfg->mg_levels > kMaxLevels) return bad("mg_levels out of range");
  const uint32_t m = 1u << cfg->mg_levels;
  if (nx % m || ny % m || nz % m)
    return bad("dims not divisible by 2^mg_levels (every multigrid level needs even dims)");
  if (cfg->bc_mode != DOB_BC_REFERENCE && cfg->bc_mode != DOB_BC_CLOSED_BOX) return bad("bad bc_mode");
  if (cfg->precision_mode == DOB_PREC_MIXED)
    return bad("the mixed-precision solve is not available without allocation; use DOB_PREC_FP32");
  if (cfg->precision_mode != DOB_PREC_FP32 && cfg->precision_mode != DOB_PREC_REFERENCE_FP16)
    return bad("bad precision_mode");
  if (cfg->mg_pre < 0 || cfg->mg_post < 0 || cfg->mg_coarse_sweeps < -1 || cfg->mg_cycles < 0)
    return bad("negative sweeps");
  const int cl = cfg->mg_levels - 1;
  if (cfg->mg_coarse_sweeps == -1 &&
      (uint64_t)(nx >> cl) * (ny >> cl) * (nz >> cl) > (uint64_t)kNoAllocDenseMax)
    return bad("mg_coarse_sweeps = -1 (exact coarsest solve) needs a coarsest grid of at most 2304 cells");

  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return cuda_fail("cudaGetDevice", e);
  if (device < 0 || device >= kMaxDevices) return bad("device ordinal beyond the supported 64");
  if (!is_device_pointer(rhs, device) || !is_device_pointer(pressure, device))
    return bad("rhs and pressure must be device memory of the current device");
  void* base = nullptr;
  int num_sms = 0;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    const dob_status st = setup_device(device);
    if (st != DOB_OK) return st;
    base = g_scratch_ptr[device];
    num_sms = g_num_sms[device];
  }

  // Carve the scratch array: the same hierarchy dob_create allocates.
  DevState s;
  memset(&s, 0, sizeof(s));
  s.g = make_grid((int)nx, (int)ny, (int)nz);
  s.prec = DOB_PREC_FP32;
  s.ref = cfg->bc_mode == DOB_BC_REFERENCE;
  s.num_sms = num_sms;
  unsigned char* cur = static_cast<unsigned char*>(base);
  s.red = reinterpret_cast<double*>(cur);
  s.redu = reinterpret_cast<unsigned int*>(cur + 512);
  s.part = reinterpret_cast<double*>(cur + kSlotBytes);
  size_t used = kSlotBytes + kPartBytes;
  auto take = [&](size_t cells) {
    float* p = reinterpret_cast<float*>(cur + used);
    used += round_up(cells * sizeof(float));
    return p;
  };
  s.p = take(n);
  s.rhs = take(n);
  s.nlev = cfg->mg_levels;
  for (int l = 0; l < s.nlev; ++l) {
    MgLevel& L = s.lv[l];
    L.d = make_grid(s.g.nx >> l, s.g.ny >> l, s.g.nz >> l);
    const float sc = (float)s.g.nx / (float)L.d.nx;
    L.h2 = sc * sc;
    if (l == 0) {
      L.e = s.p;
      L.b = s.rhs;
      continue;
    }
    L.e = take(L.d.n());
    L.b = take(L.d.n());
  }
  if (cfg->mg_coarse_sweeps < 0) {
    // The coarsest grid's inverse sits at the end of the array.  It is
    // recomputed on the host and uploaded only when its key (dims, boundary
    // mode, h^2) differs from the one the array holds; that upload waits for
    // the caller's stream (see the header).
    const MgLevel& C = s.lv[s.nlev - 1];
    float* inv = reinterpret_cast<float*>(cur + kScratchBytes - kDenseBytes);
    int h2_bits = 0;
    memcpy(&h2_bits, &C.h2, sizeof(h2_bits));
    const int key[kInvKey] = {C.d.nx, C.d.ny, C.d.nz, s.ref, h2_bits};
    bool same = true;
    {
      std::lock_guard<std::mutex> lock(g_setup_mutex);
      for (int k = 0; k < kInvKey; ++k) same = same && g_inv_key[device][k] == key[k];
    }
    if (!same) {
      const std::vector<float> h = coarse_inverse(C.d, C.h2, s.ref);
      e = cudaMemcpyAsync(inv, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice,
                          static_cast<cudaStream_t>(stream));
      if (e == cudaSuccess) e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
      if (e != cudaSuccess) return cuda_fail("coarse inverse upload", e);
      std::lock_guard<std::mutex> lock(g_setup_mutex);
      for (int k = 0; k < kInvKey; ++k) g_inv_key[device][k] = key[k];
    }
    s.cinv = inv;
    s.cn = (int)C.d.n();
  }
  if (used > kScratchBytes - kDenseBytes) return bad("internal: scratch layout exceeds the array");
  s.pre0 = cfg->reference_schedule ? 1 : cfg->mg_pre;
  s.post0 = cfg->reference_schedule ? 1 : cfg->mg_post;
  s.pre = cfg->mg_pre;
  s.post = cfg->mg_post;
  s.coarse_sweeps = cfg->mg_coarse_sweeps;
  s.cycles = cfg->mg_cycles;

  // The previous call's contents are still in the array.  The split copies
  // and coarse right-hand sides are overwritten in full and every coarse
  // correction is zero-filled before its first sweep; the reduction slots are
  // cleared here.
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  e = cudaMemsetAsync(base, 0, kSlotBytes, st);
  if (e != cudaSuccess) return cuda_fail("cudaMemsetAsync", e);
  launch_split(rhs, s.rhs, s.g, true, st);
  launch_split(pressure, s.p, s.g, true, st);
  launch_pressure_solve(s, st);
  launch_split(s.p, pressure, s.g, false, st);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail("dob_pressure_solve_noalloc launch", e);
  return DOB_OK;
}
