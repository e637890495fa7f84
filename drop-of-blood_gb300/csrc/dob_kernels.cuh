// dob_kernels.cuh — device state of one context and the launchers of every
// kernel of the step (one .cu file per kernel family).
#pragma once

#include <cuda_runtime.h>

#include <utility>
#include <vector>

#include "../../include/dropfluid.h"
#include "dob_device.cuh"

namespace dob {

constexpr int kMaxLevels = 10;

// One grid of the multigrid hierarchy.  Level 0 reuses the pressure / rhs
// arrays; every level owns a residual-free layout (residual + restriction are
// fused, so no residual array exists).
struct MgLevel {
  Grid d;
  float h2;
  float* e;            // correction (levels >= 1), FP32
  float* b;            // right-hand side (levels >= 1), FP32
  __nv_bfloat16* eh;   // BF16 arrays used by the mixed-precision inner solve
  __nv_bfloat16* bh;
};

// Red-black split index of cell (x,y,z): colour c = (x+y+z)&1 selects the
// half, and inside a half the cells are row-major with x/2 fastest.  Every
// multigrid array (p, rhs, corrections) is stored this way.
__host__ __device__ __forceinline__ size_t rb_index(const Grid& d, int x, int y, int z) {
  const size_t half = d.n() >> 1;
  return (size_t)((x + y + z) & 1) * half + ((size_t)z * d.ny + y) * (size_t)(d.nx >> 1) + (size_t)(x >> 1);
}

struct DevState {
  Grid g;    // velocity / pressure grid
  Grid gc;   // dye grid
  int prec;  // DOB_PREC_*
  int ref;   // reference boundary conditions
  int flags; // DOB_PHYS_* (reference mode only)
  int num_sms;
  StepParams* params;            // device copy of this step's parameters
  void *u, *v, *w, *u2, *v2, *w2;  // MAC faces (VS)
  void *cen, *curl;              // 4 x VS AoS
  float *p, *rhs;                // red-black split layout (rb_index)
  void *conc, *conc2, *pred;     // dye (DS)
  void* lim;                     // closed box: the predictor's tap minimum and maximum (2 x DS per cell)
  uint32_t *splatI, *splatL;
  float4* wave;
  float2* wspec;                 // wave solver (DOB_PHYS_WAVE): 512x512 complex spectra
  float* wfilm;                  // wave solver: the force pass's surfactant film
  float* parcels;
  uint32_t cap;
  // sparse dye bricks (k_fluid.cu): per 8x8x8 brick of the dye grid,
  // whether the predictor (reference mode) / a dye buffer (its lysed
  // channel in reference mode) holds a nonzero value; concA and concB are
  // the buffers cbrickA and cbrickB belong to (conc and conc2 swap every
  // step, the flags stay with their buffer; other dye arrays have none)
  const void *concA, *concB;
  uint32_t *cbrickA, *cbrickB, *pbrick;
  // per 8x8x8 brick of the dye grid, whether the splat accumulators may
  // hold a nonzero sum there (set by every splat, cleared with the bricks)
  uint32_t* sbrick;
  // light volume (reference mode, dims divisible by 4): 4 x binary16 per
  // velocity cell, and the raw and dilated occupancy of its 4x4x4 bricks
  half4* light;
  float *brick_raw, *bricks;
  double* red;                   // FP64 reduction slots
  double* part;                  // per-block partials of the mean removals: PART_SLOTS x kSumBlocks
  unsigned int* redu;            // u32 reduction slots / flags
  int nlev;
  MgLevel lv[kMaxLevels];
  int pre0, post0, pre, post, coarse_sweeps, cycles;
  // exact coarsest-grid solve (coarse_sweeps < 0): the symmetric (pseudo-)
  // inverse of the coarsest operator, n x n FP32, natural cell order
  const float* cinv;
  int cn;
  // mixed-precision defect correction: the pressure is the unevaluated sum
  // p + plo of two FP32 arrays (double-float); the correction solve runs on
  // e0 / r0 (FP32, split layout) with BF16 storage from level kMixedBF16Level
  float* plo;
  float *e0, *r0;
  int max_outer;
  double rel_tol;   // stop when ||b - A p|| <= rel_tol ||b|| (0: off)
  float div_tol_r;  // stop when max |b - A p| <= div_tol_r (0: off)
  // second and third streams of the context: capture the bodies of the
  // defect loop's conditional nodes (a round's while-node of V-cycles, the
  // if-node of a round after the first) when the step is captured
  cudaStream_t aux, aux2;
};
constexpr int kMixedBF16Level = 2;

// Adjoint (transpose-Jacobian) arrays of the closed-box FP32 step, all FP32.
// Pressure / right-hand side / multigrid adjoints are red-black split like
// their forward arrays; the rest use the natural layout.
struct AdjState {
  float *au, *av, *aw;     // adjoint of the MAC faces a stage reads
  float *au2, *av2, *aw2;  // adjoint of the faces advection / Casson write
  float4* acen;            // adjoint of the centre velocity (x, y, z, unused)
  float *ac, *ac2, *apred; // dye (input), resolved dye (output), predictor
  float *ap, *arhs;        // pressure, right-hand side (split)
  float* le[kMaxLevels];   // coarse corrections (split, levels >= 1)
  float* lb[kMaxLevels];   // coarse right-hand sides (split, levels >= 1)
  float *alpha, *gq;       // Casson adjoint scratch: per-cell alpha, 2 dL/dQ
  double* part;            // partial sums of the mean removals: 2 x kSumBlocks
  float *lam, *lamlo;      // mixed mode: adjoint pressure solve's solution pair (split)
  double* red;             // FP64 reduction slots (mean removal)
};
// relative residual of the mixed mode's adjoint pressure solve
constexpr double kAdjRelTol = 1e-6;

// reduction slot indices in DevState::red / redu
enum {
  RED_RHS_SUM = 0,
  RED_P_SUM = 1,
  RED_RHS_NORM2 = 2,
  RED_RES_NORM2 = 3,
  RED_DEFECT_NORM2 = 4,   // ||r||^2: [0] the mixed round's residual, [1] the cycle's
  RED_COUNT = 4 + 32
};
enum {
  REDU_MAXDIV = 0,
  REDU_ALIVE = 1,
  REDU_DONE = 2,          // defect loop converged (kernels of later iterations exit)
  REDU_ITERS = 3,         // mixed solve: rounds that corrected the pressure
  REDU_INNER_DONE = 4,    // mixed solve: the round's V-cycles have converged (their kernels exit)
  REDU_VCYCLES = 5,       // mixed solve: V-cycles completed in the step
  REDU_INNER_ITERS = 6,   // mixed solve: V-cycles begun in the current round
  REDU_SPEED = 7,         // closed-box step: max |centre velocity| per axis after the projection (float bits)
  REDU_DEFECT_MAX = 8,    // max |r| (float bits): [0] the round's residual, [1] the cycle's
  REDU_COUNT = 8 + 32
};
// the reduction slots as one block: RED_COUNT doubles, then REDU_COUNT u32
constexpr size_t kStatsBytes = RED_COUNT * sizeof(double) + REDU_COUNT * sizeof(unsigned int);
// the mixed solve: at most this many rounds (error-free residuals) per step,
// and V-cycles per round
constexpr int kMixedMaxRounds = 4;
constexpr int kMixedMaxCycles = 16;

// ---- block reductions ---------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_maxf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
// ---- programmatic dependent launch -------------------------------------------
// The multigrid kernels form long chains of small dependent launches (about
// 50 per V-cycle, most under 5 us).  Launched with launch_pdl, a kernel may
// be scheduled while its predecessor still runs: pdl_wait() (first statement
// of such a kernel, before any memory access) blocks until the predecessor
// grid has completed and its writes are visible, and pdl_trigger() lets the
// successor's launch begin once every CTA of this grid has started.  Both are
// no-ops for a kernel launched without the attribute.  The wait is the
// hardware grid dependency, not a spin: it ends when the predecessor ends.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
template <class... KArgs, class... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                              Args&&... args) {
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// Deterministic FP64 sums (the mean removals, whose result enters the
// state): each block stores its partial in its own slot of `part`
// (block_sum_store) and the consumer adds the slots in a fixed order
// (sum_partials), so the bits do not depend on the order in which blocks
// finish, as one FP64 atomic per block would.
constexpr int kSumBlocks = 1024;  // most blocks of a partial-sum launch (slots per array)
enum { PART_RHS = 0, PART_P = 1, PART_SLOTS = 2 };
__device__ __forceinline__ void block_sum_store(double v, double* part) {
  __shared__ double wpart[32];
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nthreads = blockDim.x * blockDim.y * blockDim.z;
  v = warp_sum(v);
  if ((tid & 31) == 0) wpart[tid >> 5] = v;
  __syncthreads();
  if (tid < 32) {
    double s = tid < (nthreads + 31) / 32 ? wpart[tid] : 0.0;
    s = warp_sum(s);
    if (tid == 0) part[blockIdx.x] = s;
  }
}
// Sum of part[0, nb) in a fixed order; call from a whole warp (every lane
// gets the same value: strided per-lane sums, then a butterfly).
__device__ __forceinline__ double sum_partials(const double* part, int nb) {
  double s = 0.0;
  for (int i = threadIdx.x & 31; i < nb; i += 32) s += part[i];
  return warp_sum(s);
}
// Sum `v` over the block and add it to *out with one FP64 atomic per block.
__device__ __forceinline__ void block_sum_atomic(double v, double* out) {
  __shared__ double part[32];
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nthreads = blockDim.x * blockDim.y * blockDim.z;
  v = warp_sum(v);
  if ((tid & 31) == 0) part[tid >> 5] = v;
  __syncthreads();
  if (tid < 32) {
    double s = tid < (nthreads + 31) / 32 ? part[tid] : 0.0;
    s = warp_sum(s);
    if (tid == 0 && s != 0.0) atomicAdd(out, s);
  }
}
// Sum of non-negative FP32 values `v` over the block into *out: FP32 within
// each warp, FP64 across warps (one FP64 operation per warp, not per thread:
// GB300's FP64 rate is a small fraction of its FP32 rate).
__device__ __forceinline__ void block_sum_atomic_f(float v, double* out) {
  __shared__ double part[32];
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nthreads = blockDim.x * blockDim.y * blockDim.z;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((tid & 31) == 0) part[tid >> 5] = (double)v;
  __syncthreads();
  if (tid == 0) {
    double s = 0.0;
    for (int w = 0; w < (nthreads + 31) / 32; ++w) s += part[w];
    if (s != 0.0) atomicAdd(out, s);
  }
}
// Max of non-negative floats via their bit patterns.
// Block maximum of unsigned values, one atomicMax per block (the bits of
// |x| order non-negative floats, +inf above them and NaN above +inf).
__device__ __forceinline__ void block_max_u32(unsigned int v, unsigned int* out) {
  __shared__ unsigned int upart[32];
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nthreads = blockDim.x * blockDim.y * blockDim.z;
  v = __reduce_max_sync(0xffffffffu, v);
  if ((tid & 31) == 0) upart[tid >> 5] = v;
  __syncthreads();
  if (tid < 32) {
    unsigned int s = tid < (nthreads + 31) / 32 ? upart[tid] : 0u;
    s = __reduce_max_sync(0xffffffffu, s);
    if (tid == 0 && s != 0u) atomicMax(out, s);
  }
}
__device__ __forceinline__ void block_max_atomic(float v, unsigned int* out) {
  __shared__ float part[32];
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nthreads = blockDim.x * blockDim.y * blockDim.z;
  v = warp_maxf(v);
  if ((tid & 31) == 0) part[tid >> 5] = v;
  __syncthreads();
  if (tid < 32) {
    float s = tid < (nthreads + 31) / 32 ? part[tid] : 0.0f;
    s = warp_maxf(s);
    if (tid == 0 && s > 0.0f) atomicMax(out, __float_as_uint(s));
  }
}

// Instantiate a launch body for the storage types of a precision mode:
//   VS = velocity storage, DS = dye storage.
#define DOB_VEL_DISPATCH(prec, ...)                                                             \
  do {                                                                                          \
    if ((prec) == DOB_PREC_REFERENCE_FP16) { using VS = __half; using DS = __half; __VA_ARGS__; } \
    else if ((prec) == DOB_PREC_MIXED) { using VS = float; using DS = __half; __VA_ARGS__; }      \
    else { using VS = float; using DS = float; __VA_ARGS__; }                                     \
  } while (0)

// ---- launchers (k_fluid.cu) -----------------------------------------------------------
void launch_init_vel(const DevState& s, cudaStream_t st);
void launch_advect_mac(const DevState& s, cudaStream_t st);
void launch_mac_to_center(const DevState& s, cudaStream_t st);
void launch_curl(const DevState& s, cudaStream_t st);
void launch_casson(const DevState& s, cudaStream_t st);
void launch_mac_rhs(const DevState& s, cudaStream_t st);
void launch_project(const DevState& s, cudaStream_t st);
// ---- the 512x512 wave solver (k_wave.cu) -------------------------------------------------
void launch_wave_step(const DevState& s, cudaStream_t st);
// ---- light volume and brick occupancy (k_light.cu) ------------------------------------------
bool light_dims_ok(const Grid& g);
// ---- the plume render (k_render.cu) --------------------------------------------------------
// lut: 256 x 64 float4 (spectral transmittance); out: W x H x 8 halves
void launch_render_plume(const DevState& s, const float4* lut, int W, int H, __half* out, cudaStream_t st);
void launch_light_volume(const DevState& s, cudaStream_t st);
// ---- closed-box column kernels of the step graph (k_box.cu) ------------------------------
// Same results as launch_casson / launch_mac_rhs / launch_project followed by
// launch_mac_to_center.  Casson needs dye on the velocity grid.
bool box_casson_applies(const DevState& s);
void launch_casson_box(const DevState& s, cudaStream_t st);   // u -> u2 (caller swaps)
// sumsq (statistics): the sum of squares of the mean-free right-hand side
void launch_mac_rhs_box(const DevState& s, cudaStream_t st, double* sumsq = nullptr);  // with the zero-mean correction
// projection of (u, v, w) into (u2, v2, w2) and the centre velocity of the
// projected faces, one pass (the caller swaps the buffers)
// maxbits: also max |div| * scale of the projected faces (statistics), as
// launch_divergence forms it; speedbits: also the largest |component| of the
// stored centre velocity (the sparse dye predictor's reach)
void launch_project_center_box(const DevState& s, cudaStream_t st, float scale = 0.0f,
                               unsigned int* maxbits = nullptr, unsigned int* speedbits = nullptr);
void launch_divergence(const DevState& s, float* out, float scale, unsigned int* maxbits, cudaStream_t st);
// reference mode: the projection of (u, v, w) into (u2, v2, w2) and the
// centre velocity of the projected faces (the MAC_TO_CENTER after it), one
// pass (the caller swaps the buffers)
void launch_project_center_ref(const DevState& s, cudaStream_t st);
// bracket: also write the minimum and maximum of the predictor's 8 dye taps
// (closed box) for launch_dye_resolve_lim.  sparse (inside a step, where the
// centre velocity is bounded: by the projection's clamp in reference mode,
// by the projection's s.redu[REDU_SPEED] in the closed box): skip the
// blocks the dye-brick flags show to be clear water (same results).  The
// resolves always maintain the flags of the dye buffer they write.
void launch_conc_predict(const DevState& s, cudaStream_t st, bool bracket = false, bool sparse = false);
void launch_dye_resolve_lim(const DevState& s, cudaStream_t st);
// dye written from outside the step (injection, field I/O, snapshots, the
// tape): every brick of both dye buffers may hold dye until the next resolve
void launch_dye_bricks_unknown(const DevState& s, cudaStream_t st);
// zero the splat accumulators: only the bricks a splat has marked (the
// others hold zeros already), then clear their marks
void launch_clear_splats(const DevState& s, cudaStream_t st);
void launch_conc_resolve(const DevState& s, cudaStream_t st, bool sparse = false);
// number of 8x8x8 dye bricks (one uint32 flag each)
size_t dye_brick_count(const Grid& gc);

// Largest coarsest grid solved exactly by the dense inverse (64 MB of FP32),
// and the size the closed-box configuration deepens its hierarchy to: one
// dense solve of up to 12 x 16 x 12 cells (a 21 MB matrix read by all SMs)
// costs less than another level of latency-bound sweeps plus a smaller
// dense solve.
constexpr int kDenseCoarseMax = 4096;
constexpr int kDenseCoarseTarget = 2304;
// Symmetric (pseudo-)inverse of the coarsest-grid operator
// A e = (sum of neighbours - diag e) / h2 (pure Neumann: the minimum-norm
// inverse on zero-mean data; Dirichlet top: the inverse), n x n FP32 in
// natural cell order.  Host code, double precision Gauss-Jordan.
std::vector<float> coarse_inverse(const Grid& c, float h2, int ref);

// ---- launchers (k_mg.cu) ---------------------------------------------------------------
// Raise the dynamic shared-memory limit of the coarse-grid kernel (once per process).
cudaError_t mg_prepare();
void launch_pressure_solve(const DevState& s, cudaStream_t st);
void launch_residual_norm(const DevState& s, double* out, cudaStream_t st);
// mean removal: launch_sum leaves per-block partials in part (kSumBlocks
// doubles), launch_sub_mean adds them in a fixed order and subtracts the mean
void launch_sum(const float* a, size_t n, double* part, int num_sms, cudaStream_t st);
// sumsq (statistics): also accumulate the sum of squares of the result there
void launch_sub_mean(float* a, size_t n, const double* part, int num_sms, cudaStream_t st, double* sumsq = nullptr);
void launch_sumsq(const float* a, size_t n, double* out, int num_sms, cudaStream_t st);
// Natural <-> red-black split copy of a level-0 array (field I/O).
void launch_split(const float* src, float* dst, const Grid& d, bool to_split, cudaStream_t st);
// One pass of the level-0 pressure smoother on the current state; returns the
// pass's algorithmic HBM bytes (read p and b, write p once).
double smoother_pass(const DevState& s, cudaStream_t st);

// ---- launchers (k_exact.cu: FMA-free, bit-reproducible on the host) -------------------
void launch_parcel_emit(const DevState& s, cudaStream_t st);
void launch_parcel_advect(const DevState& s, cudaStream_t st);
void launch_count_alive(const DevState& s, unsigned int* out, cudaStream_t st);
void launch_inject_sphere(const DevState& s, const float c[3], float r, float dye, const float vel[3], float sigma,
                          uint64_t seed, cudaStream_t st);
cudaError_t eval_math_device(int fn, const float* x, const float* y, float* out, uint32_t n);
// sum of a . vel over the MAC faces k_inject_sphere sets (FP64, into *out)
void launch_sphere_impulse(const DevState& s, const float* a_u, const float* a_v, const float* a_w, const float c[3],
                           float r, const float vel[3], double* out, cudaStream_t st);
// soft-edged drop (additive) and the gradient of the loss in its impulse
// scale and centre from the adjoint fields right after it (out[4], FP64)
void launch_inject_sphere_soft(const DevState& s, const float c[3], float r, float h, float dye, const float vel[3],
                               float sigma, uint64_t seed, cudaStream_t st);
void launch_sphere_soft_grad(const DevState& s, const float* a_u, const float* a_v, const float* a_w,
                             const float* a_c, const float c[3], float r, float h, float dye, const float vel[3],
                             float sigma, uint64_t seed, double* out, cudaStream_t st);

// ---- launchers (k_adjoint.cu): transpose of each closed-box FP32 stage ------------------
void launch_adj_advect_mac(const DevState& s, const AdjState& a, cudaStream_t st);
void launch_adj_mac_to_center(const DevState& s, const AdjState& a, cudaStream_t st);
void launch_adj_casson(const DevState& s, const AdjState& a, cudaStream_t st);
void launch_adj_mac_rhs(const DevState& s, const AdjState& a, cudaStream_t st);
void launch_adj_pressure_solve(const DevState& s, const AdjState& a, cudaStream_t st);
void launch_adj_project(const DevState& s, const AdjState& a, cudaStream_t st);
void launch_adj_conc_predict(const DevState& s, const AdjState& a, cudaStream_t st);
void launch_adj_conc_resolve(const DevState& s, const AdjState& a, cudaStream_t st);
// Raise the dynamic shared-memory limit of the transposed coarse solve.
cudaError_t adj_prepare();

}  // namespace dob
