// k_mg.cu — geometric-multigrid pressure solve (fluid.ts:557-855,
// schedule BloodDropEngine.ts:1942-2059), generalised to any number of
// grids, any pre/post sweep counts and several V-cycles per step, plus the
// FP64 pieces: compatibility / mean sums and the mixed-precision defect loop.
//
// Kernels:
//   k_rbgs             one colour of red-black Gauss-Seidel, in place
//                      (one thread per cell of that colour)
//   k_residual_restrict residual b - A e of 8 fine cells averaged into one
//                      coarse right-hand side (MG_RESIDUAL + MG_RESTRICT fused:
//                      the fine residual is never stored)
//   k_prolong_add      e_f += trilinear(e_c), cell-centred
//   k_coarse_smem      all sweeps of the coarsest grid in one CTA's shared memory
//   k_defect           FP64 residual of the FP32 pressure -> BF16, with its norm
#include <cuda_runtime.h>

#include "dob_kernels.cuh"

namespace dob {

// Round a value to the precision of the storage type T (the coarse solve keeps
// its grid in FP32 shared memory but must reproduce T-typed storage).
template <class T> __device__ __forceinline__ float as_stored(float v);
template <> __device__ __forceinline__ float as_stored<float>(float v) { return v; }
template <> __device__ __forceinline__ float as_stored<__nv_bfloat16>(float v) {
  return __bfloat162float(__float2bfloat16_rn(v));
}

__device__ __forceinline__ bool skip_now(const unsigned int* skip) { return skip != nullptr && *skip != 0u; }

// evalMgStencil (fluid.ts:568-602): neighbour sum and diagonal count, in the
// order x-, x+, y-, y+, z-, z+.  Reference BCs count the top face always
// (Dirichlet 0 ghost); the closed box counts only existing neighbours.
template <class T>
__device__ __forceinline__ void stencil(const T* a, const Grid& d, int x, int y, int z, size_t i, int ref, float& sumN,
                                        float& diag) {
  sumN = 0.0f;
  diag = ref ? 1.0f : 0.0f;
  const size_t sy = d.nx, sz = (size_t)d.nx * d.ny;
  if (x > 0) { sumN = sumN + ldv(a + i - 1); diag = diag + 1.0f; }
  if (x < d.nx - 1) { sumN = sumN + ldv(a + i + 1); diag = diag + 1.0f; }
  if (y > 0) { sumN = sumN + ldv(a + i - sy); diag = diag + 1.0f; }
  if (y < d.ny - 1) { sumN = sumN + ldv(a + i + sy); if (!ref) diag = diag + 1.0f; }
  if (z > 0) { sumN = sumN + ldv(a + i - sz); diag = diag + 1.0f; }
  if (z < d.nz - 1) { sumN = sumN + ldv(a + i + sz); diag = diag + 1.0f; }
}

// One colour of RBGS (createMgRbgsShader, fluid.ts:605-681), in place: a
// cell of one colour reads only cells of the other colour.
template <class T>
__global__ void __launch_bounds__(256) k_rbgs(Grid d, int color, float h2, int ref, T* __restrict__ a,
                                              const T* __restrict__ b, const unsigned int* __restrict__ skip) {
  if (skip_now(skip)) return;
  const int tx = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  const int x = 2 * tx + ((y + z + color) & 1);
  if (x >= d.nx || y >= d.ny) return;
  const size_t i = d.at(x, y, z);
  float sumN, diag;
  stencil(a, d, x, y, z, i, ref, sumN, diag);
  stf(a + i, (sumN - h2 * ldv(b + i)) / diag);
}

// MG_RESIDUAL + MG_RESTRICT (fluid.ts:744-800) fused: each thread owns one
// coarse cell and averages the residual of its 8 fine cells (dz, dy, dx order).
template <class T, class TC>
__global__ void __launch_bounds__(256) k_residual_restrict(Grid f, Grid c, float h2, int ref, const T* __restrict__ a,
                                                           const T* __restrict__ b, TC* __restrict__ bc,
                                                           const unsigned int* __restrict__ skip) {
  if (skip_now(skip)) return;
  const int X = blockIdx.x * blockDim.x + threadIdx.x;
  const int Y = blockIdx.y * blockDim.y + threadIdx.y;
  const int Z = blockIdx.z;
  if (X >= c.nx || Y >= c.ny) return;
  float sum = 0.0f;
#pragma unroll
  for (int dz = 0; dz < 2; ++dz)
#pragma unroll
    for (int dy = 0; dy < 2; ++dy)
#pragma unroll
      for (int dx = 0; dx < 2; ++dx) {
        const int x = 2 * X + dx, y = 2 * Y + dy, z = 2 * Z + dz;
        const size_t i = f.at(x, y, z);
        float sumN, diag;
        stencil(a, f, x, y, z, i, ref, sumN, diag);
        const float lapScaled = (sumN - diag * ldv(a + i)) / h2;
        sum = sum + (ldv(b + i) - lapScaled);
      }
  stf(bc + c.at(X, Y, Z), sum * 0.125f);
}

// MG_PROLONG_ADD (fluid.ts:806-855): cell-centred trilinear interpolation of
// the coarse correction; above the top the reference's Dirichlet ghost is 0,
// the closed box clamps (Neumann).
template <class TC>
__device__ __forceinline__ float coarse_err(const TC* e, const Grid& c, int ref, int x, int y, int z) {
  if (ref && y >= c.ny) return 0.0f;
  return ldv(e + c.at(dob_clampi(x, 0, c.nx - 1), dob_clampi(y, 0, c.ny - 1), dob_clampi(z, 0, c.nz - 1)));
}
template <class T, class TC>
__global__ void __launch_bounds__(256) k_prolong_add(Grid f, Grid c, int ref, T* __restrict__ a,
                                                     const TC* __restrict__ e, const unsigned int* __restrict__ skip) {
  if (skip_now(skip)) return;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= f.nx || y >= f.ny) return;
  const float cx = (((float)x + 0.5f) / (float)f.nx) * (float)c.nx - 0.5f;
  const float cy = (((float)y + 0.5f) / (float)f.ny) * (float)c.ny - 0.5f;
  const float cz = (((float)z + 0.5f) / (float)f.nz) * (float)c.nz - 0.5f;
  const float bx = floorf(cx), by = floorf(cy), bz = floorf(cz);
  const int ix = (int)bx, iy = (int)by, iz = (int)bz;
  const float fx = cx - bx, fy = cy - by, fz = cz - bz;
  const float c000 = coarse_err(e, c, ref, ix, iy, iz), c100 = coarse_err(e, c, ref, ix + 1, iy, iz);
  const float c010 = coarse_err(e, c, ref, ix, iy + 1, iz), c110 = coarse_err(e, c, ref, ix + 1, iy + 1, iz);
  const float c001 = coarse_err(e, c, ref, ix, iy, iz + 1), c101 = coarse_err(e, c, ref, ix + 1, iy, iz + 1);
  const float c011 = coarse_err(e, c, ref, ix, iy + 1, iz + 1), c111 = coarse_err(e, c, ref, ix + 1, iy + 1, iz + 1);
  const float x00 = dob_mix(c000, c100, fx), x10 = dob_mix(c010, c110, fx);
  const float x01 = dob_mix(c001, c101, fx), x11 = dob_mix(c011, c111, fx);
  const float corr = dob_mix(dob_mix(x00, x10, fy), dob_mix(x01, x11, fy), fz);
  const size_t i = f.at(x, y, z);
  stf(a + i, ldv(a + i) + corr);
}

template <class T>
__global__ void k_fill_zero(T* __restrict__ a, size_t n, const unsigned int* __restrict__ skip) {
  if (skip_now(skip)) return;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    a[i] = T(0.0f);
}

// MG_COARSE_SOLVE_L3 (fluid.ts:687-739) for any coarsest grid that fits in
// shared memory: zero start, `sweeps` red-black sweeps, one CTA.
template <class T>
__global__ void __launch_bounds__(1024) k_coarse_smem(Grid d, float h2, int ref, int sweeps, T* __restrict__ e,
                                                      const T* __restrict__ b, const unsigned int* __restrict__ skip) {
  if (skip_now(skip)) return;
  extern __shared__ float smem[];
  const int n = (int)d.n();
  float* se = smem;
  float* sb = smem + n;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    se[k] = 0.0f;
    sb[k] = ldv(b + k);
  }
  __syncthreads();
  const int sy = d.nx, sz = d.nx * d.ny;
  for (int s = 0; s < sweeps; ++s) {
    for (int color = 0; color < 2; ++color) {
      for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const int x = k % d.nx;
        const int y = (k / d.nx) % d.ny;
        const int z = k / sz;
        if (((x + y + z) & 1) != color) continue;
        float sumN = 0.0f, diag = ref ? 1.0f : 0.0f;
        if (x > 0) { sumN = sumN + se[k - 1]; diag = diag + 1.0f; }
        if (x < d.nx - 1) { sumN = sumN + se[k + 1]; diag = diag + 1.0f; }
        if (y > 0) { sumN = sumN + se[k - sy]; diag = diag + 1.0f; }
        if (y < d.ny - 1) { sumN = sumN + se[k + sy]; if (!ref) diag = diag + 1.0f; }
        if (z > 0) { sumN = sumN + se[k - sz]; diag = diag + 1.0f; }
        if (z < d.nz - 1) { sumN = sumN + se[k + sz]; diag = diag + 1.0f; }
        se[k] = as_stored<T>((sumN - h2 * sb[k]) / diag);
      }
      __syncthreads();
    }
  }
  for (int k = threadIdx.x; k < n; k += blockDim.x) stf(e + k, se[k]);
}

// ---- FP64 pieces ---------------------------------------------------------------------
__global__ void k_sum64(const float* __restrict__ a, size_t n, double* __restrict__ out) {
  double s = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    s += (double)a[i];
  block_sum_atomic(s, out);
}
__global__ void k_sumsq64(const float* __restrict__ a, size_t n, double* __restrict__ out) {
  double s = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double v = (double)a[i];
    s += v * v;
  }
  block_sum_atomic(s, out);
}
__global__ void k_sub_mean(float* __restrict__ a, size_t n, const double* __restrict__ sum) {
  const double mean = *sum / (double)n;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    a[i] = (float)((double)a[i] - mean);
}

// r = b - A p in FP64 (FP32 inputs); optionally stored as BF16; ||r||^2 summed.
__global__ void __launch_bounds__(256) k_defect(Grid d, float h2f, int ref, const float* __restrict__ p,
                                                const float* __restrict__ b, __nv_bfloat16* __restrict__ r_out,
                                                double* __restrict__ norm2, const unsigned int* __restrict__ skip) {
  if (skip_now(skip)) return;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  double rr = 0.0;
  if (x < d.nx && y < d.ny) {
    const size_t i = d.at(x, y, z);
    const size_t sy = d.nx, sz = (size_t)d.nx * d.ny;
    double sumN = 0.0, diag = ref ? 1.0 : 0.0;
    if (x > 0) { sumN += (double)p[i - 1]; diag += 1.0; }
    if (x < d.nx - 1) { sumN += (double)p[i + 1]; diag += 1.0; }
    if (y > 0) { sumN += (double)p[i - sy]; diag += 1.0; }
    if (y < d.ny - 1) { sumN += (double)p[i + sy]; if (!ref) diag += 1.0; }
    if (z > 0) { sumN += (double)p[i - sz]; diag += 1.0; }
    if (z < d.nz - 1) { sumN += (double)p[i + sz]; diag += 1.0; }
    const double r = (double)b[i] - (sumN - diag * (double)p[i]) / (double)h2f;
    if (r_out) r_out[i] = __float2bfloat16_rn((float)r);
    rr = r * r;
  }
  if (norm2) block_sum_atomic(rr, norm2);
}

// Converged when ||r|| <= tol ||b||: sets the skip flag every later kernel of
// the defect loop reads, and counts executed iterations.
__global__ void k_defect_check(const double* __restrict__ rnorm2, const double* __restrict__ bnorm2, double tol,
                               unsigned int* __restrict__ done, unsigned int* __restrict__ iters) {
  if (*done) return;
  const double rn = sqrt(*rnorm2), bn = sqrt(*bnorm2);
  if (bn == 0.0 || rn <= tol * bn) *done = 1u;
  else *iters += 1u;
}

// p += e (FP32 pressure, BF16 correction)
__global__ void k_add_correction(float* __restrict__ p, const __nv_bfloat16* __restrict__ e, size_t n,
                                 const unsigned int* __restrict__ skip) {
  if (skip_now(skip)) return;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    p[i] = p[i] + __bfloat162float(e[i]);
}

// ---- host side ----------------------------------------------------------------------
static inline dim3 g_cells(const Grid& d) { return dim3((d.nx + 31) / 32, (d.ny + 7) / 8, d.nz); }
static inline dim3 g_half(const Grid& d) { return dim3((d.nx / 2 + 31) / 32, (d.ny + 7) / 8, d.nz); }
static inline dim3 b_cells() { return dim3(32, 8, 1); }

cudaError_t mg_prepare() {
  const int bytes = 200 * 1024;
  cudaError_t e = cudaFuncSetAttribute(k_coarse_smem<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_coarse_smem<__nv_bfloat16>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  return e;
}

void launch_sum(const float* a, size_t n, double* out, int num_sms, cudaStream_t st) {
  cudaMemsetAsync(out, 0, sizeof(double), st);
  k_sum64<<<num_sms * 4, 256, 0, st>>>(a, n, out);
}
void launch_sub_mean(float* a, size_t n, const double* sum, int num_sms, cudaStream_t st) {
  k_sub_mean<<<num_sms * 4, 256, 0, st>>>(a, n, sum);
}
void launch_sumsq(const float* a, size_t n, double* out, int num_sms, cudaStream_t st) {
  k_sumsq64<<<num_sms * 4, 256, 0, st>>>(a, n, out);
}

template <class T>
static void smooth(const DevState& s, int l, T* a, const T* b, int sweeps, const unsigned int* skip, cudaStream_t st) {
  const MgLevel& L = s.lv[l];
  for (int k = 0; k < sweeps; ++k) {
    k_rbgs<T><<<g_half(L.d), b_cells(), 0, st>>>(L.d, 0, L.h2, s.ref, a, b, skip);
    k_rbgs<T><<<g_half(L.d), b_cells(), 0, st>>>(L.d, 1, L.h2, s.ref, a, b, skip);
  }
}

template <class T>
static void coarse_solve(const DevState& s, int l, T* e, const T* b, const unsigned int* skip, cudaStream_t st) {
  const MgLevel& L = s.lv[l];
  const size_t bytes = 2 * L.d.n() * sizeof(float);
  if (bytes <= 200 * 1024) {
    k_coarse_smem<T><<<1, 1024, bytes, st>>>(L.d, L.h2, s.ref, s.coarse_sweeps, e, b, skip);
  } else {
    k_fill_zero<T><<<s.num_sms, 256, 0, st>>>(e, L.d.n(), skip);
    smooth<T>(s, l, e, b, s.coarse_sweeps, skip, st);
  }
}

// One V-cycle on (x0, b0); per-level arrays E[l], B[l] for l >= 1.
template <class T>
static void vcycle(const DevState& s, T* x0, const T* b0, T* const* E, T* const* B, const unsigned int* skip,
                   cudaStream_t st) {
  const int L = s.nlev;
  if (L == 1) {
    smooth<T>(s, 0, x0, b0, s.pre + s.post, skip, st);
    return;
  }
  smooth<T>(s, 0, x0, b0, s.pre0, skip, st);
  k_residual_restrict<T, T><<<g_cells(s.lv[1].d), b_cells(), 0, st>>>(s.lv[0].d, s.lv[1].d, s.lv[0].h2, s.ref, x0, b0,
                                                                      B[1], skip);
  for (int l = 1; l < L - 1; ++l) {
    k_fill_zero<T><<<s.num_sms, 256, 0, st>>>(E[l], s.lv[l].d.n(), skip);
    smooth<T>(s, l, E[l], B[l], s.pre, skip, st);
    k_residual_restrict<T, T><<<g_cells(s.lv[l + 1].d), b_cells(), 0, st>>>(s.lv[l].d, s.lv[l + 1].d, s.lv[l].h2,
                                                                            s.ref, E[l], B[l], B[l + 1], skip);
  }
  coarse_solve<T>(s, L - 1, E[L - 1], B[L - 1], skip, st);
  for (int l = L - 2; l >= 1; --l) {
    k_prolong_add<T, T><<<g_cells(s.lv[l].d), b_cells(), 0, st>>>(s.lv[l].d, s.lv[l + 1].d, s.ref, E[l], E[l + 1], skip);
    smooth<T>(s, l, E[l], B[l], s.post, skip, st);
  }
  k_prolong_add<T, T><<<g_cells(s.lv[0].d), b_cells(), 0, st>>>(s.lv[0].d, s.lv[1].d, s.ref, x0, E[1], skip);
  smooth<T>(s, 0, x0, b0, s.post0, skip, st);
}

double smoother_pass(const DevState& s, cudaStream_t st) {
  smooth<float>(s, 0, s.p, s.rhs, 1, nullptr, st);
  return 12.0 * (double)s.g.n();
}

void launch_residual_norm(const DevState& s, double* out, cudaStream_t st) {
  cudaMemsetAsync(out, 0, sizeof(double), st);
  k_defect<<<g_cells(s.g), b_cells(), 0, st>>>(s.g, s.lv[0].h2, s.ref, s.p, s.rhs, nullptr, out, nullptr);
}

void launch_pressure_solve(const DevState& s, cudaStream_t st) {
  if (s.prec == DOB_PREC_MIXED) {
    __nv_bfloat16* E[kMaxLevels];
    __nv_bfloat16* B[kMaxLevels];
    for (int l = 0; l < s.nlev; ++l) { E[l] = s.lv[l].eh; B[l] = s.lv[l].bh; }
    unsigned int* done = s.redu + REDU_DONE;
    cudaMemsetAsync(s.redu + REDU_DONE, 0, 2 * sizeof(unsigned int), st);  // done, iters
    cudaMemsetAsync(s.red + RED_RHS_NORM2, 0, sizeof(double) * (RED_COUNT - RED_RHS_NORM2), st);
    k_sumsq64<<<s.num_sms * 4, 256, 0, st>>>(s.rhs, s.g.n(), s.red + RED_RHS_NORM2);
    const size_t n = s.g.n();
    for (int it = 0; it < s.max_outer; ++it) {
      double* rn2 = s.red + RED_DEFECT_NORM2 + (it < 31 ? it : 31);
      k_defect<<<g_cells(s.g), b_cells(), 0, st>>>(s.g, s.lv[0].h2, s.ref, s.p, s.rhs, s.r0h, rn2, done);
      k_defect_check<<<1, 1, 0, st>>>(rn2, s.red + RED_RHS_NORM2, s.rel_tol, done, s.redu + REDU_ITERS);
      k_fill_zero<__nv_bfloat16><<<s.num_sms * 4, 256, 0, st>>>(s.e0h, n, done);
      for (int c = 0; c < s.cycles; ++c) vcycle<__nv_bfloat16>(s, s.e0h, s.r0h, E, B, done, st);
      k_add_correction<<<s.num_sms * 4, 256, 0, st>>>(s.p, s.e0h, n, done);
    }
  } else {
    float* E[kMaxLevels];
    float* B[kMaxLevels];
    for (int l = 0; l < s.nlev; ++l) { E[l] = s.lv[l].e; B[l] = s.lv[l].b; }
    for (int c = 0; c < s.cycles; ++c) vcycle<float>(s, s.p, s.rhs, E, B, nullptr, st);
  }
  if (!s.ref) {
    launch_sum(s.p, s.g.n(), s.red + RED_P_SUM, s.num_sms, st);
    launch_sub_mean(s.p, s.g.n(), s.red + RED_P_SUM, s.num_sms, st);
  }
}

}  // namespace dob
