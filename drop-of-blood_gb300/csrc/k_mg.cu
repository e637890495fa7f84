// k_mg.cu — geometric-multigrid pressure solve (fluid.ts:557-855,
// schedule BloodDropEngine.ts:1942-2059), generalised to any number of
// grids, any pre/post sweep counts and several V-cycles per step, plus the
// FP64 pieces: compatibility / mean sums and the mixed-precision defect loop.
//
// Memory layout: every multigrid array (pressure, right-hand side, the
// corrections and right-hand sides of the coarse levels) is stored
// red-black split: the cells of colour c = (x+y+z)&1 occupy half c of the
// array, row-major with x/2 fastest (rb_index).  A half-sweep of one colour
// then reads only the other half plus its own right-hand side and writes its
// own half, with consecutive threads on consecutive words: 3 x N/2 words of
// traffic instead of touching every line of both colours.
//
// Kernels:
//   k_rbgs_v4           one colour of red-black Gauss-Seidel, four cells of a
//                       row and 1-4 planes per thread, 16-byte loads (rows
//                       with nx % 8 == 0)
//   k_rbgs_split        the same, one thread per cell (other rows)
//   k_residual_restrict2 residual b - A e of the 8 fine cells of each of two
//                       coarse cells, averaged into their right-hand sides
//                       (MG_RESIDUAL + MG_RESTRICT fused: the fine residual is
//                       never stored)
//   k_prolong_add2      e_f += trilinear(e_c), cell-centred, two coarse cells
//                       per thread
//   k_coarse_dense      exact coarsest solve e = M b with a precomputed dense
//                       (pseudo-)inverse
//   k_coarse_cluster    every sweep of the coarsest grid inside one
//                       thread-block cluster: each CTA keeps a slab of planes in
//                       shared memory, reads the neighbour slabs' boundary
//                       planes through distributed shared memory, and the
//                       half-sweeps are separated by hardware cluster barriers
//   k_defect_df4        residual of the pressure (double-float in the mixed
//   (k_defect_df)       mode) formed with error-free FP32 transformations, its
//                       max and norm (statistics and the mixed defect loop)
// The V-cycle kernels are launched with programmatic dependent launch
// (launch_pdl): each may be scheduled while its predecessor drains.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <cmath>
#include <utility>
#include <vector>

#include "dob_kernels.cuh"

namespace cg = cooperative_groups;

namespace dob {

template <class T> __device__ __forceinline__ float as_stored(float v);
template <> __device__ __forceinline__ float as_stored<float>(float v) { return v; }
template <> __device__ __forceinline__ float as_stored<__nv_bfloat16>(float v) {
  return __bfloat162float(__float2bfloat16_rn(v));
}

__device__ __forceinline__ bool skip_now(const unsigned int* skip) { return skip != nullptr && *skip != 0u; }

// evalMgStencil (fluid.ts:568-602) on a red-black split array: neighbour sum
// and diagonal count in the order x-, x+, y-, y+, z-, z+.  Reference BCs
// count the top face always (Dirichlet 0 ghost); the closed box counts only
// existing neighbours.  `oth` is the other colour's half, `r` the row base
// and k = x/2 of the cell.
template <class T>
__device__ __forceinline__ void stencil_rb(const T* oth, const Grid& d, int x, int y, int z, size_t r, int k, int ref,
                                           float& sumN, float& diag) {
  const int hx = d.nx >> 1;
  sumN = 0.0f;
  diag = ref ? 1.0f : 0.0f;
  if (x > 0) { sumN = sumN + ldv(oth + r + ((x - 1) >> 1)); diag = diag + 1.0f; }
  if (x < d.nx - 1) { sumN = sumN + ldv(oth + r + ((x + 1) >> 1)); diag = diag + 1.0f; }
  if (y > 0) { sumN = sumN + ldv(oth + r - hx + k); diag = diag + 1.0f; }
  if (y < d.ny - 1) { sumN = sumN + ldv(oth + r + hx + k); if (!ref) diag = diag + 1.0f; }
  if (z > 0) { sumN = sumN + ldv(oth + r - (size_t)d.ny * hx + k); diag = diag + 1.0f; }
  if (z < d.nz - 1) { sumN = sumN + ldv(oth + r + (size_t)d.ny * hx + k); diag = diag + 1.0f; }
}

// Value of the split array at natural coordinates.
template <class T>
__device__ __forceinline__ float rb_at(const T* a, const Grid& d, int x, int y, int z) {
  return ldv(a + rb_index(d, x, y, z));
}

// One colour of RBGS (createMgRbgsShader, fluid.ts:605-681), in place.
// zoth: the other colour is zero (the first half-sweep from a zero guess), so
// its values are not read; the result has the same bits as with zeroed
// memory.
template <class T>
__global__ void __launch_bounds__(256) k_rbgs_split(Grid d, int color, float h2, int ref, int zoth,
                                                    T* __restrict__ a, const T* __restrict__ b,
                                                    const unsigned int* __restrict__ skip) {
  pdl_wait();
  pdl_trigger();
  if (skip_now(skip)) return;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  const int hx = d.nx >> 1;
  if (k >= hx || y >= d.ny) return;
  const int x = 2 * k + ((y + z + color) & 1);
  const size_t half = d.n() >> 1;
  T* own = a + (size_t)color * half;
  const T* oth = a + (size_t)(1 - color) * half;
  const size_t r = ((size_t)z * d.ny + y) * hx;
  const size_t i = r + k;
  const float bv = ldv(b + (size_t)color * half + i);
  float val;
  if (zoth) {
    const bool in = x > 0 && x < d.nx - 1 && y > 0 && y < d.ny - 1 && z > 0 && z < d.nz - 1;
    const float diag = (ref ? 1.0f : 0.0f) + (x > 0 ? 1.0f : 0.0f) + (x < d.nx - 1 ? 1.0f : 0.0f) +
                       (y > 0 ? 1.0f : 0.0f) + ((y < d.ny - 1 && !ref) ? 1.0f : 0.0f) + (z > 0 ? 1.0f : 0.0f) +
                       (z < d.nz - 1 ? 1.0f : 0.0f);
    val = in ? (0.0f - h2 * bv) * (1.0f / 6.0f) : (0.0f - h2 * bv) / diag;
  } else if (x > 0 && x < d.nx - 1 && y > 0 && y < d.ny - 1 && z > 0 && z < d.nz - 1) {
    // interior: six neighbours, diagonal 6 in both boundary modes
    const size_t sz = (size_t)d.ny * hx;
    const float sumN = ((((ldv(oth + r + ((x - 1) >> 1)) + ldv(oth + r + ((x + 1) >> 1))) + ldv(oth + i - hx)) +
                         ldv(oth + i + hx)) + ldv(oth + i - sz)) + ldv(oth + i + sz);
    val = (sumN - h2 * bv) * (1.0f / 6.0f);
  } else {
    float sumN, diag;
    stencil_rb(oth, d, x, y, z, r, k, ref, sumN, diag);
    val = (sumN - h2 * bv) / diag;
  }
  stf(own + i, val);
}

// Four consecutive cells of one colour in one row: (x, y, z) with
// x = 2k + p, k = k0..k0+3 and the same parity p = (y + z + colour) & 1 for
// all four, so their +-x neighbours in the other colour are words k0-1+p ..
// k0+3+p of the same row (one 16-byte vector plus one scalar) and their
// +-y / +-z neighbours and right-hand sides are 16-byte vectors too.
template <class T> struct Vec4Ld;
template <> struct Vec4Ld<float> {
  __device__ __forceinline__ static float4 ld(const float* p) { return *reinterpret_cast<const float4*>(p); }
  __device__ __forceinline__ static void st(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
};
template <> struct Vec4Ld<__nv_bfloat16> {
  __device__ __forceinline__ static float4 ld(const __nv_bfloat16* p) {
    const uint2 r = *reinterpret_cast<const uint2*>(p);
    const __nv_bfloat162 a = *reinterpret_cast<const __nv_bfloat162*>(&r.x);
    const __nv_bfloat162 b = *reinterpret_cast<const __nv_bfloat162*>(&r.y);
    const float2 fa = __bfloat1622float2(a), fb = __bfloat1622float2(b);
    return make_float4(fa.x, fa.y, fb.x, fb.y);
  }
  __device__ __forceinline__ static void st(__nv_bfloat16* p, float4 v) {
    const __nv_bfloat162 a = __floats2bfloat162_rn(v.x, v.y);
    const __nv_bfloat162 b = __floats2bfloat162_rn(v.z, v.w);
    uint2 r;
    r.x = *reinterpret_cast<const uint32_t*>(&a);
    r.y = *reinterpret_cast<const uint32_t*>(&b);
    *reinterpret_cast<uint2*>(p) = r;
  }
};
__device__ __forceinline__ float f4get(const float4& v, int j) {
  return j == 0 ? v.x : (j == 1 ? v.y : (j == 2 ? v.z : v.w));
}

// One colour of RBGS, four cells per thread and ZC planes per thread (rows
// with nx % 8 == 0, nz % ZC == 0).
// Block (bx, by): threadIdx.x runs over the Q = nx/8 quads of a row and
// threadIdx.y over rows, so a warp holds whole rows back to back with no idle
// lanes; blockIdx.z picks ZC consecutive planes.  The other colour's words
// k0..k0+3 of row (y, z') are the x-neighbour source of plane z' and the
// z-neighbours of planes z' - 1 and z' + 1, so marching over ZC planes loads
// each of them once: per plane one centre vector, two y-neighbour vectors,
// one scalar and the right-hand side instead of six vectors and a scalar, and
// every thread has ZC planes of loads in flight.  Boundaries are handled
// without divergence: a missing neighbour is loaded from a clamped in-range
// address and enters the sum with weight 0 (adding an exact 0 leaves the sum
// unchanged, so the sum equals the neighbour-skipping evalMgStencil order);
// only lanes whose diagonal is not 6 take the short IEEE-division branch.
// Offsets are 32-bit (split halves have fewer than 2^30 words).  `own` and
// `oth` are the two halves of the level's array (disjoint).  ZOTH: the other
// colour is zero (first half-sweep from a zero guess) and is not read.
template <class T, int ZC, bool ZOTH>
__global__ void __launch_bounds__(256) k_rbgs_v4(Grid d, int color, float h2, int ref, T* __restrict__ own,
                                                 const T* __restrict__ oth, const T* __restrict__ bown,
                                                 const unsigned int* __restrict__ skip) {
  pdl_wait();
  pdl_trigger();
  if (skip_now(skip)) return;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z0 = blockIdx.z * ZC;
  const uint32_t hx = (uint32_t)d.nx >> 1;
  const uint32_t k0 = 4u * (uint32_t)q;
  if (k0 >= hx || y >= d.ny) return;
  const uint32_t sz = (uint32_t)d.ny * hx;
  const uint32_t r0 = (uint32_t)z0 * sz + (uint32_t)y * hx + k0;
  const bool has_ym = y > 0, has_yp = y < d.ny - 1;
  const bool has_zlo = z0 > 0, has_zhi = z0 + ZC < d.nz;
  const uint32_t oym = has_ym ? hx : 0u, oyp = has_yp ? hx : 0u;
  // the word outside the vector: k0-1 (parity 0) or k0+4 (parity 1), absent at the row ends
  const bool has_e0 = k0 > 0, has_e1 = k0 + 4 < hx;
  const uint32_t ke0 = has_e0 ? k0 - 1 : k0, ke1 = has_e1 ? k0 + 4 : k0 + 3;
  const float wym = has_ym ? 1.0f : 0.0f, wyp = has_yp ? 1.0f : 0.0f;
  const float dy = wym + (ref ? 1.0f : wyp);  // +y face always counted with the Dirichlet top
  const int p0 = (y + z0 + color) & 1;
  const float4 zero4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  float4 C[ZC + 2];  // C[i + 1] = other colour, plane z0 + i, words k0..k0+3
  C[0] = ZOTH ? zero4 : Vec4Ld<T>::ld(oth + (has_zlo ? r0 - sz : r0));
#pragma unroll
  for (int i = 0; i < ZC; ++i) C[i + 1] = ZOTH ? zero4 : Vec4Ld<T>::ld(oth + r0 + i * sz);
  C[ZC + 1] = ZOTH ? zero4 : Vec4Ld<T>::ld(oth + (has_zhi ? r0 + ZC * sz : r0 + (ZC - 1) * sz));
#pragma unroll
  for (int i = 0; i < ZC; ++i) {
    const uint32_t r = r0 + i * sz;
    const int p = p0 ^ (i & 1);
    const float4 bv = Vec4Ld<T>::ld(bown + r);
    const float4 ym = ZOTH ? zero4 : Vec4Ld<T>::ld(oth + r - oym);
    const float4 yp = ZOTH ? zero4 : Vec4Ld<T>::ld(oth + r + oyp);
    const float ex = ZOTH ? 0.0f : ldv(oth + r - k0 + (p == 0 ? ke0 : ke1));
    const float wex = (p == 0 ? has_e0 : has_e1) ? 1.0f : 0.0f;
    const float wzm = (i > 0 || has_zlo) ? 1.0f : 0.0f;
    const float wzp = (i < ZC - 1 || has_zhi) ? 1.0f : 0.0f;
    const float dyz = dy + (wzm + wzp);
    const float4 cm = C[i + 1], zm = C[i], zp = C[i + 2];
    float res[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float xm = p == 0 ? (j == 0 ? ex : f4get(cm, j - 1)) : f4get(cm, j);
      const float xp = p == 0 ? f4get(cm, j) : (j == 3 ? ex : f4get(cm, j + 1));
      const float wxm = (p == 0 && j == 0) ? wex : 1.0f;
      const float wxp = (p == 1 && j == 3) ? wex : 1.0f;
      float sumN = wxm * xm;
      sumN = fmaf(wxp, xp, sumN);
      sumN = fmaf(wym, f4get(ym, j), sumN);
      sumN = fmaf(wyp, f4get(yp, j), sumN);
      sumN = fmaf(wzm, f4get(zm, j), sumN);
      sumN = fmaf(wzp, f4get(zp, j), sumN);
      const float diag = dyz + (wxm + wxp);
      const float t = sumN - h2 * f4get(bv, j);
      res[j] = diag == 6.0f ? t * (1.0f / 6.0f) : t / diag;
    }
    Vec4Ld<T>::st(own + r, make_float4(res[0], res[1], res[2], res[3]));
  }
}

// ---- two coarse cells per thread (fine rows with nx % 4 == 0) ----------------------------
// Thread q owns coarse cells X = 2q, 2q+1 of coarse row (Y, Z), i.e. fine
// cells x = 4q..4q+3 of the fine rows y0+dy, z0+dz.  In the split layout the
// even cells x = 4q, 4q+2 of a fine row are words 2q, 2q+1 of one half and the
// odd cells x = 4q+1, 4q+3 the same words of the other half, so each fine row
// is two 8-byte loads; consecutive threads read consecutive words.
template <class T> struct Pair;
template <> struct Pair<float> {
  __device__ __forceinline__ static float2 ld(const float* p) { return *reinterpret_cast<const float2*>(p); }
  __device__ __forceinline__ static void st(float* p, float2 v) { *reinterpret_cast<float2*>(p) = v; }
};
template <> struct Pair<__nv_bfloat16> {
  __device__ __forceinline__ static float2 ld(const __nv_bfloat16* p) {
    return __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(p));
  }
  __device__ __forceinline__ static void st(__nv_bfloat16* p, float2 v) {
    *reinterpret_cast<__nv_bfloat162*>(p) = __floats2bfloat162_rn(v.x, v.y);
  }
};
// The four cells x = 4q..4q+3 of fine row (y, z) in natural order.
struct Row4 {
  float v[4];
};
template <class T>
__device__ __forceinline__ Row4 ld_row4(const T* a, uint32_t half, uint32_t r, uint32_t w, int par) {
  // par = (y + z) & 1: colour of the even cells
  const float2 e = Pair<T>::ld(a + (par ? half : 0u) + r + w);
  const float2 o = Pair<T>::ld(a + (par ? 0u : half) + r + w);
  Row4 R;
  R.v[0] = e.x; R.v[1] = o.x; R.v[2] = e.y; R.v[3] = o.y;
  return R;
}

// MG_RESIDUAL + MG_RESTRICT fused, two coarse cells per thread.  Per fine
// cell the neighbour sum follows evalMgStencil's order (x-, x+, y-, y+, z-,
// z+) with absent neighbours entering as exact zeros, so every residual and
// the (dz, dy, dx) averaging order match k_residual_restrict.  1/h2 is a power
// of two, so scaling by it equals the division.  Capped at 64 registers (4
// blocks per SM): 17.2 -> 16.0 us at 192x256x192.
// The body of k_residual_restrict2 for coarse cells X = 2q, 2q+1 of coarse
// row (Y, Z); rr / ra (optional) accumulate r^2 and max |r| of the fine cells.
template <class T, class TC>
// ered (optional): also the coarse level's first red half-sweep from a zero
// guess at the pair's red cell (k_rbgs_v4's ZOTH arithmetic: the neighbours
// are zeros, so the value is -h2c b / diag of the right-hand side as stored).
__device__ __forceinline__ void restrict_pair(Grid f, Grid c, float inv_h2, int ref, const T* __restrict__ a,
                                              const T* __restrict__ b, TC* __restrict__ bc, int q, int Y, int Z,
                                              float* rr, float* ra, TC* __restrict__ ered = nullptr,
                                              float h2c = 0.0f) {
  const uint32_t hx = (uint32_t)f.nx >> 1, half = (uint32_t)(f.n() >> 1), sz = (uint32_t)f.ny * hx;
  const uint32_t w = 2u * (uint32_t)q;
  const int y0 = 2 * Y, z0 = 2 * Z;
  auto rowb = [&](int y, int z) -> uint32_t { return (uint32_t)z * sz + (uint32_t)y * hx; };
  // block rows B[dz][dy], their x-neighbours, and the rows around the block
  Row4 B[2][2], Bb[2][2], Ym[2], Yp[2], Zm[2], Zp[2];
  float exm[2][2], exp_[2][2];
  const bool has_xm = q > 0, has_xp = 2 * q + 2 < c.nx;
#pragma unroll
  for (int dz = 0; dz < 2; ++dz)
#pragma unroll
    for (int dy = 0; dy < 2; ++dy) {
      const int y = y0 + dy, z = z0 + dz, par = (y + z) & 1;
      const uint32_t r = rowb(y, z);
      B[dz][dy] = ld_row4(a, half, r, w, par);
      Bb[dz][dy] = ld_row4(b, half, r, w, par);
      // x = 4q-1 is odd (half !par, word 2q-1); x = 4q+4 is even (half par, word 2q+2)
      exm[dz][dy] = ldv(a + (par ? 0u : half) + r + (has_xm ? w - 1 : w));
      exp_[dz][dy] = ldv(a + (par ? half : 0u) + r + (has_xp ? w + 2 : w + 1));
    }
  const bool has_ym = y0 > 0, has_yp = y0 + 2 < f.ny, has_zm = z0 > 0, has_zp = z0 + 2 < f.nz;
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int ym = has_ym ? y0 - 1 : y0, yp = has_yp ? y0 + 2 : y0 + 1;
    const int zm = has_zm ? z0 - 1 : z0, zp = has_zp ? z0 + 2 : z0 + 1;
    Ym[u] = ld_row4(a, half, rowb(ym, z0 + u), w, (ym + z0 + u) & 1);
    Yp[u] = ld_row4(a, half, rowb(yp, z0 + u), w, (yp + z0 + u) & 1);
    Zm[u] = ld_row4(a, half, rowb(y0 + u, zm), w, (y0 + u + zm) & 1);
    Zp[u] = ld_row4(a, half, rowb(y0 + u, zp), w, (y0 + u + zp) & 1);
  }
  const float wxm0 = has_xm ? 1.0f : 0.0f, wxp3 = has_xp ? 1.0f : 0.0f;
  float sum[2] = {0.0f, 0.0f};
#pragma unroll
  for (int dz = 0; dz < 2; ++dz)
#pragma unroll
    for (int dy = 0; dy < 2; ++dy) {
      const float wym = (dy == 1 || has_ym) ? 1.0f : 0.0f;
      const float wyp = (dy == 0 || has_yp) ? 1.0f : 0.0f;
      const float wzm = (dz == 1 || has_zm) ? 1.0f : 0.0f;
      const float wzp = (dz == 0 || has_zp) ? 1.0f : 0.0f;
      const float dyz = (wym + wzm + wzp) + (ref ? 1.0f : wyp);
      const Row4& P = B[dz][dy];
      const Row4& Pym = dy ? B[dz][0] : Ym[dz];
      const Row4& Pyp = dy ? Yp[dz] : B[dz][1];
      const Row4& Pzm = dz ? B[0][dy] : Zm[dy];
      const Row4& Pzp = dz ? Zp[dy] : B[1][dy];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const float xm = i > 0 ? P.v[i - 1] : exm[dz][dy];
        const float xp = i < 3 ? P.v[i + 1] : exp_[dz][dy];
        const float wxm = i == 0 ? wxm0 : 1.0f;
        const float wxp = i == 3 ? wxp3 : 1.0f;
        float sumN = wxm * xm;
        sumN = fmaf(wxp, xp, sumN);
        sumN = fmaf(wym, Pym.v[i], sumN);
        sumN = fmaf(wyp, Pyp.v[i], sumN);
        sumN = fmaf(wzm, Pzm.v[i], sumN);
        sumN = fmaf(wzp, Pzp.v[i], sumN);
        const float diag = dyz + (wxm + wxp);
        const float lap = (sumN - diag * P.v[i]) * inv_h2;
        const float res = Bb[dz][dy].v[i] - lap;
        sum[i >> 1] = sum[i >> 1] + res;
        if (rr) {
          *rr = fmaf(res, res, *rr);
          *ra = fmaxf(*ra, fabsf(res));
        }
      }
    }
  const uint32_t hc = (uint32_t)c.nx >> 1, halfc = (uint32_t)(c.n() >> 1);
  const uint32_t rc = ((uint32_t)Z * c.ny + Y) * hc + (uint32_t)q;
  const int pc = (Y + Z) & 1;  // colour of coarse X = 2q
  stf(bc + (pc ? halfc : 0u) + rc, sum[0] * 0.125f);
  stf(bc + (pc ? 0u : halfc) + rc, sum[1] * 0.125f);
  if (ered) {
    const int X = pc ? 2 * q + 1 : 2 * q;  // the red cell of the pair
    const float bv = as_stored<TC>((pc ? sum[1] : sum[0]) * 0.125f);
    const float wxm = X > 0 ? 1.0f : 0.0f, wxp = X < c.nx - 1 ? 1.0f : 0.0f;
    const float wym = Y > 0 ? 1.0f : 0.0f, wyp = Y < c.ny - 1 ? 1.0f : 0.0f;
    const float wzm = Z > 0 ? 1.0f : 0.0f, wzp = Z < c.nz - 1 ? 1.0f : 0.0f;
    const float dyz = (wym + (ref ? 1.0f : wyp)) + (wzm + wzp);
    const float diag = dyz + (wxm + wxp);
    const float t = 0.0f - h2c * bv;
    stf(ered + rc, diag == 6.0f ? t * (1.0f / 6.0f) : t / diag);
  }
}

// norm2 / maxbits (RED, the mixed solve's convergence test): also ||r||^2
// and max |r| over the fine cells, one FP64 add and one max per block.
template <class T, class TC, bool RED>
__global__ void __launch_bounds__(256, 4) k_residual_restrict2(Grid f, Grid c, float inv_h2, int ref,
                                                            const T* __restrict__ a, const T* __restrict__ b,
                                                            TC* __restrict__ bc, const unsigned int* __restrict__ skip,
                                                            double* __restrict__ norm2, unsigned int* __restrict__ maxbits,
                                                            TC* __restrict__ ered, float h2c) {
  pdl_wait();
  pdl_trigger();
  if (skip_now(skip)) return;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int Y = blockIdx.y * blockDim.y + threadIdx.y;
  const int Z = blockIdx.z;
  if (RED) {  // the reduction needs every thread of the block at its barrier
    float rr = 0.0f, ra = 0.0f;
    if (2 * q < c.nx && Y < c.ny) restrict_pair<T, TC>(f, c, inv_h2, ref, a, b, bc, q, Y, Z, &rr, &ra);
    block_sum_atomic_f(rr, norm2);
    block_max_atomic(ra, maxbits);
    return;
  }
  if (2 * q >= c.nx || Y >= c.ny) return;
  restrict_pair<T, TC>(f, c, inv_h2, ref, a, b, bc, q, Y, Z, nullptr, nullptr, ered, h2c);
}

// MG_PROLONG_ADD, two coarse cells per thread (and ZC coarse planes per
// thread, keeping the coarse taps X-1..X+2 x Y-1..Y+1 of planes Z-1..Z+1 in
// registers; clamped, 0 above a Dirichlet top; four planes per thread onto
// a fine level of at least 2^22 cells, where the rolling taps save the
// loads (box192's level 0: 18.5 -> 13.6 us), one plane on smaller levels,
// bound by latency): the 16
// fine cells of a coarse plane pair are updated with 8-byte
// read-modify-writes per fine row, all rows of a plane loaded before the
// first store (BLACK: only the colour-1 pair of each row, for a red
// half-sweep to follow).  Weights use the same per-cell formula as
// k_prolong_add.
template <class T, class TC, bool BLACK, int ZC>
__global__ void __launch_bounds__(256, ZC == 4 ? 3 : 4) k_prolong_add2(Grid f, Grid c, int ref, T* __restrict__ a,
                                                      const TC* __restrict__ e, const unsigned int* __restrict__ skip) {
  pdl_wait();
  pdl_trigger();
  if (skip_now(skip)) return;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int Y = blockIdx.y * blockDim.y + threadIdx.y;
  const int Z0 = blockIdx.z * ZC;
  if (2 * q >= c.nx || Y >= c.ny) return;
  const uint32_t hc = (uint32_t)c.nx >> 1, halfc = (uint32_t)(c.n() >> 1);
  auto load_plane = [&](int zz, float (&tp)[3][4]) {
    zz = dob_clampi(zz, 0, c.nz - 1);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const int yy = Y - 1 + j;
      const bool zero_row = ref && yy >= c.ny;
      const int yc = dob_clampi(yy, 0, c.ny - 1);
      const uint32_t rc = ((uint32_t)zz * c.ny + yc) * hc;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int xx = dob_clampi(2 * q - 1 + i, 0, c.nx - 1);
        const float v = ldf(e + (((xx + yc + zz) & 1) ? halfc : 0u) + rc + (uint32_t)(xx >> 1));
        tp[j][i] = zero_row ? 0.0f : v;
      }
    }
  };
  float t[3][3][4];  // coarse taps at (2q-1+i, Y-1+j, Z-1+k)
  load_plane(Z0 - 1, t[0]);
  load_plane(Z0, t[1]);
  const uint32_t hx = (uint32_t)f.nx >> 1, half = (uint32_t)(f.n() >> 1), sz = (uint32_t)f.ny * hx;
  const uint32_t w = 2u * (uint32_t)q;
  // fractional coordinates: x = 4q + i, y = 2Y + dy, z = 2Z + dz
  float fxv[4], fyv[2];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float cx = __fmaf_rn(div_by((float)(4 * q + i) + 0.5f, (float)f.nx, f.rx), (float)c.nx, -0.5f);  // one rounding
    fxv[i] = cx - floorf(cx);
  }
#pragma unroll
  for (int d = 0; d < 2; ++d) {
    const float cy = __fmaf_rn(div_by((float)(2 * Y + d) + 0.5f, (float)f.ny, f.ry), (float)c.ny, -0.5f);
    fyv[d] = cy - floorf(cy);
  }
  // the fine rows of coarse plane Z (BLACK: the colour-1 pair of each row)
  auto load_rows = [&](int Z, float2 (&ve)[2][2], float2 (&vo)[2][2]) {
#pragma unroll
    for (int dz = 0; dz < 2; ++dz)
#pragma unroll
      for (int dy = 0; dy < 2; ++dy) {
        const int y = 2 * Y + dy, z = 2 * Z + dz, par = (y + z) & 1;
        const uint32_t r = (uint32_t)z * sz + (uint32_t)y * hx + w;
        if (BLACK) {
          ve[dz][dy] = Pair<T>::ld(a + half + r);
        } else {
          ve[dz][dy] = Pair<T>::ld(a + (par ? half : 0u) + r);
          vo[dz][dy] = Pair<T>::ld(a + (par ? 0u : half) + r);
        }
      }
  };
  // The fine rows of each coarse plane are loaded before any of its stores,
  // and those of the next plane before this plane's stores (the compiler
  // cannot move a load of `a` above a store through it; the rows of
  // different planes are different words), so a thread's planes overlap
  // their load latencies.
  float2 ve[2][2], vo[2][2];
  load_rows(Z0, ve, vo);
#pragma unroll
  for (int zi = 0; zi < ZC; ++zi) {
    const int Z = Z0 + zi;
    load_plane(Z + 1, t[2]);
    float2 ne[2][2], no[2][2];
    if (zi + 1 < ZC) load_rows(Z + 1, ne, no);
    float fzv[2];
#pragma unroll
    for (int d = 0; d < 2; ++d) {
      const float cz = __fmaf_rn(div_by((float)(2 * Z + d) + 0.5f, (float)f.nz, f.rz), (float)c.nz, -0.5f);
      fzv[d] = cz - floorf(cz);
    }
#pragma unroll
    for (int dz = 0; dz < 2; ++dz)
#pragma unroll
      for (int dy = 0; dy < 2; ++dy) {
        const int y = 2 * Y + dy, z = 2 * Z + dz, par = (y + z) & 1;
        const uint32_t r = (uint32_t)z * sz + (uint32_t)y * hx + w;
        float corr[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          // fine x = 4q+i: base coarse tap 2q-1 + (i+1)/2 -> index (i+1)>>1 into t
          const int bi = (i + 1) >> 1;
          const float fx = fxv[i], fy = fyv[dy], fz = fzv[dz];
          const float x00 = dob_mix(t[dz][dy][bi], t[dz][dy][bi + 1], fx);
          const float x10 = dob_mix(t[dz][dy + 1][bi], t[dz][dy + 1][bi + 1], fx);
          const float x01 = dob_mix(t[dz + 1][dy][bi], t[dz + 1][dy][bi + 1], fx);
          const float x11 = dob_mix(t[dz + 1][dy + 1][bi], t[dz + 1][dy + 1][bi + 1], fx);
          corr[i] = dob_mix(dob_mix(x00, x10, fy), dob_mix(x01, x11, fy), fz);
        }
        if (BLACK) {  // only the colour-1 pair of the row: cells x = 4q + par, 4q + par + 2
          const float2 vb = ve[dz][dy];
          Pair<T>::st(a + half + r,
                      par ? make_float2(vb.x + corr[0], vb.y + corr[2]) : make_float2(vb.x + corr[1], vb.y + corr[3]));
        } else {
          const float2 e2 = ve[dz][dy], o2 = vo[dz][dy];
          Pair<T>::st(a + (par ? half : 0u) + r, make_float2(e2.x + corr[0], e2.y + corr[2]));
          Pair<T>::st(a + (par ? 0u : half) + r, make_float2(o2.x + corr[1], o2.y + corr[3]));
        }
      }
    if (zi + 1 < ZC) {
#pragma unroll
      for (int dz = 0; dz < 2; ++dz)
#pragma unroll
        for (int dy = 0; dy < 2; ++dy) {
          ve[dz][dy] = ne[dz][dy];
          vo[dz][dy] = no[dz][dy];
        }
    }
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        t[0][j][i] = t[1][j][i];
        t[1][j][i] = t[2][j][i];
      }
  }
}

// Exact coarsest-grid solve e = M b with the dense symmetric inverse M
// (n <= 4096 cells).  CTA c forms rows 32c..32c+31 of e: b is gathered into
// shared memory in natural order, lane l of warp w sums M[i][32c + l] b[i]
// over i = w, w + 32, ... (M is symmetric, so column 32c + l is row 32c + l;
// each warp reads 128 consecutive bytes per i; 32 warps keep n/32 loads per
// lane independent), and the warps' partial sums are added in shared memory.  n/32 CTAs read M (up to 4 MB, resident
// in L2 across cycles) in parallel instead of one SM reading all of it.
template <class T>
__global__ void __launch_bounds__(1024) k_coarse_dense(Grid d, const float* __restrict__ M, int n,
                                                      T* __restrict__ e, const T* __restrict__ b,
                                                      const unsigned int* __restrict__ skip) {
  pdl_wait();
  pdl_trigger();
  if (skip_now(skip)) return;
  extern __shared__ float sbv[];  // b in natural order (n), then 32 x 32 partial sums
  float* part = sbv + n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int x = i % d.nx, y = (i / d.nx) % d.ny, z = i / (d.nx * d.ny);
    sbv[i] = ldv(b + rb_index(d, x, y, z));
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int j = blockIdx.x * 32 + lane;
  float acc = 0.0f;
  if (j < n) {
#pragma unroll 8
    for (int i = w; i < n; i += 32) acc = fmaf(M[(size_t)i * n + j], sbv[i], acc);
  }
  part[w * 32 + lane] = acc;
  __syncthreads();
  if (w == 0 && j < n) {
    float sum = part[lane];
#pragma unroll
    for (int k = 1; k < 32; ++k) sum += part[k * 32 + lane];
    const int x = j % d.nx, y = (j / d.nx) % d.ny, z = j / (d.nx * d.ny);
    stf(e + rb_index(d, x, y, z), sum);
  }
}

template <class T>
__global__ void k_fill_zero(T* __restrict__ a, size_t n, const unsigned int* __restrict__ skip) {
  pdl_wait();
  pdl_trigger();
  if (skip_now(skip)) return;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    a[i] = T(0.0f);
}

// MG_COARSE_SOLVE_L3 (fluid.ts:687-739) spread over a thread-block cluster of
// CS CTAs: CTA r owns z-planes [r*pz, (r+1)*pz) of the coarsest grid (pz =
// nz/CS) in its shared memory (natural layout), zero start, `sweeps` sweeps.
// Neighbouring planes of other CTAs are read through distributed shared
// memory; every half-sweep ends with a cluster barrier, so a colour only
// ever reads the other colour's finished values, exactly like the
// reference's single-workgroup solve.
template <class T, int CS>
__global__ void __cluster_dims__(CS, 1, 1) __launch_bounds__(512)
    k_coarse_cluster(Grid d, float h2, int ref, int sweeps, T* __restrict__ e, const T* __restrict__ b,
                     const unsigned int* __restrict__ skip) {
  pdl_wait();
  pdl_trigger();
  cg::cluster_group cl = cg::this_cluster();
  extern __shared__ float csm[];
  const int rank = (int)cl.block_rank();
  const int pz = d.nz / CS;
  const int plane = d.nx * d.ny;
  const int nloc = pz * plane;
  float* se = csm;
  float* sb = csm + nloc;
  const bool skipping = skip_now(skip);  // uniform: every CTA takes the same path
  const int z0 = rank * pz;
  for (int k = threadIdx.x; k < nloc; k += blockDim.x) {
    const int zl = k / plane, rem = k - zl * plane;
    const int y = rem / d.nx, x = rem - y * d.nx;
    se[k] = 0.0f;
    sb[k] = skipping ? 0.0f : rb_at(b, d, x, y, z0 + zl);
  }
  const float* below = rank > 0 ? cl.map_shared_rank(se, rank - 1) + (pz - 1) * plane : nullptr;
  const float* above = rank < CS - 1 ? cl.map_shared_rank(se, rank + 1) : nullptr;
  cl.sync();
  const int nsw = skipping ? 0 : sweeps;
  for (int s = 0; s < nsw; ++s) {
    for (int color = 0; color < 2; ++color) {
      const int hxc = d.nx >> 1;
      for (int q = threadIdx.x; q < (nloc >> 1); q += blockDim.x) {  // the cells of this colour
        const int row = q / hxc, kx = q - row * hxc;
        const int zl = row / d.ny, y = row - zl * d.ny;
        const int z = z0 + zl;
        const int x = 2 * kx + ((y + z + color) & 1);
        const int rem = y * d.nx + x;
        const int k = zl * plane + rem;
        float sumN = 0.0f, diag = ref ? 1.0f : 0.0f;
        if (x > 0) { sumN = sumN + se[k - 1]; diag = diag + 1.0f; }
        if (x < d.nx - 1) { sumN = sumN + se[k + 1]; diag = diag + 1.0f; }
        if (y > 0) { sumN = sumN + se[k - d.nx]; diag = diag + 1.0f; }
        if (y < d.ny - 1) { sumN = sumN + se[k + d.nx]; if (!ref) diag = diag + 1.0f; }
        if (z > 0) { sumN = sumN + (zl > 0 ? se[k - plane] : below[rem]); diag = diag + 1.0f; }
        if (z < d.nz - 1) { sumN = sumN + (zl < pz - 1 ? se[k + plane] : above[rem]); diag = diag + 1.0f; }
        se[k] = as_stored<T>((sumN - h2 * sb[k]) / diag);
      }
      cl.sync();
    }
  }
  if (!skipping)
    for (int k = threadIdx.x; k < nloc; k += blockDim.x) {
      const int zl = k / plane, rem = k - zl * plane;
      const int y = rem / d.nx, x = rem - y * d.nx;
      stf(e + rb_index(d, x, y, z0 + zl), se[k]);
    }
  cl.sync();  // keep this CTA's shared memory alive until its neighbours are done reading it
}

// ---- FP64 pieces ---------------------------------------------------------------------
// Sum of a float array for the FP64 compatibility / mean sums.  Each thread
// accumulates its strided elements as an unevaluated pair hi + lo of floats
// with error-free TwoSum updates (Knuth, TAOCP vol. 2, 4.2.2), which keeps
// the partial exact to about 2^-48 relative without FP64 work per element
// (GB300's FP64 rate is a small fraction of its FP32 rate); the partials are
// then reduced in FP64.
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float x) {
  const float s = hi + x;
  const float bp = s - hi;
  const float err = (hi - (s - bp)) + (x - bp);
  hi = s;
  lo = lo + err;
}
__global__ void k_sum64(const float* __restrict__ a, size_t n, double* __restrict__ part) {
  float hi = 0.0f, lo = 0.0f;
  const size_t n4 = n >> 2;
  const float4* a4 = reinterpret_cast<const float4*>(a);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x) {
    const float4 v = a4[i];
    two_sum_acc(hi, lo, v.x);
    two_sum_acc(hi, lo, v.y);
    two_sum_acc(hi, lo, v.z);
    two_sum_acc(hi, lo, v.w);
  }
  for (size_t i = 4 * n4 + blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    two_sum_acc(hi, lo, a[i]);
  block_sum_store((double)hi + (double)lo, part);
}
// sum of squares: per-thread error-free FP32 accumulation, FP64 across threads
// (16-byte loads: with one word per thread and iteration too few bytes are
// in flight, 33 us for 37.7 MB)
__global__ void k_sumsq64(const float* __restrict__ a, size_t n, double* __restrict__ out) {
  float hi = 0.0f, lo = 0.0f;
  auto acc = [&](float v) {
    const float sq = v * v;
    two_sum_acc(hi, lo, sq);
    lo += fmaf(v, v, -sq);  // the rounding error of the square
  };
  const size_t n4 = n >> 2;
  const float4* a4 = reinterpret_cast<const float4*>(a);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x) {
    const float4 v = a4[i];
    acc(v.x); acc(v.y); acc(v.z); acc(v.w);
  }
  for (size_t i = 4 * n4 + blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    acc(a[i]);
  block_sum_atomic((double)hi + (double)lo, out);
}
// a[i] -= mean, with the mean summed in FP64 (k_sum64's nb partials, added
// in a fixed order) and applied in FP32; sumsq (statistics): also the sum
// of squares of the result, accumulated as k_sumsq64 does (no separate
// pass over the array).
__global__ void k_sub_mean(float* __restrict__ a, size_t n, const double* __restrict__ part, int nb,
                           double* __restrict__ sumsq) {
  __shared__ float s_mean;
  if (threadIdx.x < 32) {
    const double sum = sum_partials(part, nb);
    if (threadIdx.x == 0) s_mean = (float)(sum / (double)n);
  }
  __syncthreads();
  const float mean = s_mean;
  const size_t n4 = n >> 2;
  float4* a4 = reinterpret_cast<float4*>(a);
  float hi = 0.0f, lo = 0.0f;
  auto acc = [&](float v) {
    const float sq = v * v;
    two_sum_acc(hi, lo, sq);
    lo += fmaf(v, v, -sq);
  };
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x) {
    float4 v = a4[i];
    v.x = v.x - mean; v.y = v.y - mean; v.z = v.z - mean; v.w = v.w - mean;
    a4[i] = v;
    if (sumsq) { acc(v.x); acc(v.y); acc(v.z); acc(v.w); }
  }
  for (size_t i = 4 * n4 + blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    a[i] = a[i] - mean;
    if (sumsq) acc(a[i]);
  }
  if (sumsq) block_sum_atomic((double)hi + (double)lo, sumsq);
}

// ---- mixed precision: double-float pressure --------------------------------------------
// The pressure is p + plo (two FP32 arrays, |plo| <= ulp(p)/2), updated with
// error-free transformations, so the residual b - A p can fall far below the
// FP32 rounding of p itself (~1e-5 relative for this problem) with FP32
// arithmetic only.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bp = s - a;
  e = (a - (s - bp)) + (b - bp);
}
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {  // |a| >= |b|
  s = a + b;
  e = b - (s - a);
}
// r = b - A (p + plo) at level 0 (h2 = 1): the neighbour sum of p and
// diag * p are formed exactly as double-float, so the cancellation against b
// loses nothing; r is stored FP32 (split layout, the correction solve's
// right-hand side), max |r| and ||r||^2 are reduced.
__global__ void __launch_bounds__(256) k_defect_df(Grid d, int ref, const float* __restrict__ p,
                                                   const float* __restrict__ plo, const float* __restrict__ b,
                                                   float* __restrict__ r_out, double* __restrict__ norm2,
                                                   unsigned int* __restrict__ maxbits,
                                                   const unsigned int* __restrict__ skip) {
  if (skip_now(skip)) return;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  float rr = 0.0f, ra = 0.0f;
  if (x < d.nx && y < d.ny) {
    float sh = 0.0f, sl = 0.0f, low = 0.0f, diag = ref ? 1.0f : 0.0f;
    auto add = [&](int xx, int yy, int zz) {
      const size_t j = rb_index(d, xx, yy, zz);
      float e;
      two_sum(sh, p[j], sh, e);
      sl += e;
      if (plo) low += plo[j];
      diag += 1.0f;
    };
    if (x > 0) add(x - 1, y, z);
    if (x < d.nx - 1) add(x + 1, y, z);
    if (y > 0) add(x, y - 1, z);
    if (y < d.ny - 1) {
      const size_t j = rb_index(d, x, y + 1, z);
      float e;
      two_sum(sh, p[j], sh, e);
      sl += e;
      if (plo) low += plo[j];
      if (!ref) diag += 1.0f;
    }
    if (z > 0) add(x, y, z - 1);
    if (z < d.nz - 1) add(x, y, z + 1);
    const size_t i = rb_index(d, x, y, z);
    const float pc = p[i];
    const float prod = diag * pc;
    const float perr = fmaf(diag, pc, -prod);  // diag * pc = prod + perr exactly
    float th, te;
    two_sum(sh, -prod, th, te);                // A p = th + (te + sl - perr + low - diag plo)
    const float tl = ((te + sl) - perr) + (plo ? fmaf(-diag, plo[i], low) : low);
    const float r = (b[i] - th) - tl;
    if (r_out) r_out[i] = r;
    rr = r * r;
    ra = fabsf(r);
  }
  if (norm2) block_sum_atomic_f(rr, norm2);
  if (maxbits) block_max_atomic(ra, maxbits);
}

// k_defect_df on the red-black split layout with the smoother's thread
// shape: four consecutive same-colour cells of a row per thread (16-byte
// loads), ZC planes per thread (with ZC > 1 the other colour's row vectors
// serve three planes each), blockIdx.z = 2 * (group of `zs` z-chunks) +
// colour.  Absent neighbours enter with weight 0 (an exact zero added to the
// double-float sum changes nothing), so every cell's r has the bits of
// k_defect_df.  One FP64 add and one max per block: a block walks `zs`
// chunks so that the reductions' same-address atomics stay few (one per
// plane and colour cost 12 of 57 us at 192x256x192; four planes per block:
// 51 us, 78 registers; capped at 64 it spills and runs no faster).  Rows
// with nx % 8 == 0.
template <int ZC>
__global__ void __launch_bounds__(256) k_defect_df4(Grid d, int ref, const float* __restrict__ p,
                                                    const float* __restrict__ plo, const float* __restrict__ b,
                                                    float* __restrict__ r_out, double* __restrict__ norm2,
                                                    unsigned int* __restrict__ maxbits,
                                                    const unsigned int* __restrict__ skip, int zs) {
  pdl_wait();
  pdl_trigger();
  if (skip_now(skip)) return;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int color = blockIdx.z & 1;
  const uint32_t hx = (uint32_t)d.nx >> 1;
  const uint32_t k0 = 4u * (uint32_t)q;
  float rr = 0.0f, ra = 0.0f;
  for (int zc = 0; zc < zs; ++zc) {
    const int z0 = ((blockIdx.z >> 1) * zs + zc) * ZC;
    if (z0 >= d.nz) break;
    if (k0 < hx && y < d.ny) {
      const uint32_t half = (uint32_t)(d.n() >> 1);
      const uint32_t sz = (uint32_t)d.ny * hx;
      const uint32_t own = color ? half : 0u, oth = color ? 0u : half;
      const uint32_t r0 = (uint32_t)z0 * sz + (uint32_t)y * hx + k0;
      const bool has_ym = y > 0, has_yp = y < d.ny - 1;
      const bool has_zlo = z0 > 0, has_zhi = z0 + ZC < d.nz;
      const uint32_t oym = has_ym ? hx : 0u, oyp = has_yp ? hx : 0u;
      const bool has_e0 = k0 > 0, has_e1 = k0 + 4 < hx;
      const uint32_t ke0 = has_e0 ? k0 - 1 : k0, ke1 = has_e1 ? k0 + 4 : k0 + 3;
      const float wym = has_ym ? 1.0f : 0.0f, wyp = has_yp ? 1.0f : 0.0f;
      const int p0 = (y + z0 + color) & 1;
      const bool df = plo != nullptr;
      const float4 zero4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      auto ld4f = [](const float* a) { return *reinterpret_cast<const float4*>(a); };
      const uint32_t rzlo = has_zlo ? r0 - sz : r0, rzhi = has_zhi ? r0 + ZC * sz : r0 + (ZC - 1) * sz;
      float4 C[ZC + 2], L[ZC + 2];  // other colour's p and plo, planes z0 - 1 .. z0 + ZC
      C[0] = ld4f(p + oth + rzlo);
      L[0] = df ? ld4f(plo + oth + rzlo) : zero4;
#pragma unroll
      for (int i = 0; i < ZC; ++i) {
        C[i + 1] = ld4f(p + oth + r0 + i * sz);
        L[i + 1] = df ? ld4f(plo + oth + r0 + i * sz) : zero4;
      }
      C[ZC + 1] = ld4f(p + oth + rzhi);
      L[ZC + 1] = df ? ld4f(plo + oth + rzhi) : zero4;
#pragma unroll
      for (int i = 0; i < ZC; ++i) {
        const uint32_t r = r0 + i * sz;
        const int par = p0 ^ (i & 1);
        const float4 pc = ld4f(p + own + r), bv = ld4f(b + own + r);
        const float4 lc = df ? ld4f(plo + own + r) : zero4;
        const float4 ym = ld4f(p + oth + r - oym), yp = ld4f(p + oth + r + oyp);
        const float4 lym = df ? ld4f(plo + oth + r - oym) : zero4, lyp = df ? ld4f(plo + oth + r + oyp) : zero4;
        const uint32_t kex = r - k0 + (par == 0 ? ke0 : ke1);
        const float ex = p[oth + kex], lex = df ? plo[oth + kex] : 0.0f;
        const float wex = (par == 0 ? has_e0 : has_e1) ? 1.0f : 0.0f;
        const float wzm = (i > 0 || has_zlo) ? 1.0f : 0.0f;
        const float wzp = (i < ZC - 1 || has_zhi) ? 1.0f : 0.0f;
        const float4 cm = C[i + 1], zm = C[i], zp = C[i + 2];
        const float4 lcm = L[i + 1], lzm = L[i], lzp = L[i + 2];
        float res[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const float xm = par == 0 ? (j == 0 ? ex : f4get(cm, j - 1)) : f4get(cm, j);
          const float xp = par == 0 ? f4get(cm, j) : (j == 3 ? ex : f4get(cm, j + 1));
          const float lxm = par == 0 ? (j == 0 ? lex : f4get(lcm, j - 1)) : f4get(lcm, j);
          const float lxp = par == 0 ? f4get(lcm, j) : (j == 3 ? lex : f4get(lcm, j + 1));
          const float wxm = (par == 0 && j == 0) ? wex : 1.0f;
          const float wxp = (par == 1 && j == 3) ? wex : 1.0f;
          // neighbour order x-, x+, y-, y+, z-, z+ as k_defect_df
          const float nv[6] = {wxm * xm, wxp * xp, wym * f4get(ym, j), wyp * f4get(yp, j), wzm * f4get(zm, j),
                               wzp * f4get(zp, j)};
          const float nl[6] = {wxm * lxm, wxp * lxp, wym * f4get(lym, j), wyp * f4get(lyp, j), wzm * f4get(lzm, j),
                               wzp * f4get(lzp, j)};
          float sh = 0.0f, sl = 0.0f, low = 0.0f;
#pragma unroll
          for (int k = 0; k < 6; ++k) {
            float e;
            two_sum(sh, nv[k], sh, e);
            sl += e;
            low += nl[k];
          }
          const float diag = (ref ? 1.0f : 0.0f) + wxm + wxp + wym + (ref ? 0.0f : wyp) + wzm + wzp;
          const float pcj = f4get(pc, j);
          const float prod = diag * pcj;
          const float perr = fmaf(diag, pcj, -prod);
          float th, te;
          two_sum(sh, -prod, th, te);
          const float tl = ((te + sl) - perr) + (df ? fmaf(-diag, f4get(lc, j), low) : low);
          const float rv = (f4get(bv, j) - th) - tl;
          res[j] = rv;
          rr = fmaf(rv, rv, rr);
          ra = fmaxf(ra, fabsf(rv));
        }
        if (r_out) *reinterpret_cast<float4*>(r_out + own + r) = make_float4(res[0], res[1], res[2], res[3]);
      }
    }
  }
  if (norm2) block_sum_atomic_f(rr, norm2);
  if (maxbits) block_max_atomic(ra, maxbits);
}

// Convergence test of the mixed solve: max |r| <= div_tol_r and ||r|| <=
// rel_tol ||b|| (a zero tolerance switches its test off).  The tested slots
// are cleared for the next accumulation.
__device__ __forceinline__ bool mixed_converged(unsigned int* maxbits, double* rnorm2, const double* bnorm2,
                                                float div_tol_r, double rel_tol) {
  const bool div_ok = div_tol_r <= 0.0f || __uint_as_float(*maxbits) <= div_tol_r;
  const double rn = sqrt(*rnorm2), bn = sqrt(*bnorm2);
  const bool rel_ok = rel_tol <= 0.0 || bn == 0.0 || rn <= rel_tol * bn;
  *maxbits = 0u;
  *rnorm2 = 0.0;
  return div_ok && rel_ok;
}

// Test of a round's error-free residual r0 = b - A (p + plo).  Converged (or
// an earlier round was): `done` and `inner_done` make every later kernel of
// the solve return at once (the round's first cycle test then leaves its
// loop off).  Otherwise the round counts, its cycle counter starts at the
// `untested` cycles that open it, which count as completed V-cycles.  With
// `use_cond` the test also sets `cond` (the if-node of a captured round) to
// whether the round runs.
__global__ void k_mixed_round_check(unsigned int* __restrict__ maxbits, double* __restrict__ rnorm2,
                                    const double* __restrict__ bnorm2, float div_tol_r, double rel_tol,
                                    unsigned int* __restrict__ done, unsigned int* __restrict__ inner_done,
                                    unsigned int* __restrict__ rounds, unsigned int* __restrict__ inner_iters,
                                    unsigned int* __restrict__ vcycles, int untested,
                                    cudaGraphConditionalHandle cond, int use_cond) {
  if (*done) {
    *inner_done = 1u;
    if (use_cond) cudaGraphSetConditional(cond, 0u);
    return;
  }
  if (mixed_converged(maxbits, rnorm2, bnorm2, div_tol_r, rel_tol)) {
    *done = 1u;
    *inner_done = 1u;
    if (use_cond) cudaGraphSetConditional(cond, 0u);
    return;
  }
  if (use_cond) cudaGraphSetConditional(cond, 1u);
  *rounds = *rounds + 1u;
  *inner_done = 0u;
  *inner_iters = (unsigned int)untested;
  *vcycles = *vcycles + (unsigned int)untested;
}

// Test of the correction after a V-cycle's level-0 pre-smoothing, on the
// residual r0 - A e that the restriction formed: converged -> `inner_done`
// (the round's remaining kernels return at once where they read it) and the
// loop ends.  Otherwise the cycle goes on; the loop ends once max_cycles
// cycles have begun.  The first test of a round comes before its loop;
// `completes`: the test closes a loop iteration, which completed a cycle.
__global__ void k_mixed_cycle_check(unsigned int* __restrict__ maxbits, double* __restrict__ rnorm2,
                                    const double* __restrict__ bnorm2, float div_tol_r, double rel_tol,
                                    int max_cycles, int completes, unsigned int* __restrict__ inner_done,
                                    unsigned int* __restrict__ inner_iters, unsigned int* __restrict__ vcycles,
                                    cudaGraphConditionalHandle cond, int use_cond) {
  if (*inner_done) {
    *maxbits = 0u;
    *rnorm2 = 0.0;
    if (use_cond) cudaGraphSetConditional(cond, 0u);
    return;
  }
  const unsigned int n = *inner_iters + 1u;  // the cycle this pre-smoothing began
  *inner_iters = n;
  if (completes) *vcycles = *vcycles + 1u;   // the loop body completed the previous cycle
  if (mixed_converged(maxbits, rnorm2, bnorm2, div_tol_r, rel_tol) || n > (unsigned int)max_cycles) {
    *inner_done = 1u;
    if (use_cond) cudaGraphSetConditional(cond, 0u);
    return;
  }
  if (use_cond) cudaGraphSetConditional(cond, 1u);
}

// (p, plo) += e, error-free (same split layout)
__global__ void k_add_df(float* __restrict__ p, float* __restrict__ plo, const float* __restrict__ e, size_t n,
                         const unsigned int* __restrict__ skip) {
  if (skip_now(skip)) return;
  const size_t n4 = n >> 2;
  float4* p4 = reinterpret_cast<float4*>(p);
  float4* l4 = reinterpret_cast<float4*>(plo);
  const float4* e4 = reinterpret_cast<const float4*>(e);
  auto upd = [](float& hi, float& lo, float ev) {
    float s, err;
    two_sum(hi, ev, s, err);
    fast_two_sum(s, err + lo, hi, lo);
  };
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x) {
    float4 h = p4[i], l = l4[i];
    const float4 ev = e4[i];
    upd(h.x, l.x, ev.x); upd(h.y, l.y, ev.y); upd(h.z, l.z, ev.z); upd(h.w, l.w, ev.w);
    p4[i] = h;
    l4[i] = l;
  }
  for (size_t i = 4 * n4 + blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float h = p[i], l = plo[i];
    upd(h, l, e[i]);
    p[i] = h;
    plo[i] = l;
  }
}
// sum of p + plo (per-thread double-float, FP64 across threads)
// (16-byte loads, as k_sum64)
__global__ void k_sum_df(const float* __restrict__ p, const float* __restrict__ plo, size_t n,
                         double* __restrict__ part) {
  float hi = 0.0f, lo = 0.0f;
  auto acc = [&](float ph, float pl) {
    float e;
    two_sum(hi, ph, hi, e);
    lo += e + pl;
  };
  const size_t n4 = n >> 2;
  const float4* p4 = reinterpret_cast<const float4*>(p);
  const float4* l4 = reinterpret_cast<const float4*>(plo);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x) {
    const float4 h = p4[i], l = l4[i];
    acc(h.x, l.x); acc(h.y, l.y); acc(h.z, l.z); acc(h.w, l.w);
  }
  for (size_t i = 4 * n4 + blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    acc(p[i], plo[i]);
  block_sum_store((double)hi + (double)lo, part);
}
// (p, plo) -= mean, with the mean (k_sum_df's nb partials, added in a fixed
// order) as a double-float pair
__global__ void k_sub_mean_df(float* __restrict__ p, float* __restrict__ plo, size_t n,
                              const double* __restrict__ part, int nb) {
  __shared__ float s_mh, s_ml;
  if (threadIdx.x < 32) {
    const double m = sum_partials(part, nb) / (double)n;
    if (threadIdx.x == 0) {
      s_mh = (float)m;
      s_ml = (float)(m - (double)s_mh);
    }
  }
  __syncthreads();
  const float mh = s_mh, ml = s_ml;
  auto upd = [&](float& ph, float& pl) {
    float s, err;
    two_sum(ph, -mh, s, err);
    fast_two_sum(s, (err + pl) - ml, ph, pl);
  };
  const size_t n4 = n >> 2;
  float4* p4 = reinterpret_cast<float4*>(p);
  float4* l4 = reinterpret_cast<float4*>(plo);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x) {
    float4 h = p4[i], l = l4[i];
    upd(h.x, l.x); upd(h.y, l.y); upd(h.z, l.z); upd(h.w, l.w);
    p4[i] = h;
    l4[i] = l;
  }
  for (size_t i = 4 * n4 + blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    upd(p[i], plo[i]);
}

// Natural <-> red-black split layout (host field I/O).
__global__ void k_to_split(const float* __restrict__ nat, float* __restrict__ rb, Grid d) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= d.nx || y >= d.ny) return;
  rb[rb_index(d, x, y, z)] = nat[d.at(x, y, z)];
}
__global__ void k_from_split(const float* __restrict__ rb, float* __restrict__ nat, Grid d) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= d.nx || y >= d.ny) return;
  nat[d.at(x, y, z)] = rb[rb_index(d, x, y, z)];
}

// ---- host side ----------------------------------------------------------------------
static inline dim3 g_cells(const Grid& d) { return dim3((d.nx + 31) / 32, (d.ny + 7) / 8, d.nz); }
static inline dim3 g_half(const Grid& d) { return dim3((d.nx / 2 + 31) / 32, (d.ny + 7) / 8, d.nz); }
static inline dim3 b_cells() { return dim3(32, 8, 1); }
// k_rbgs_v4 launch shape: x over the nx/8 quads of a row, y over rows.
static inline dim3 quad_block(const Grid& d) {
  const int q = d.nx / 8;
  const int bx = q < 256 ? q : 256;
  int by = 256 / bx;
  if (by > d.ny) by = d.ny;
  return dim3(bx, by, 1);
}
// k_residual_restrict2 / k_prolong_add2 launch shape over the coarse grid:
// x over the nx/2 coarse pairs of a row, y over coarse rows.
static inline dim3 pair_block(const Grid& c) {
  const int q = c.nx / 2;
  const int bx = q < 256 ? q : 256;
  int by = 256 / bx;
  if (by > c.ny) by = c.ny;
  return dim3(bx, by, 1);
}
static inline dim3 pair_grid(const Grid& c, const dim3& b) {
  const int q = c.nx / 2;
  return dim3((q + b.x - 1) / b.x, (c.ny + b.y - 1) / b.y, c.nz);
}
// norm2 / maxbits: also reduce ||r||^2 and max |r| of level l's residual
// (the mixed solve's convergence test)
template <class T, class TC = T>
// ered: also the first red half-sweep from zero of level l + 1 (its
// smoothing then starts with the black half-sweep)
static void restrict_level(const DevState& s, int l, const T* x, const T* b, TC* bc, const unsigned int* skip,
                           cudaStream_t st, double* norm2 = nullptr, unsigned int* maxbits = nullptr,
                           TC* ered = nullptr) {
  const Grid f = s.lv[l].d, c = s.lv[l + 1].d;  // nx % 4 == 0 on every transfer level
  const dim3 bp = pair_block(c);
  const float h2c = s.lv[l + 1].h2;
  if (norm2)
    launch_pdl(k_residual_restrict2<T, TC, true>, pair_grid(c, bp), bp, 0, st, f, c, 1.0f / s.lv[l].h2, s.ref, x, b,
               bc, skip, norm2, maxbits, (TC*)nullptr, h2c);
  else
    launch_pdl(k_residual_restrict2<T, TC, false>, pair_grid(c, bp), bp, 0, st, f, c, 1.0f / s.lv[l].h2, s.ref, x, b,
               bc, skip, norm2, maxbits, ered, h2c);
}
static inline dim3 quad_grid(const Grid& d, const dim3& b) {
  const int q = d.nx / 8;
  return dim3((q + b.x - 1) / b.x, (d.ny + b.y - 1) / b.y, d.nz);
}

void launch_split(const float* src, float* dst, const Grid& d, bool to_split, cudaStream_t st) {
  if (to_split) k_to_split<<<g_cells(d), b_cells(), 0, st>>>(src, dst, d);
  else k_from_split<<<g_cells(d), b_cells(), 0, st>>>(src, dst, d);
}

template <class T, int CS>
static cudaError_t cluster_attr() {
  return cudaFuncSetAttribute(k_coarse_cluster<T, CS>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

cudaError_t mg_prepare() {
  cudaError_t e = cluster_attr<float, 8>();
  if (e == cudaSuccess) e = cluster_attr<float, 4>();
  if (e == cudaSuccess) e = cluster_attr<float, 2>();
  if (e == cudaSuccess) e = cluster_attr<float, 1>();
  if (e == cudaSuccess) e = cluster_attr<__nv_bfloat16, 8>();
  if (e == cudaSuccess) e = cluster_attr<__nv_bfloat16, 4>();
  if (e == cudaSuccess) e = cluster_attr<__nv_bfloat16, 2>();
  if (e == cudaSuccess) e = cluster_attr<__nv_bfloat16, 1>();
  return e;
}

// blocks of the partial-sum launches (one slot each in a kSumBlocks array)
static int sum_blocks(int num_sms) { return num_sms * 4 < kSumBlocks ? num_sms * 4 : kSumBlocks; }
void launch_sum(const float* a, size_t n, double* part, int num_sms, cudaStream_t st) {
  k_sum64<<<sum_blocks(num_sms), 256, 0, st>>>(a, n, part);
}
void launch_sub_mean(float* a, size_t n, const double* part, int num_sms, cudaStream_t st, double* sumsq) {
  k_sub_mean<<<num_sms * 4, 256, 0, st>>>(a, n, part, sum_blocks(num_sms), sumsq);
}
void launch_sumsq(const float* a, size_t n, double* out, int num_sms, cudaStream_t st) {
  k_sumsq64<<<num_sms * 4, 256, 0, st>>>(a, n, out);
}

// One half-sweep of colour c on level l: k_rbgs_v4 on rows with nx % 8 == 0,
// else the scalar kernel.  Planes per thread: the most of 4, 2, 1 that still
// leaves two waves of 1024 threads per SM (measured at 192x256x192: 20.5 us
// per red+black pass with 2 planes against 24.6 us with 1; at 96x128x96 one
// plane per thread is fastest).  Every level has even dims, so nz % 2 == 0.
// zoth: the other colour is zero and is not read.
template <class T, bool ZOTH>
static void half_sweep_v4(const DevState& s, const MgLevel& L, int c, T* own, const T* oth, const T* bown,
                          const unsigned int* skip, cudaStream_t st) {
  const dim3 bq = quad_block(L.d);
  dim3 gq = quad_grid(L.d, bq);
  const size_t threads = (L.d.n() >> 1) / 4, wave2 = (size_t)s.num_sms * 2048;
  if (L.d.nz % 4 == 0 && threads / 4 >= wave2) {
    gq.z = L.d.nz / 4;
    launch_pdl(k_rbgs_v4<T, 4, ZOTH>, gq, bq, 0, st, L.d, c, L.h2, s.ref, own, oth, bown, skip);
  } else if (threads / 2 >= wave2) {
    gq.z = L.d.nz / 2;
    launch_pdl(k_rbgs_v4<T, 2, ZOTH>, gq, bq, 0, st, L.d, c, L.h2, s.ref, own, oth, bown, skip);
  } else {
    launch_pdl(k_rbgs_v4<T, 1, ZOTH>, gq, bq, 0, st, L.d, c, L.h2, s.ref, own, oth, bown, skip);
  }
}
template <class T>
static void half_sweep(const DevState& s, int l, int c, bool zoth, T* a, const T* b, const unsigned int* skip,
                       cudaStream_t st) {
  const MgLevel& L = s.lv[l];
  if (L.d.nx % 8 != 0) {
    launch_pdl(k_rbgs_split<T>, g_half(L.d), b_cells(), 0, st, L.d, c, L.h2, s.ref, zoth ? 1 : 0, a, b, skip);
    return;
  }
  const size_t half = L.d.n() >> 1;
  T* own = a + (c ? half : 0);
  const T* oth = a + (c ? 0 : half);
  const T* bown = b + (c ? half : 0);
  if (zoth) half_sweep_v4<T, true>(s, L, c, own, oth, bown, skip, st);
  else half_sweep_v4<T, false>(s, L, c, own, oth, bown, skip, st);
}

// `sweeps` red-black sweeps on level l, in place.  zero_first: the input is
// zero (the first red half-sweep then reads no neighbours, and the black
// half-sweep never reads its own old values, so nothing is filled unless
// there are no sweeps); ec: coarse correction to add first.
// red_done: the first red half-sweep from zero was formed by the restriction
// into this level (restrict_level's ered)
template <class T, class TC = T>
static void smooth(const DevState& s, int l, T* a, const T* b, int sweeps, bool zero_first, const TC* ec,
                   const unsigned int* skip, cudaStream_t st, bool red_done = false) {
  const MgLevel& L = s.lv[l];
  if (zero_first && sweeps == 0) launch_pdl(k_fill_zero<T>, dim3(s.num_sms * 2), dim3(256), 0, st, a, L.d.n(), skip);
  if (ec) {
    // With a sweep to follow, only the black cells need the correction: the
    // red half-sweep overwrites every red cell without reading it, and the
    // black half-sweep then overwrites the black ones (same bits either way).
    const Grid dc = s.lv[l + 1].d;
    const dim3 bp = pair_block(dc);  // every transfer level has nx % 4 == 0
    const dim3 gp = pair_grid(dc, bp);
    if (L.d.n() >= ((size_t)1 << 22) && dc.nz % 4 == 0) {  // four coarse planes per thread
      dim3 g4 = gp;
      g4.z = dc.nz / 4;
      if (sweeps > 0) launch_pdl(k_prolong_add2<T, TC, true, 4>, g4, bp, 0, st, L.d, dc, s.ref, a, ec, skip);
      else launch_pdl(k_prolong_add2<T, TC, false, 4>, g4, bp, 0, st, L.d, dc, s.ref, a, ec, skip);
    } else if (sweeps > 0) {
      launch_pdl(k_prolong_add2<T, TC, true, 1>, gp, bp, 0, st, L.d, dc, s.ref, a, ec, skip);
    } else {
      launch_pdl(k_prolong_add2<T, TC, false, 1>, gp, bp, 0, st, L.d, dc, s.ref, a, ec, skip);
    }
  }
  for (int k = 0; k < sweeps; ++k)
    for (int c = 0; c < 2; ++c) {
      if (red_done && k == 0 && c == 0) continue;
      half_sweep<T>(s, l, c, zero_first && k == 0 && c == 0, a, b, skip, st);
    }
}

template <class T, int CS>
static void launch_cluster(const MgLevel& L, int ref, int sweeps, T* e, const T* b, const unsigned int* skip,
                           cudaStream_t st) {
  const size_t smem = 2 * (L.d.n() / CS) * sizeof(float);
  launch_pdl(k_coarse_cluster<T, CS>, dim3(CS), dim3(512), smem, st, L.d, L.h2, ref, sweeps, e, b, skip);
}

template <class T>
static void coarse_solve(const DevState& s, int l, T* e, const T* b, const unsigned int* skip, cudaStream_t st) {
  const MgLevel& L = s.lv[l];
  if (s.coarse_sweeps < 0) {  // exact: e = M b with the precomputed inverse
    launch_pdl(k_coarse_dense<T>, dim3((s.cn + 31) / 32), dim3(1024), (s.cn + 1024) * sizeof(float), st, L.d,
               s.cinv, s.cn, e, b, skip);
    return;
  }
  int cs = 0;
  for (int c : {8, 4, 2, 1})
    if (L.d.nz % c == 0 && 2 * (L.d.n() / c) * sizeof(float) <= 200 * 1024) { cs = c; break; }
  switch (cs) {
    case 8: launch_cluster<T, 8>(L, s.ref, s.coarse_sweeps, e, b, skip, st); break;
    case 4: launch_cluster<T, 4>(L, s.ref, s.coarse_sweeps, e, b, skip, st); break;
    case 2: launch_cluster<T, 2>(L, s.ref, s.coarse_sweeps, e, b, skip, st); break;
    case 1: launch_cluster<T, 1>(L, s.ref, s.coarse_sweeps, e, b, skip, st); break;
    default: smooth<T, T>(s, l, e, b, s.coarse_sweeps, true, nullptr, skip, st); break;
  }
}

// One V-cycle on (x0, b0); per-level arrays E[l], B[l] for l >= 1.
// zero0: x0 is zero on entry.
template <class T>
static void vcycle(const DevState& s, T* x0, const T* b0, T* const* E, T* const* B, bool zero0,
                   const unsigned int* skip, cudaStream_t st) {
  const int L = s.nlev;
  if (L == 1) {
    smooth<T, T>(s, 0, x0, b0, s.pre + s.post, zero0, nullptr, skip, st);
    return;
  }
  smooth<T, T>(s, 0, x0, b0, s.pre0, zero0, nullptr, skip, st);
  // each level in between starts its smoothing from zero: its first red
  // half-sweep reads only its right-hand side, so the restriction forming
  // that right-hand side also forms it (one launch fewer per level)
  const bool fuse = s.pre > 0;
  restrict_level<T>(s, 0, x0, b0, B[1], skip, st, nullptr, nullptr, fuse && L > 2 ? E[1] : nullptr);
  for (int l = 1; l < L - 1; ++l) {
    smooth<T, T>(s, l, E[l], B[l], s.pre, true, nullptr, skip, st, fuse);
    restrict_level<T>(s, l, E[l], B[l], B[l + 1], skip, st, nullptr, nullptr,
                      fuse && l + 1 < L - 1 ? E[l + 1] : nullptr);
  }
  coarse_solve<T>(s, L - 1, E[L - 1], B[L - 1], skip, st);
  for (int l = L - 2; l >= 1; --l) smooth<T, T>(s, l, E[l], B[l], s.post, false, E[l + 1], skip, st);
  smooth<T, T>(s, 0, x0, b0, s.post0, false, E[1], skip, st);
}

// ---- the mixed-precision correction solve --------------------------------------------------
// Level arrays of the correction V-cycle: FP32 below kMixedBF16Level, BF16
// from it on (the coarse levels carry only the smooth part of the error).
struct MixLv {
  float *ef, *bf;
  __nv_bfloat16 *eh, *bh;
  bool h;
};
static void mix_smooth(const DevState& s, int l, const MixLv* M, int sweeps, bool zero, bool add_coarse,
                       const unsigned int* skip, cudaStream_t st) {
  const bool ch = add_coarse && M[l + 1].h;
  if (M[l].h) {
    smooth<__nv_bfloat16, __nv_bfloat16>(s, l, M[l].eh, M[l].bh, sweeps, zero, add_coarse ? M[l + 1].eh : nullptr,
                                         skip, st);
  } else if (ch) {
    smooth<float, __nv_bfloat16>(s, l, M[l].ef, M[l].bf, sweeps, zero, M[l + 1].eh, skip, st);
  } else {
    smooth<float, float>(s, l, M[l].ef, M[l].bf, sweeps, zero, add_coarse ? M[l + 1].ef : nullptr, skip, st);
  }
}
static void mix_restrict(const DevState& s, int l, const MixLv* M, const unsigned int* skip, cudaStream_t st) {
  if (M[l].h) restrict_level<__nv_bfloat16, __nv_bfloat16>(s, l, M[l].eh, M[l].bh, M[l + 1].bh, skip, st);
  else if (M[l + 1].h) restrict_level<float, __nv_bfloat16>(s, l, M[l].ef, M[l].bf, M[l + 1].bh, skip, st);
  else restrict_level<float, float>(s, l, M[l].ef, M[l].bf, M[l + 1].bf, skip, st);
}
double smoother_pass(const DevState& s, cudaStream_t st) {
  smooth<float, float>(s, 0, s.p, s.rhs, 1, false, nullptr, nullptr, st);
  // a red and a black half-sweep each read the other colour's half and their
  // own right-hand-side half and write their own half: 3 x N/2 words each
  return 2.0 * 3.0 * 0.5 * 4.0 * (double)s.g.n();
}

// r = b - A (p + plo) on the finest grid, ||r||^2 and max |r|: the vector
// kernel on rows with nx % 8 == 0, else one thread per cell.
constexpr int kDefectPlanes = 4;
static void defect(const DevState& s, float* r_out, double* norm2, unsigned int* maxbits, const unsigned int* skip,
                   cudaStream_t st) {
  const Grid& d = s.g;
  if (d.nx % 8 != 0) {
    k_defect_df<<<g_cells(d), b_cells(), 0, st>>>(d, s.ref, s.p, s.plo, s.rhs, r_out, norm2, maxbits, skip);
    return;
  }
  // one plane per thread: 57 us at 192x256x192 against 69 us with two
  // (100 registers) and 144 us for one thread per cell; a block walking
  // kDefectPlanes planes (one reduction per block): 51 us
  const dim3 bq = quad_block(d);
  dim3 gq = quad_grid(d, bq);
  gq.z = 2 * ((d.nz + kDefectPlanes - 1) / kDefectPlanes);
  launch_pdl(k_defect_df4<1>, gq, bq, 0, st, d, s.ref, s.p, s.plo, s.rhs, r_out, norm2, maxbits, skip,
             (int)kDefectPlanes);
}

void launch_residual_norm(const DevState& s, double* out, cudaStream_t st) {
  // the error-free residual of p (+ plo in the mixed mode) in FP32 arithmetic
  cudaMemsetAsync(out, 0, sizeof(double), st);
  defect(s, nullptr, out, nullptr, nullptr, st);
}

// Mixed precision: rounds of defect correction.  Each round forms the
// residual r0 = b - A (p + plo) of the double-float pressure without
// rounding loss and tests it (k_mixed_round_check): converged -> this and
// every later round return at once (device flags, so the step stays one
// captured graph).  Otherwise the round solves A e = r0 by V-cycles on e
// from zero (FP32 levels 0-1, BF16 coarser) and tests, after each cycle's
// level-0 pre-smoothing, the residual r0 - A e that the restriction forms
// anyway (k_residual_restrict2 with its reductions, k_mixed_cycle_check),
// stopping there once it meets the targets; then (p, plo) += e without
// rounding loss.  The correction is small against p, so its FP32 residual
// has no rounding floor at the targets: the error-free residual is formed
// once per round (usually one round per step), not once per V-cycle, and no
// separate check pass runs.  The first round may open with `mg_cycles`
// untested cycles that read no flag.  Inside a stream capture each round's
// loop is a conditional while-node rotated so that each iteration ends at a
// test (body: the rest of a cycle, then the next cycle's pre-smoothing,
// restriction and test), so its kernels read no skip flag; the round's
// first test, before the loop, switches it on.  Each round after the first
// is captured as an if-node that the round's residual test switches on, so
// rounds that are not needed (usually all after the first) launch nothing.
// Outside a capture, kMixedMaxCycles iterations per round are enqueued and
// the kernels after convergence return at once.
static void mixed_solve(const DevState& s, cudaStream_t st) {
  const size_t n = s.g.n();
  MixLv M[kMaxLevels];
  M[0] = {s.e0, s.r0, nullptr, nullptr, false};
  for (int l = 1; l < s.nlev; ++l) {
    const bool h = l >= kMixedBF16Level;
    M[l] = {h ? nullptr : s.lv[l].e, h ? nullptr : s.lv[l].b, h ? s.lv[l].eh : nullptr, h ? s.lv[l].bh : nullptr, h};
  }
  unsigned int* done = s.redu + REDU_DONE;
  unsigned int* inner_done = s.redu + REDU_INNER_DONE;
  double* bn2 = s.red + RED_RHS_NORM2;
  double* rn2 = s.red + RED_DEFECT_NORM2;        // [0] round, [1] cycle
  unsigned int* rmax = s.redu + REDU_DEFECT_MAX;  // [0] round, [1] cycle
  cudaMemsetAsync(s.redu + REDU_DONE, 0, 5 * sizeof(unsigned int), st);  // done .. inner_iters
  cudaMemsetAsync(rmax, 0, 2 * sizeof(unsigned int), st);
  cudaMemsetAsync(s.red + RED_RHS_NORM2, 0, sizeof(double) * (RED_COUNT - RED_RHS_NORM2), st);
  k_sumsq64<<<s.num_sms * 4, 256, 0, st>>>(s.rhs, n, bn2);
  const int rounds = s.max_outer < 1 ? 1 : (s.max_outer > kMixedMaxRounds ? kMixedMaxRounds : s.max_outer);
  const int L = s.nlev;  // >= 2 in the mixed mode
  const int untested = s.cycles < 0 ? 0 : (s.cycles > kMixedMaxCycles ? kMixedMaxCycles : s.cycles);
  // a cycle's level-0 pre-smoothing, restriction and test
  auto head = [&](cudaStream_t q, const unsigned int* skip, cudaGraphConditionalHandle cond, int use_cond,
                  int completes) {
    mix_smooth(s, 0, M, s.pre0, false, false, skip, q);
    restrict_level<float, float>(s, 0, M[0].ef, M[0].bf, M[1].bf, skip, q, rn2 + 1, rmax + 1);
    k_mixed_cycle_check<<<1, 1, 0, q>>>(rmax + 1, rn2 + 1, bn2, s.div_tol_r, s.rel_tol, kMixedMaxCycles, completes,
                                        inner_done, s.redu + REDU_INNER_ITERS, s.redu + REDU_VCYCLES, cond,
                                        use_cond);
  };
  // the rest of the cycle: coarser levels and the level-0 post-smoothing
  auto tail = [&](cudaStream_t q, const unsigned int* skip) {
    for (int l = 1; l < L - 1; ++l) {
      mix_smooth(s, l, M, s.pre, true, false, skip, q);
      mix_restrict(s, l, M, skip, q);
    }
    if (M[L - 1].h) coarse_solve<__nv_bfloat16>(s, L - 1, M[L - 1].eh, M[L - 1].bh, skip, q);
    else coarse_solve<float>(s, L - 1, M[L - 1].ef, M[L - 1].bf, skip, q);
    for (int l = L - 2; l >= 1; --l) mix_smooth(s, l, M, s.post, false, true, skip, q);
    mix_smooth(s, 0, M, s.post0, false, true, skip, q);
  };
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaGraph_t top = nullptr;
  if (s.aux && s.aux2 && cudaStreamGetCaptureInfo(st, &cs, nullptr, &top, nullptr, nullptr, nullptr) != cudaSuccess) {
    cudaGetLastError();
    cs = cudaStreamCaptureStatusNone;
  }
  const bool captured = cs == cudaStreamCaptureStatusActive;
  auto new_handle = [&]() {
    cudaGraphConditionalHandle h = 0;
    cudaGraphConditionalHandleCreate(&h, top, 0u, cudaGraphCondAssignDefault);
    return h;
  };
  // a conditional node after the work captured so far on q; its body is
  // captured on `body` between open_cond and close_cond
  auto open_cond = [&](cudaStream_t q, cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type,
                       cudaStream_t body) {
    cudaStreamCaptureStatus qs;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    cudaStreamGetCaptureInfo(q, &qs, nullptr, &g, &deps, nullptr, &ndeps);
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = type;
    np.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &np);
    cudaStreamBeginCaptureToGraph(body, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                  cudaStreamCaptureModeRelaxed);
    return node;
  };
  auto close_cond = [&](cudaStream_t q, cudaGraphNode_t node, cudaStream_t body) {
    cudaGraph_t g = nullptr;
    cudaStreamEndCapture(body, &g);
    cudaStreamUpdateCaptureDependencies(q, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
  };
  // a round's cycles after its first test: the while-node that the test
  // switched on, or kMixedMaxCycles flag-guarded iterations
  auto cycles = [&](cudaStream_t q, cudaGraphConditionalHandle cond) {
    if (captured) {
      cudaGraphNode_t node = open_cond(q, cond, cudaGraphCondTypeWhile, s.aux);
      tail(s.aux, nullptr);
      head(s.aux, nullptr, cond, 1, 1);
      close_cond(q, node, s.aux);
    } else {
      for (int it = 0; it < kMixedMaxCycles; ++it) {
        tail(q, inner_done);
        head(q, inner_done, 0, 0, 1);
      }
    }
  };
  // round 0: its first `untested` cycles (the first from e = 0) read no
  // flag, so a step whose pressure already meets the targets still runs them
  {
    const cudaGraphConditionalHandle cond = captured ? new_handle() : 0;
    defect(s, s.r0, rn2, rmax, done, st);
    k_mixed_round_check<<<1, 1, 0, st>>>(rmax, rn2, bn2, s.div_tol_r, s.rel_tol, done, inner_done,
                                         s.redu + REDU_ITERS, s.redu + REDU_INNER_ITERS, s.redu + REDU_VCYCLES,
                                         untested, 0, 0);
    for (int c = 0; c < untested; ++c) {
      mix_smooth(s, 0, M, s.pre0, c == 0, false, nullptr, st);
      restrict_level<float, float>(s, 0, M[0].ef, M[0].bf, M[1].bf, nullptr, st);
      tail(st, nullptr);
    }
    if (untested == 0)
      launch_pdl(k_fill_zero<float>, dim3(s.num_sms * 2), dim3(256), 0, st, s.e0, n, (const unsigned int*)done);
    head(st, done, cond, captured ? 1 : 0, 0);
    cycles(st, cond);
    k_add_df<<<s.num_sms * 4, 256, 0, st>>>(s.p, s.plo, s.e0, n, done);
  }
  // the later rounds.  Captured: round r's test (after round r - 1) sets the
  // handle of an if-node that holds the whole round, so a round that is not
  // needed launches nothing; inside it `done` is clear, and its kernels read
  // no flag.  Otherwise every round is enqueued and returns at once once
  // `done` is set.
  if (rounds > 1) {
    cudaGraphConditionalHandle h = captured ? new_handle() : 0;
    defect(s, s.r0, rn2, rmax, done, st);
    k_mixed_round_check<<<1, 1, 0, st>>>(rmax, rn2, bn2, s.div_tol_r, s.rel_tol, done, inner_done,
                                         s.redu + REDU_ITERS, s.redu + REDU_INNER_ITERS, s.redu + REDU_VCYCLES, 0,
                                         h, captured ? 1 : 0);
    for (int r = 1; r < rounds; ++r) {
      const bool last = r + 1 == rounds;
      if (captured) {
        const cudaGraphConditionalHandle cond = new_handle();
        const cudaGraphConditionalHandle next = last ? 0 : new_handle();
        const cudaGraphNode_t node = open_cond(st, h, cudaGraphCondTypeIf, s.aux2);
        launch_pdl(k_fill_zero<float>, dim3(s.num_sms * 2), dim3(256), 0, s.aux2, s.e0, n,
                   (const unsigned int*)nullptr);
        head(s.aux2, nullptr, cond, 1, 0);
        cycles(s.aux2, cond);
        k_add_df<<<s.num_sms * 4, 256, 0, s.aux2>>>(s.p, s.plo, s.e0, n, nullptr);
        if (!last) {
          defect(s, s.r0, rn2, rmax, nullptr, s.aux2);
          k_mixed_round_check<<<1, 1, 0, s.aux2>>>(rmax, rn2, bn2, s.div_tol_r, s.rel_tol, done, inner_done,
                                                   s.redu + REDU_ITERS, s.redu + REDU_INNER_ITERS,
                                                   s.redu + REDU_VCYCLES, 0, next, 1);
        }
        close_cond(st, node, s.aux2);
        h = next;
      } else {
        launch_pdl(k_fill_zero<float>, dim3(s.num_sms * 2), dim3(256), 0, st, s.e0, n, (const unsigned int*)done);
        head(st, done, 0, 0, 0);
        cycles(st, 0);
        k_add_df<<<s.num_sms * 4, 256, 0, st>>>(s.p, s.plo, s.e0, n, done);
        if (!last) {
          defect(s, s.r0, rn2, rmax, done, st);
          k_mixed_round_check<<<1, 1, 0, st>>>(rmax, rn2, bn2, s.div_tol_r, s.rel_tol, done, inner_done,
                                               s.redu + REDU_ITERS, s.redu + REDU_INNER_ITERS,
                                               s.redu + REDU_VCYCLES, 0, 0, 0);
        }
      }
    }
  }
  if (!s.ref) {
    double* part = s.part + PART_P * kSumBlocks;
    k_sum_df<<<sum_blocks(s.num_sms), 256, 0, st>>>(s.p, s.plo, n, part);
    k_sub_mean_df<<<s.num_sms * 4, 256, 0, st>>>(s.p, s.plo, n, part, sum_blocks(s.num_sms));
  }
}

// Eigenpairs of the 1D coarse operator along one axis (graph Laplacian of a
// row of n cells, V[k * n + i] = eigenvector k at cell i, orthonormal):
// Neumann at both ends (closed box; x and z of the reference mode):
// cos(pi k (i + 1/2) / n), 2 - 2 cos(pi k / n); Neumann below and the
// Dirichlet ghost above the top cell (y of the reference mode):
// cos(t (i + 1/2)) with t = pi (k + 1/2) / (n + 1/2), 2 - 2 cos t.
static void axis_eigen(int n, bool dirichlet_top, std::vector<double>& V, std::vector<double>& mu) {
  const double pi = 3.14159265358979323846;
  V.assign((size_t)n * n, 0.0);
  mu.assign(n, 0.0);
  for (int k = 0; k < n; ++k) {
    const double t = dirichlet_top ? pi * (k + 0.5) / (n + 0.5) : pi * k / n;
    mu[k] = 2.0 - 2.0 * std::cos(t);
    double nrm = 0.0;
    for (int i = 0; i < n; ++i) {
      const double v = std::cos(t * (i + 0.5));
      V[(size_t)k * n + i] = v;
      nrm += v * v;
    }
    nrm = 1.0 / std::sqrt(nrm);
    for (int i = 0; i < n; ++i) V[(size_t)k * n + i] *= nrm;
  }
  if (!dirichlet_top) mu[0] = 0.0;  // the constant mode, exactly
}

// Dense (pseudo-)inverse of the coarsest operator A = -L / h2, L the 7-point
// graph Laplacian with the level's boundary terms, in natural cell order.
// L is the Kronecker sum of the three axis operators, so with their
// eigenpairs (v, mu) M = -h2 sum over modes with mu_x + mu_y + mu_z > 0 of
// phi phi^T / (mu_x + mu_y + mu_z), phi = v_x (x) v_y (x) v_z; the zero mode
// of the closed box (the constants) is left out, which gives the
// minimum-norm inverse.  Each column is formed by three 1D transforms:
// O(n (nx + ny + nz)) per column instead of Gauss-Jordan's O(n^2).
std::vector<float> coarse_inverse(const Grid& c, float h2, int ref) {
  const int nx = c.nx, ny = c.ny, nz = c.nz, n = (int)c.n();
  std::vector<double> Vx, Vy, Vz, mx, my, mz;
  axis_eigen(nx, false, Vx, mx);
  axis_eigen(ny, ref != 0, Vy, my);
  axis_eigen(nz, false, Vz, mz);
  std::vector<float> out((size_t)n * n);
  std::vector<double> coef((size_t)n), t1((size_t)n), t2((size_t)n);
  for (int bz = 0; bz < nz; ++bz)
    for (int by = 0; by < ny; ++by)
      for (int bx = 0; bx < nx; ++bx) {
        const int b = (bz * ny + by) * nx + bx;
        // coef[l][j][i] = v_i(bx) v_j(by) v_l(bz) / mu_ijl
        for (int l = 0; l < nz; ++l)
          for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
              const double m = mx[i] + my[j] + mz[l];
              coef[((size_t)l * ny + j) * nx + i] =
                  m > 0.0 ? Vx[(size_t)i * nx + bx] * Vy[(size_t)j * ny + by] * Vz[(size_t)l * nz + bz] / m : 0.0;
            }
        // back to cells: x, then y, then z
        for (int l = 0; l < nz; ++l)
          for (int j = 0; j < ny; ++j)
            for (int ax = 0; ax < nx; ++ax) {
              double acc = 0.0;
              for (int i = 0; i < nx; ++i) acc += Vx[(size_t)i * nx + ax] * coef[((size_t)l * ny + j) * nx + i];
              t1[((size_t)l * ny + j) * nx + ax] = acc;
            }
        for (int l = 0; l < nz; ++l)
          for (int ay = 0; ay < ny; ++ay)
            for (int ax = 0; ax < nx; ++ax) {
              double acc = 0.0;
              for (int j = 0; j < ny; ++j) acc += Vy[(size_t)j * ny + ay] * t1[((size_t)l * ny + j) * nx + ax];
              t2[((size_t)l * ny + ay) * nx + ax] = acc;
            }
        for (int az = 0; az < nz; ++az)
          for (int ay = 0; ay < ny; ++ay)
            for (int ax = 0; ax < nx; ++ax) {
              double acc = 0.0;
              for (int l = 0; l < nz; ++l) acc += Vz[(size_t)l * nz + az] * t2[((size_t)l * ny + ay) * nx + ax];
              out[(size_t)((az * ny + ay) * nx + ax) * n + b] = (float)(-(double)h2 * acc);
            }
      }
  return out;
}

void launch_pressure_solve(const DevState& s, cudaStream_t st) {
  if (s.prec == DOB_PREC_MIXED) {
    mixed_solve(s, st);
    return;
  }
  const size_t n = s.g.n();
  float *E[kMaxLevels], *B[kMaxLevels];
  for (int l = 0; l < s.nlev; ++l) { E[l] = s.lv[l].e; B[l] = s.lv[l].b; }
  for (int c = 0; c < s.cycles; ++c) vcycle<float>(s, s.p, s.rhs, E, B, false, nullptr, st);
  if (!s.ref) {
    launch_sum(s.p, n, s.part + PART_P * kSumBlocks, s.num_sms, st);
    launch_sub_mean(s.p, n, s.part + PART_P * kSumBlocks, s.num_sms, st);
  }
}

}  // namespace dob
