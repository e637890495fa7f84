// dob_device.cuh — device-side data layout and shared helpers of the
// GB300 fluid step.
//
// HBM layout (x fastest, index = (z*ny + y)*nx + x):
//   MAC velocity   u, v, w       3 SoA arrays of VS (float | binary16)
//   centre velocity              AoS 4 x VS (x, y, z, 0) — one 16 B (8 B) gather per tap
//   curl                         AoS 4 x VS (wx, wy, wz, |w|)
//   pressure p, rhs b            float; MG levels float (BF16 in the mixed inner solve)
//   conc (reference mode)        AoS 4 x DS (intact, lysed, ox/shear, bed) on the dye grid
//   dye  (closed box)            1 x DS on the dye grid
//   predictor                    1 x DS (the .g channel CONC_PREDICT writes)
//   splat accumulators           2 x u32 on the dye grid
//   parcels                      AoS 8 x float (RbcParcel, 32 B)
// VS/DS are the velocity/dye storage types; arithmetic is always FP32.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include "dob_math.h"

namespace dob {

constexpr int kMaxDrops = 8;
constexpr int kWaveN = 512;
constexpr float kSplatScale = 65536.0f;
constexpr float kSplatInv = 1.52587891e-5f;  // (1/65536).toExponential(8), advect.ts:125
constexpr float kParcelMass = 0.13400f;      // particles.ts:14, 177

// Per-step parameters, resident in device memory and refreshed by one small
// host->device copy before each step (so a captured step graph stays valid).
struct StepParams {
  float U[128];        // the reference's SimUniforms block (common.ts:31-43)
  float dt;            // effective dt (reference: clamp(U[38], 0, 0.025))
  float dmin[3];
  float dmax[3];
  float dsize[3];
  float rdsize[3];     // 1 / dsize (IEEE quotients, formed on the host)
  float damp;          // advection damping
  float sharp;         // MacCormack sharpness
  float tau_y, mu_p, dx;
  uint32_t spawn_count;
  uint32_t cursor;
  uint32_t high_water;
  uint32_t advect_count;
  int32_t step_index;
};

struct Grid {
  int nx, ny, nz;
  // 1/nx, 1/ny, 1/nz as IEEE quotients (make_grid): the kernels divide by the
  // grid's dimensions through them (div_by) instead of forming the
  // reciprocals per thread.  Grids built only for indexing leave them 0.
  float rx, ry, rz;
  __host__ __device__ size_t n() const { return (size_t)nx * ny * nz; }
  __host__ __device__ size_t at(int x, int y, int z) const { return ((size_t)z * ny + y) * nx + x; }
};
inline Grid make_grid(int nx, int ny, int nz) {
  return Grid{nx, ny, nz, 1.0f / (float)nx, 1.0f / (float)ny, 1.0f / (float)nz};
}

// ---- storage types -------------------------------------------------------------
struct alignas(8) half4 {
  __half x, y, z, w;
};

template <class S> struct Vec4Of;
template <> struct Vec4Of<float> { using type = float4; };
template <> struct Vec4Of<__half> { using type = half4; };

__device__ __forceinline__ float ldf(const float* p) { return __ldg(p); }
__device__ __forceinline__ float ldf(const __half* p) { return __half2float(__ldg(p)); }
__device__ __forceinline__ float ldf(const __nv_bfloat16* p) { return __bfloat162float(__ldg(p)); }
__device__ __forceinline__ float ldv(const float* p) { return *p; }
__device__ __forceinline__ float ldv(const __half* p) { return __half2float(*p); }
__device__ __forceinline__ float ldv(const __nv_bfloat16* p) { return __bfloat162float(*p); }
__device__ __forceinline__ void stf(float* p, float v) { *p = v; }
__device__ __forceinline__ void stf(__half* p, float v) { *p = __float2half_rn(v); }
__device__ __forceinline__ void stf(__nv_bfloat16* p, float v) { *p = __float2bfloat16_rn(v); }

__device__ __forceinline__ float4 ld4(const float4* p) { return __ldg(p); }
__device__ __forceinline__ float4 ld4(const half4* p) {
  const uint2 r = __ldg(reinterpret_cast<const uint2*>(p));
  const __half2 a = *reinterpret_cast<const __half2*>(&r.x);
  const __half2 b = *reinterpret_cast<const __half2*>(&r.y);
  const float2 fa = __half22float2(a), fb = __half22float2(b);
  return make_float4(fa.x, fa.y, fb.x, fb.y);
}
__device__ __forceinline__ void st4(float4* p, float4 v) { *p = v; }
__device__ __forceinline__ void st4(half4* p, float4 v) {
  const __half2 a = __floats2half2_rn(v.x, v.y);
  const __half2 b = __floats2half2_rn(v.z, v.w);
  uint2 r;
  r.x = *reinterpret_cast<const uint32_t*>(&a);
  r.y = *reinterpret_cast<const uint32_t*>(&b);
  *reinterpret_cast<uint2*>(p) = r;
}

// ---- WebGPU linear / clamp-to-edge sampling (texel = uvw*dims - 0.5) ----------
// The 8 taps are base + {0,ox} + {0,oy} + {0,oz} with 32-bit offsets (grids
// are limited to < 2^31 cells); clamping to the edge makes an offset 0.
struct Taps {
  uint32_t base, ox, oy, oz;
  float fx, fy, fz;
};
__device__ __forceinline__ Taps taps_at(const Grid& g, float cx, float cy, float cz) {  // texel coordinates
  Taps t;
  const float bx = floorf(cx), by = floorf(cy), bz = floorf(cz);
  t.fx = cx - bx; t.fy = cy - by; t.fz = cz - bz;
  const int ix = (int)bx, iy = (int)by, iz = (int)bz;
  const int x0 = dob_clampi(ix, 0, g.nx - 1), x1 = dob_clampi(ix + 1, 0, g.nx - 1);
  const int y0 = dob_clampi(iy, 0, g.ny - 1), y1 = dob_clampi(iy + 1, 0, g.ny - 1);
  const int z0 = dob_clampi(iz, 0, g.nz - 1), z1 = dob_clampi(iz + 1, 0, g.nz - 1);
  const uint32_t sy = (uint32_t)g.nx, sz = (uint32_t)g.nx * (uint32_t)g.ny;
  t.base = (uint32_t)z0 * sz + (uint32_t)y0 * sy + (uint32_t)x0;
  t.ox = (uint32_t)(x1 - x0);
  t.oy = (uint32_t)(y1 - y0) * sy;
  t.oz = (uint32_t)(z1 - z0) * sz;
  return t;
}
// texel coordinate u n - 1/2 as one FMA (the same bits in every kernel;
// unfused under DOB_UNFUSED)
__device__ __forceinline__ float texel(float u, int n) {
#if defined(DOB_UNFUSED)
  return u * (float)n - 0.5f;
#else
  return __fmaf_rn(u, (float)n, -0.5f);
#endif
}
__device__ __forceinline__ Taps make_taps(const Grid& g, float u, float v, float w) {
  return taps_at(g, texel(u, g.nx), texel(v, g.ny), texel(w, g.nz));
}
// make_taps for coordinates in [0.001, 0.999], where the semi-Lagrangian
// kernels clamp every sample point first: the floor of u n - 1/2 is then in
// [-1, n-1], so only the lower tap can leave the grid (below) and only the
// upper one (above), and each is clamped at that one end: the same taps
// with two integer operations per axis fewer.
__device__ __forceinline__ Taps make_taps_in(const Grid& g, float u, float v, float w) {
  const float cx = texel(u, g.nx), cy = texel(v, g.ny), cz = texel(w, g.nz);
  Taps t;
  const float bx = floorf(cx), by = floorf(cy), bz = floorf(cz);
  t.fx = cx - bx; t.fy = cy - by; t.fz = cz - bz;
  const int ix = (int)bx, iy = (int)by, iz = (int)bz;
  const int x0 = max(ix, 0), x1 = min(ix + 1, g.nx - 1);
  const int y0 = max(iy, 0), y1 = min(iy + 1, g.ny - 1);
  const int z0 = max(iz, 0), z1 = min(iz + 1, g.nz - 1);
  const uint32_t sy = (uint32_t)g.nx, sz = (uint32_t)g.nx * (uint32_t)g.ny;
  t.base = (uint32_t)z0 * sz + (uint32_t)y0 * sy + (uint32_t)x0;
  t.ox = (uint32_t)(x1 - x0);
  t.oy = (uint32_t)(y1 - y0) * sy;
  t.oz = (uint32_t)(z1 - z0) * sz;
  return t;
}
// make_taps with the texel coordinate formed without FMA contraction (the
// rounded product, then the subtraction), as the host oracle forms it.  At
// a fixed cell-centre or face-centre point uvw * dims rounds back to the
// exact texel coordinate on the grids used here, so the fractional parts
// are exact (0 or 1/2) and the taps of weight 0 carry exactly 0, which the
// adjoint's scatter skips.
__device__ __forceinline__ float texel_exact(float u, int n) { return __fadd_rn(__fmul_rn(u, (float)n), -0.5f); }
__device__ __forceinline__ Taps make_taps_exact(const Grid& g, float u, float v, float w) {
  return taps_at(g, texel_exact(u, g.nx), texel_exact(v, g.ny), texel_exact(w, g.nz));
}
template <class S> __device__ __forceinline__ float lerp8(const Taps& t, const S* a) {
  const S* p = a + t.base;
  const float x00 = dob_mix(ldf(p), ldf(p + t.ox), t.fx);
  const float x10 = dob_mix(ldf(p + t.oy), ldf(p + t.oy + t.ox), t.fx);
  const float x01 = dob_mix(ldf(p + t.oz), ldf(p + t.oz + t.ox), t.fx);
  const float x11 = dob_mix(ldf(p + t.oz + t.oy), ldf(p + t.oz + t.oy + t.ox), t.fx);
  const float y0 = dob_mix(x00, x10, t.fy);
  const float y1 = dob_mix(x01, x11, t.fy);
  return dob_mix(y0, y1, t.fz);
}
// The 8 taps of a scalar field; lerp8 of them, and their minimum and maximum
// (the MacCormack limiter's bracket: the trees keep the second operand on
// ties, in the tap order base, +x, +y, +xy, +z, +xz, +yz, +xyz).
template <class S> __device__ __forceinline__ void load8(const Taps& t, const S* a, float c[8]) {
  const S* p = a + t.base;
  c[0] = ldf(p); c[1] = ldf(p + t.ox); c[2] = ldf(p + t.oy); c[3] = ldf(p + t.oy + t.ox);
  c[4] = ldf(p + t.oz); c[5] = ldf(p + t.oz + t.ox); c[6] = ldf(p + t.oz + t.oy); c[7] = ldf(p + t.oz + t.oy + t.ox);
}
__device__ __forceinline__ float min8(const float c[8]) {
  return dob_minf(dob_minf(dob_minf(c[0], c[1]), dob_minf(c[2], c[3])), dob_minf(dob_minf(c[4], c[5]), dob_minf(c[6], c[7])));
}
__device__ __forceinline__ float max8(const float c[8]) {
  return dob_maxf(dob_maxf(dob_maxf(c[0], c[1]), dob_maxf(c[2], c[3])), dob_maxf(dob_maxf(c[4], c[5]), dob_maxf(c[6], c[7])));
}
__device__ __forceinline__ float tri(float c000, float c100, float c010, float c110, float c001, float c101,
                                     float c011, float c111, const Taps& t) {
  const float x00 = dob_mix(c000, c100, t.fx), x10 = dob_mix(c010, c110, t.fx);
  const float x01 = dob_mix(c001, c101, t.fx), x11 = dob_mix(c011, c111, t.fx);
  return dob_mix(dob_mix(x00, x10, t.fy), dob_mix(x01, x11, t.fy), t.fz);
}
// Interpolate the first `NC` channels (3 or 4) of a 4-wide AoS field.
template <int NC, class V4> __device__ __forceinline__ float4 lerp8xn(const Taps& t, const V4* a) {
  const V4* p = a + t.base;
  const float4 c0 = ld4(p), c1 = ld4(p + t.ox), c2 = ld4(p + t.oy), c3 = ld4(p + t.oy + t.ox);
  const float4 c4 = ld4(p + t.oz), c5 = ld4(p + t.oz + t.ox), c6 = ld4(p + t.oz + t.oy);
  const float4 c7 = ld4(p + t.oz + t.oy + t.ox);
  float4 r;
  r.x = tri(c0.x, c1.x, c2.x, c3.x, c4.x, c5.x, c6.x, c7.x, t);
  r.y = tri(c0.y, c1.y, c2.y, c3.y, c4.y, c5.y, c6.y, c7.y, t);
  r.z = tri(c0.z, c1.z, c2.z, c3.z, c4.z, c5.z, c6.z, c7.z, t);
  r.w = NC == 4 ? tri(c0.w, c1.w, c2.w, c3.w, c4.w, c5.w, c6.w, c7.w, t) : 0.0f;
  return r;
}
template <class V4> __device__ __forceinline__ float4 lerp8x4(const Taps& t, const V4* a) { return lerp8xn<4>(t, a); }
template <class V4> __device__ __forceinline__ dob_v3 sample_center(const Grid& g, const V4* cen, dob_v3 uvw) {
  const Taps t = make_taps(g, uvw.x, uvw.y, uvw.z);
  const float4 r = lerp8xn<3>(t, cen);
  return v3(r.x, r.y, r.z);
}
// sample_center at a point clamped to [0.001, 0.999] (make_taps_in)
template <class V4> __device__ __forceinline__ dob_v3 sample_center_in(const Grid& g, const V4* cen, dob_v3 uvw) {
  const Taps t = make_taps_in(g, uvw.x, uvw.y, uvw.z);
  const float4 r = lerp8xn<3>(t, cen);
  return v3(r.x, r.y, r.z);
}
// First three channels of a 4-wide AoS field at taps of a fixed cell-centre
// or face-centre point (make_taps_exact).  There at least two of the three
// fractions are exactly 0, and the 8-tap interpolation reduces to a linear
// interpolation along the remaining axis (mixing with weight exactly 0
// returns the first operand), so only two taps are read: the same value (up
// to the sign of a zero) for a quarter of the loads.  Other taps take the
// 8-tap path.
template <class V4> __device__ __forceinline__ dob_v3 lerp8x3_fixed(const Taps& t, const V4* cen) {
  uint32_t o;
  float f;
  if (t.fy == 0.0f && t.fz == 0.0f) { o = t.ox; f = t.fx; }
  else if (t.fx == 0.0f && t.fz == 0.0f) { o = t.oy; f = t.fy; }
  else if (t.fx == 0.0f && t.fy == 0.0f) { o = t.oz; f = t.fz; }
  else {
    const float4 r = lerp8xn<3>(t, cen);
    return v3(r.x, r.y, r.z);
  }
  const float4 c0 = ld4(cen + t.base), c1 = ld4(cen + t.base + o);
  return v3(dob_mix(c0.x, c1.x, f), dob_mix(c0.y, c1.y, f), dob_mix(c0.z, c1.z, f));
}
// the centre velocity at a fixed cell-centre or face-centre point
template <class V4> __device__ __forceinline__ dob_v3 sample_center_exact(const Grid& g, const V4* cen, dob_v3 uvw) {
  return lerp8x3_fixed(make_taps_exact(g, uvw.x, uvw.y, uvw.z), cen);
}
// sample_center_exact at the centre of cell i = (x, y, z) of g, uvw =
// (index + 1/2) / dims.  When the texel coordinates come out as the cell's
// indices, all three fractions are 0 and the interpolation is the cell's
// own value (up to the sign of a zero, which the traces that use it cannot
// see: they add the displacement to a coordinate of at least 1e-3), read
// directly instead of forming the taps.
template <class V4>
__device__ __forceinline__ dob_v3 center_at_cell(const Grid& g, const V4* cen, dob_v3 uvw, int x, int y, int z,
                                                 size_t i) {
  if (texel_exact(uvw.x, g.nx) == (float)x && texel_exact(uvw.y, g.ny) == (float)y &&
      texel_exact(uvw.z, g.nz) == (float)z) {
    const float4 c = ld4(cen + i);
    return v3(c.x, c.y, c.z);
  }
  return sample_center_exact(g, cen, uvw);
}
// sample_center_exact at the centre of the upper face of cell i normal to
// one axis (o: the index step to the cell across the face) when the face's
// texel coordinates are exact (index + 1/2 along the axis, the indices
// across it): the two taps of weight 1/2 that lerp8x3_fixed reads.
template <class V4> __device__ __forceinline__ dob_v3 face_mean(const V4* cen, size_t i, size_t o) {
  const float4 a = ld4(cen + i), b = ld4(cen + i + o);
  const float h = 0.5f;
  return v3(dob_mix(a.x, b.x, h), dob_mix(a.y, b.y, h), dob_mix(a.z, b.z, h));
}

// 512x512 wave texture, bilinear clamp-to-edge, worldXZToWaveUV (common.ts:65-67).
__device__ __forceinline__ float4 sample_wave(const float4* wave, float x, float z, float lo, float hi) {
  const float su = dob_clampf((x + 1.60f) / 3.20f, lo, hi);
  const float sv = dob_clampf((z + 1.60f) / 3.20f, lo, hi);
  const float cx = su * (float)kWaveN - 0.5f, cy = sv * (float)kWaveN - 0.5f;
  const float bx = floorf(cx), by = floorf(cy);
  const float fx = cx - bx, fy = cy - by;
  const int x0 = dob_clampi((int)bx, 0, kWaveN - 1), x1 = dob_clampi((int)bx + 1, 0, kWaveN - 1);
  const int y0 = dob_clampi((int)by, 0, kWaveN - 1), y1 = dob_clampi((int)by + 1, 0, kWaveN - 1);
  const float4 a00 = __ldg(wave + y0 * kWaveN + x0), a10 = __ldg(wave + y0 * kWaveN + x1);
  const float4 a01 = __ldg(wave + y1 * kWaveN + x0), a11 = __ldg(wave + y1 * kWaveN + x1);
  float4 r;
  r.x = dob_mix(dob_mix(a00.x, a10.x, fx), dob_mix(a01.x, a11.x, fx), fy);
  r.y = dob_mix(dob_mix(a00.y, a10.y, fx), dob_mix(a01.y, a11.y, fx), fy);
  r.z = dob_mix(dob_mix(a00.z, a10.z, fx), dob_mix(a01.z, a11.z, fx), fy);
  r.w = dob_mix(dob_mix(a00.w, a10.w, fx), dob_mix(a01.w, a11.w, fx), fy);
  return r;
}

__device__ __forceinline__ dob_v3 dmin_of(const StepParams& P) { return v3(P.dmin[0], P.dmin[1], P.dmin[2]); }
__device__ __forceinline__ dob_v3 dsize_of(const StepParams& P) { return v3(P.dsize[0], P.dsize[1], P.dsize[2]); }
__device__ __forceinline__ dob_v3 to_world(const StepParams& P, dob_v3 uvw) { return dmin_of(P) + uvw * dsize_of(P); }
__device__ __forceinline__ dob_v3 to_uvw(const StepParams& P, dob_v3 p) { return (p - dmin_of(P)) / dsize_of(P); }
__device__ __forceinline__ float drop(const StepParams& P, int d, int k) { return P.U[64 + 8 * d + k]; }

// ---- division by a per-launch divisor ----------------------------------------------
// a / d from the correctly rounded reciprocal rd = 1/d, with one remainder
// correction (Markstein, "Computation of elementary functions on the IBM
// RISC System/6000 processor", IBM J. Res. Dev. 34(1), 1990): q = RN(a rd)
// is within one ulp of a/d, the remainder a - d q is exact in one FMA, and
// RN(q + (a - d q) rd) is the correctly rounded quotient a/d, barring
// overflow and subnormal intermediates.  Three instructions against the
// IEEE division's subroutine.  Used for texture coordinates (cell index /
// dims, displacement / domain size), which are then added to or subtracted
// from a coordinate of at least 1e-3: there a subnormal quotient (which may
// differ in its last place) and -0/d (which gives +0) leave the result
// unchanged, so the coordinates equal the IEEE division's; for the
// adjoints of those displacements, where the two cases change nothing
// above 2^-126; and for the Casson coefficients (a shear rate / 2 dx and
// nu dt / dx^2: non-negative numerators, zero or normal), where the theorem
// gives the IEEE quotient itself.
struct Recip3 {
  dob_v3 d, r;
};
__device__ __forceinline__ Recip3 recip3(dob_v3 d) { return {d, v3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z)}; }
// the grid's dimensions and the domain size with their host-formed reciprocals
__device__ __forceinline__ Recip3 grid_recip(const Grid& g) {
  return {v3((float)g.nx, (float)g.ny, (float)g.nz), v3(g.rx, g.ry, g.rz)};
}
__device__ __forceinline__ Recip3 dom_recip(const StepParams& P) {
  return {v3(P.dsize[0], P.dsize[1], P.dsize[2]), v3(P.rdsize[0], P.rdsize[1], P.rdsize[2])};
}
__device__ __forceinline__ float div_by(float a, float d, float rd) {
  const float q = __fmul_rn(a, rd);
  return __fmaf_rn(__fmaf_rn(-q, d, a), rd, q);
}
__device__ __forceinline__ dob_v3 operator/(dob_v3 a, const Recip3& b) {
  return v3(div_by(a.x, b.d.x, b.r.x), div_by(a.y, b.d.y, b.r.y), div_by(a.z, b.d.z, b.r.z));
}

}  // namespace dob
