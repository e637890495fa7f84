// k_adjoint.cu — discrete adjoint (transpose of the Jacobian) of every stage
// of the closed-box step, FP32 and mixed precision.
//
// Each kernel is the exact transpose of the linearisation of one forward
// kernel at the forward state it is given (the "tape"):
//   advection        transpose of the trilinear interpolation of the face
//                    values at the departure point, plus the chain through
//                    the RK2 departure point into the centre velocity
//                    (scattered with atomics: several cells can sample the
//                    same texel)
//   centre average   transpose of the face -> centre average
//   Casson viscosity explicit Laplacian with coefficient alpha(|grad u|, c):
//                    transpose of the stencil plus the alpha chain (two
//                    passes: per-cell coefficients, then a gather)
//   divergence / projection  D^T and G^T with the wall masks
//   pressure solve   FP32 (a fixed number of V-cycles): every V-cycle run
//                    backwards with the transposed smoother half-sweeps,
//                    restriction and prolongation; mixed (solved to a
//                    tolerance): the adjoint of an exact solve, the same
//                    solver on the adjoint right-hand side
//   dye predict / MacCormack resolve  transposed samples; the limiter passes
//                    the adjoint through, or to the neighbourhood tap that
//                    supplied the clamped value
// Where the forward is not differentiable (clamps at their bounds, the
// limiter's min/max selection, |grad u| = 0) the adjoint takes the branch the
// forward took, i.e. the one-sided derivative of the executed expression.
//
// Adjoint arrays are FP32, natural layout except the pressure / right-hand
// side / multigrid ones (red-black split like their forward arrays).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "dob_kernels.cuh"

namespace cg = cooperative_groups;

namespace dob {

// ---- trilinear helpers --------------------------------------------------------------------
__device__ __forceinline__ void tri_w(const Taps& t, float w[8]) {
  const float gx = 1.0f - t.fx, gy = 1.0f - t.fy, gz = 1.0f - t.fz;
  w[0] = gx * gy * gz; w[1] = t.fx * gy * gz; w[2] = gx * t.fy * gz; w[3] = t.fx * t.fy * gz;
  w[4] = gx * gy * t.fz; w[5] = t.fx * gy * t.fz; w[6] = gx * t.fy * t.fz; w[7] = t.fx * t.fy * t.fz;
}
__device__ __forceinline__ uint32_t tap_at(const Taps& t, int k) {
  return t.base + ((k & 1) ? t.ox : 0u) + ((k & 2) ? t.oy : 0u) + ((k & 4) ? t.oz : 0u);
}
// d lerp8 / d(fx, fy, fz) of a scalar field.  Linear interpolation has a
// slope kink at every grid node; where a sample sits on a node along an axis
// (e.g. a departure point of fluid at rest) the slope along that axis is the
// mean of the slopes on either side, the value central differences see.  "On
// a node" means a fraction of exactly 0 (kNodeBand = 0; a positive band would
// also catch samples within that many texel units of a node from either side).
// NodeLo gives the element offsets from the base node to the node below it
// and from the node above the base to the next one (0 where clamp-to-edge
// makes the function flat).
constexpr float kNodeBand = 0.0f;
struct NodeLo {
  uint32_t lx, ly, lz;  // base -> base - 1
  uint32_t hx, hy, hz;  // base + 1 -> base + 2
};
__device__ __forceinline__ NodeLo node_lo(const Grid& g, float u, float v, float w) {
  const int ix = dob_clampi((int)floorf(texel(u, g.nx)), 0, g.nx - 1);  // as make_taps forms it
  const int iy = dob_clampi((int)floorf(texel(v, g.ny)), 0, g.ny - 1);
  const int iz = dob_clampi((int)floorf(texel(w, g.nz)), 0, g.nz - 1);
  const uint32_t sy = (uint32_t)g.nx, sz = (uint32_t)g.nx * (uint32_t)g.ny;
  NodeLo n;
  n.lx = ix > 0 ? 1u : 0u;
  n.ly = iy > 0 ? sy : 0u;
  n.lz = iz > 0 ? sz : 0u;
  n.hx = ix + 2 <= g.nx - 1 ? 1u : 0u;
  n.hy = iy + 2 <= g.ny - 1 ? sy : 0u;
  n.hz = iz + 2 <= g.nz - 1 ? sz : 0u;
  return n;
}
template <class F>
__device__ __forceinline__ dob_v3 dfrac_core(const Taps& t, const NodeLo& n, F val) {
  const uint32_t b = t.base;
  const float c0 = val(b), c1 = val(b + t.ox), c2 = val(b + t.oy), c3 = val(b + t.oy + t.ox);
  const float c4 = val(b + t.oz), c5 = val(b + t.oz + t.ox), c6 = val(b + t.oz + t.oy);
  const float c7 = val(b + t.oz + t.oy + t.ox);
  const float x00 = dob_mix(c0, c1, t.fx), x10 = dob_mix(c2, c3, t.fx);
  const float x01 = dob_mix(c4, c5, t.fx), x11 = dob_mix(c6, c7, t.fx);
  float dfx = dob_mix(dob_mix(c1 - c0, c3 - c2, t.fy), dob_mix(c5 - c4, c7 - c6, t.fy), t.fz);
  float dfy = dob_mix(x10 - x00, x11 - x01, t.fz);
  const float y0 = dob_mix(x00, x10, t.fy), y1 = dob_mix(x01, x11, t.fy);
  float dfz = y1 - y0;
  if (t.fx <= kNodeBand) {  // node at the base: slope below it from base - 1
    const uint32_t o = b - n.lx;
    const float l0 = val(o), l2 = val(o + t.oy), l4 = val(o + t.oz), l6 = val(o + t.oz + t.oy);
    dfx = 0.5f * (dfx + dob_mix(dob_mix(c0 - l0, c2 - l2, t.fy), dob_mix(c4 - l4, c6 - l6, t.fy), t.fz));
  } else if (t.fx >= 1.0f - kNodeBand) {  // node at base + 1: slope above it to base + 2
    const uint32_t o = b + t.ox + n.hx;
    const float h0 = val(o), h2 = val(o + t.oy), h4 = val(o + t.oz), h6 = val(o + t.oz + t.oy);
    dfx = 0.5f * (dfx + dob_mix(dob_mix(h0 - c1, h2 - c3, t.fy), dob_mix(h4 - c5, h6 - c7, t.fy), t.fz));
  }
  if (t.fy <= kNodeBand) {
    const uint32_t o = b - n.ly;
    const float l00 = dob_mix(val(o), val(o + t.ox), t.fx);
    const float l01 = dob_mix(val(o + t.oz), val(o + t.oz + t.ox), t.fx);
    dfy = 0.5f * (dfy + dob_mix(x00 - l00, x01 - l01, t.fz));
  } else if (t.fy >= 1.0f - kNodeBand) {
    const uint32_t o = b + t.oy + n.hy;
    const float h00 = dob_mix(val(o), val(o + t.ox), t.fx);
    const float h01 = dob_mix(val(o + t.oz), val(o + t.oz + t.ox), t.fx);
    dfy = 0.5f * (dfy + dob_mix(h00 - x10, h01 - x11, t.fz));
  }
  if (t.fz <= kNodeBand) {
    const uint32_t o = b - n.lz;
    const float m0 = dob_mix(val(o), val(o + t.ox), t.fx);
    const float m1 = dob_mix(val(o + t.oy), val(o + t.oy + t.ox), t.fx);
    dfz = 0.5f * (dfz + (y0 - dob_mix(m0, m1, t.fy)));
  } else if (t.fz >= 1.0f - kNodeBand) {
    const uint32_t o = b + t.oz + n.hz;
    const float m0 = dob_mix(val(o), val(o + t.ox), t.fx);
    const float m1 = dob_mix(val(o + t.oy), val(o + t.oy + t.ox), t.fx);
    dfz = 0.5f * (dfz + (dob_mix(m0, m1, t.fy) - y1));
  }
  return v3(dfx, dfy, dfz);
}
template <class S>
__device__ __forceinline__ dob_v3 lerp8_dfrac(const Taps& t, const NodeLo& n, const S* a) {
  return dfrac_core(t, n, [&](uint32_t k) { return ldv(a + k); });
}
// sum over the xyz channels of a float4 field: sum_ch g_ch * d lerp8_ch / d(fx, fy, fz)
// (the derivative is linear in the values, so the channels are contracted first)
__device__ __forceinline__ dob_v3 lerp8x3_dfrac(const Taps& t, const NodeLo& n, const float4* a, dob_v3 g) {
  return dfrac_core(t, n, [&](uint32_t k) {
    const float4 c = a[k];
    return g.x * c.x + g.y * c.y + g.z * c.z;
  });
}
// transpose of lerp8: a[tap k] += g * w_k
__device__ __forceinline__ void scatter8(float* a, const Taps& t, float g) {
  if (g == 0.0f) return;
  float w[8];
  tri_w(t, w);
#pragma unroll
  for (int k = 0; k < 8; ++k)
    if (w[k] != 0.0f) atomicAdd(a + tap_at(t, k), g * w[k]);
}
__device__ __forceinline__ void scatter8v(float4* a, const Taps& t, dob_v3 g) {
  if (g.x == 0.0f && g.y == 0.0f && g.z == 0.0f) return;
  float w[8];
  tri_w(t, w);
#pragma unroll
  for (int k = 0; k < 8; ++k)
    if (w[k] != 0.0f) atomicAdd(a + tap_at(t, k), make_float4(g.x * w[k], g.y * w[k], g.z * w[k], 0.0f));
}
// derivative mask of dob_clampf(v, lo, hi): 1 where the value passed through
__device__ __forceinline__ float pass(float v, float lo, float hi) { return (v > lo && v < hi) ? 1.0f : 0.0f; }
__device__ __forceinline__ dob_v3 pass3(dob_v3 v, float lo, float hi) {
  return v3(pass(v.x, lo, hi), pass(v.y, lo, hi), pass(v.z, lo, hi));
}

#define ADJ_CELL                                     \
  const int x = blockIdx.x * blockDim.x + threadIdx.x; \
  const int y = blockIdx.y * blockDim.y + threadIdx.y; \
  const int z = blockIdx.z;                          \
  if (x >= g.nx || y >= g.ny) return;                \
  const size_t i = g.at(x, y, z);

// ---- FLUID_ADVECT_MAC (closed box) ------------------------------------------------------------
// Forward per face: B = trace_back(cen, F) (RK2 with clamps), value =
// damp * lerp8(u_k, clamp(B - half-cell offset)).  Adjoint of the output
// au2 -> au (face values) and acen (centre velocity).
__device__ __forceinline__ void adj_face(const Grid& g, const float* uk, const float4* cen, float4* acen, float* auk,
                                         dob_v3 F, int comp, float gout, float dtv, const Recip3& dom,
                                         dob_v3 dims) {
  if (gout == 0.0f) return;
  // forward recompute
  const dob_v3 F0 = clamp3(F, 0.002f, 0.998f);
  const Taps t0 = make_taps_exact(g, F0.x, F0.y, F0.z);  // as trace_back forms it
  const dob_v3 v0 = lerp8x3_fixed(t0, cen);
  const dob_v3 M = F - (0.5f * (v0 * dtv)) / dom;
  const dob_v3 Mc = clamp3(M, 0.002f, 0.998f);
  const Taps tM = make_taps_in(g, Mc.x, Mc.y, Mc.z);
  const float4 vmr = lerp8xn<3>(tM, cen);
  const dob_v3 vMid = v3(vmr.x, vmr.y, vmr.z);
  const dob_v3 B = F - (vMid * dtv) / dom;
  const dob_v3 Bc = clamp3(B, 0.002f, 0.998f);
  dob_v3 S = Bc;
  if (comp == 0) S.x = S.x - 0.5f * g.rx;
  if (comp == 1) S.y = S.y - 0.5f * g.ry;
  if (comp == 2) S.z = S.z - 0.5f * g.rz;
  const dob_v3 Sc = clamp3(S, 0.001f, 0.999f);
  const Taps tS = make_taps_in(g, Sc.x, Sc.y, Sc.z);
  // backward
  scatter8(auk, tS, gout);
  const dob_v3 gS = (gout * lerp8_dfrac(tS, node_lo(g, Sc.x, Sc.y, Sc.z), uk)) * dims * pass3(S, 0.001f, 0.999f);
  const dob_v3 gB = gS * pass3(B, 0.002f, 0.998f);
  const dob_v3 gvMid = -(gB * dtv) / dom;
  scatter8v(acen, tM, gvMid);
  const dob_v3 gM = lerp8x3_dfrac(tM, node_lo(g, Mc.x, Mc.y, Mc.z), cen, gvMid) * dims * pass3(M, 0.002f, 0.998f);
  const dob_v3 gv0 = -(0.5f * (gM * dtv)) / dom;
  scatter8v(acen, t0, gv0);
}

// One thread per face (grid z = 3 nz: the face's axis is blockIdx.z % 3,
// uniform over the block), so a thread holds one face's trace; capped at 64
// registers (4 blocks per SM, a 12-byte spill): the kernel is bound by the
// latency of its gathers, and twice the resident warps of the uncapped
// three-face thread hide more of it.
__global__ void __launch_bounds__(256, 4) k_adj_advect_mac(Grid g, const StepParams* __restrict__ Pp,
                                                        const float* __restrict__ u, const float* __restrict__ v,
                                                        const float* __restrict__ w, const float4* __restrict__ cen,
                                                        const float* __restrict__ au2, const float* __restrict__ av2,
                                                        const float* __restrict__ aw2, float* au, float* av, float* aw,
                                                        float4* acen) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int comp = blockIdx.z % 3, z = blockIdx.z / 3;
  if (x >= g.nx || y >= g.ny) return;
  const size_t i = g.at(x, y, z);
  const StepParams& P = *Pp;
  const dob_v3 dims = v3((float)g.nx, (float)g.ny, (float)g.nz);
  const Recip3 dimr = grid_recip(g), dom = dom_recip(P);
  const float dtv = P.dt;
  const float damp = P.damp;
  const bool wall = comp == 0 ? x >= g.nx - 1 : comp == 1 ? y >= g.ny - 1 : z >= g.nz - 1;
  const float* ga = comp == 0 ? au2 : comp == 1 ? av2 : aw2;
  const float gout = wall ? 0.0f : ga[i] * damp;
  const dob_v3 F = v3((float)x + (comp == 0 ? 1.0f : 0.5f), (float)y + (comp == 1 ? 1.0f : 0.5f),
                      (float)z + (comp == 2 ? 1.0f : 0.5f)) / dimr;
  adj_face(g, comp == 0 ? u : comp == 1 ? v : w, cen, acen, comp == 0 ? au : comp == 1 ? av : aw, F, comp, gout, dtv,
           dom, dims);
}

// ---- FLUID_MAC_TO_CENTER (closed box): au += C^T acen ---------------------------------------
__global__ void __launch_bounds__(256) k_adj_mac_to_center(Grid g, const float4* __restrict__ acen, float* au,
                                                           float* av, float* aw) {
  ADJ_CELL
  const float4 c = acen[i];
  if (x < g.nx - 1) au[i] += 0.5f * c.x + 0.5f * acen[i + 1].x;
  if (y < g.ny - 1) av[i] += 0.5f * c.y + 0.5f * acen[i + g.nx].y;
  if (z < g.nz - 1) aw[i] += 0.5f * c.z + 0.5f * acen[i + (size_t)g.nx * g.ny].z;
}

// ---- FLUID_CASSON_FORCES (closed box) ----------------------------------------------------------
__device__ __forceinline__ dob_v3 ldm(const Grid& g, const float* u, const float* v, const float* w, int x, int y,
                                      int z) {
  const size_t j = g.at(dob_clampi(x, 0, g.nx - 1), dob_clampi(y, 0, g.ny - 1), dob_clampi(z, 0, g.nz - 1));
  return v3(u[j], v[j], w[j]);
}
__device__ __forceinline__ dob_v3 out_adj(const Grid& g, const float* au2, const float* av2, const float* aw2, int x,
                                          int y, int z) {
  const size_t j = g.at(x, y, z);
  return v3(x >= g.nx - 1 ? 0.0f : au2[j], y >= g.ny - 1 ? 0.0f : av2[j], z >= g.nz - 1 ? 0.0f : aw2[j]);
}
// Pass 1: per cell, alpha and G = 2 dL/dQ (Q = |grad u|^2 of the Casson
// shear rate); the dye adjoint of the cell.
template <class DS>
__global__ void __launch_bounds__(256, 5) k_adj_casson1(Grid g, const StepParams* __restrict__ Pp,
                                                     const float* __restrict__ u, const float* __restrict__ v,
                                                     const float* __restrict__ w, const DS* __restrict__ dye,
                                                     const float* __restrict__ au2, const float* __restrict__ av2,
                                                     const float* __restrict__ aw2, float* __restrict__ alpha_out,
                                                     float* __restrict__ gq_out, float* ac) {
  ADJ_CELL
  const StepParams& P = *Pp;
  const float dtv = P.dt;
  const dob_v3 mac = v3(u[i], v[i], w[i]);
  const dob_v3 mXp = ldm(g, u, v, w, x + 1, y, z), mXn = ldm(g, u, v, w, x - 1, y, z);
  const dob_v3 mYp = ldm(g, u, v, w, x, y + 1, z), mYn = ldm(g, u, v, w, x, y - 1, z);
  const dob_v3 mZp = ldm(g, u, v, w, x, y, z + 1), mZn = ldm(g, u, v, w, x, y, z - 1);
  const dob_v3 du = mXp - mXn, dv = mYp - mYn, dw = mZp - mZn;
  const dob_v3 lap = (mXp + mXn + mYp + mYn + mZp + mZn) - 6.0f * mac;
  const float cval = ldv(dye + i);
  const float c = dob_clampf(cval, 0.0f, 1.5f);
  const float dxv = P.dx;
  const float Q = dot3(du, du) + dot3(dv, dv) + dot3(dw, dw);
  const float gdot = dob_sqrt(Q) / (2.0f * dxv);
  const float sqrtMu = dob_sqrt(P.mu_p);
  const float S = dob_sqrt(P.tau_y * c * c / (gdot + 0.4f));
  const float nu = (sqrtMu + S) * (sqrtMu + S);
  const float araw = nu * dtv / (dxv * dxv);
  const float alpha = dob_minf(araw, 0.125f);
  alpha_out[i] = alpha;
  float G = 0.0f;
  if (araw < 0.125f) {
    const dob_v3 o = out_adj(g, au2, av2, aw2, x, y, z);
    const float ab = dot3(o, lap);
    const float nub = ab * dtv / (dxv * dxv);
    const float Sb = nub * 2.0f * (sqrtMu + S);
    const float K = dob_sqrt(P.tau_y / (gdot + 0.4f));
    ac[i] += Sb * K * pass(cval, 0.0f, 1.5f);
    const float gb = Sb * (-S / (2.0f * (gdot + 0.4f)));
    if (Q > 0.0f) G = 2.0f * (gb / (2.0f * dxv)) / (2.0f * dob_sqrt(Q));
  }
  gq_out[i] = G;
}
// Pass 2: gather the adjoint of each face value from the cells whose
// (clamped) stencils read it.
__global__ void __launch_bounds__(256) k_adj_casson2(Grid g, const float* __restrict__ u, const float* __restrict__ v,
                                                     const float* __restrict__ w, const float* __restrict__ au2,
                                                     const float* __restrict__ av2, const float* __restrict__ aw2,
                                                     const float* __restrict__ alpha, const float* __restrict__ gq,
                                                     float* au, float* av, float* aw) {
  ADJ_CELL
  const int n[3] = {g.nx, g.ny, g.nz};
  const int jc[3] = {x, y, z};
  const dob_v3 o = out_adj(g, au2, av2, aw2, x, y, z);
  const float aj = alpha[i], Gj = gq[i];
  const dob_v3 mj = v3(u[i], v[i], w[i]);
  int ncl = 0;
  dob_v3 acc = v3(0.0f, 0.0f, 0.0f);
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    int e[3] = {0, 0, 0};
    e[d] = 1;
    if (jc[d] > 0) {  // i = j - e_d: j is its + neighbour
      const int ix = x - e[0], iy = y - e[1], iz = z - e[2];
      const size_t ii = g.at(ix, iy, iz);
      const dob_v3 oi = out_adj(g, au2, av2, aw2, ix, iy, iz);
      const dob_v3 mm = ldm(g, u, v, w, x - 2 * e[0], y - 2 * e[1], z - 2 * e[2]);
      acc = acc + alpha[ii] * oi + gq[ii] * (mj - mm);
    } else {
      ++ncl;  // the - neighbour of j clamps onto j
      const dob_v3 mp = ldm(g, u, v, w, x + e[0], y + e[1], z + e[2]);
      acc = acc - Gj * (mp - mj);
    }
    if (jc[d] < n[d] - 1) {  // i = j + e_d: j is its - neighbour
      const int ix = x + e[0], iy = y + e[1], iz = z + e[2];
      const size_t ii = g.at(ix, iy, iz);
      const dob_v3 oi = out_adj(g, au2, av2, aw2, ix, iy, iz);
      const dob_v3 mp = ldm(g, u, v, w, x + 2 * e[0], y + 2 * e[1], z + 2 * e[2]);
      acc = acc + alpha[ii] * oi - gq[ii] * (mp - mj);
    } else {
      ++ncl;  // the + neighbour of j clamps onto j
      const dob_v3 mm = ldm(g, u, v, w, x - e[0], y - e[1], z - e[2]);
      acc = acc + Gj * (mj - mm);
    }
  }
  const float self = 1.0f - 6.0f * aj + aj * (float)ncl;
  acc = acc + self * o;
  au[i] += acc.x;
  av[i] += acc.y;
  aw[i] += acc.z;
}

// ---- FLUID_MAC_RHS (closed box): au += D^T arhs (arhs already mean-free) -----------------------
__global__ void __launch_bounds__(256) k_adj_mac_rhs(Grid g, const float* __restrict__ arhs, float* au, float* av,
                                                     float* aw) {
  ADJ_CELL
  const float bj = arhs[rb_index(g, x, y, z)];
  if (x < g.nx - 1) au[i] += bj - arhs[rb_index(g, x + 1, y, z)];
  if (y < g.ny - 1) av[i] += bj - arhs[rb_index(g, x, y + 1, z)];
  if (z < g.nz - 1) aw[i] += bj - arhs[rb_index(g, x, y, z + 1)];
}

// ---- FLUID_MAC_PROJECT (closed box): au <- W au, ap += D(W au) --------------------------------
__global__ void __launch_bounds__(256) k_adj_project(Grid g, float* au, float* av, float* aw, float* ap) {
  ADJ_CELL
  const float ox = x < g.nx - 1 ? au[i] : 0.0f;
  const float oy = y < g.ny - 1 ? av[i] : 0.0f;
  const float oz = z < g.nz - 1 ? aw[i] : 0.0f;
  const float oxm = x > 0 ? au[i - 1] : 0.0f;
  const float oym = y > 0 ? av[i - g.nx] : 0.0f;
  const float ozm = z > 0 ? aw[i - (size_t)g.nx * g.ny] : 0.0f;
  ap[rb_index(g, x, y, z)] += (ox - oxm) + (oy - oym) + (oz - ozm);
  // wall faces are zeroed by the forward; no neighbour reads them
  if (x == g.nx - 1) au[i] = 0.0f;
  if (y == g.ny - 1) av[i] = 0.0f;
  if (z == g.nz - 1) aw[i] = 0.0f;
}

// ---- multigrid transposes (red-black split arrays) ---------------------------------------------
__device__ __forceinline__ float mg_diag(const Grid& d, int ref, int x, int y, int z) {
  float s = ref ? 1.0f : 0.0f;
  s += (x > 0 ? 1.0f : 0.0f) + (x < d.nx - 1 ? 1.0f : 0.0f) + (y > 0 ? 1.0f : 0.0f);
  s += (!ref && y < d.ny - 1) ? 1.0f : 0.0f;
  s += (z > 0 ? 1.0f : 0.0f) + (z < d.nz - 1 ? 1.0f : 0.0f);
  return s;
}
// sum over the existing neighbours n of (x,y,z) of xb(n) / diag(n)
__device__ __forceinline__ float nbr_scaled_sum(const float* xb, const Grid& d, int ref, int x, int y, int z) {
  float s = 0.0f;
  if (x > 0) s += xb[rb_index(d, x - 1, y, z)] / mg_diag(d, ref, x - 1, y, z);
  if (x < d.nx - 1) s += xb[rb_index(d, x + 1, y, z)] / mg_diag(d, ref, x + 1, y, z);
  if (y > 0) s += xb[rb_index(d, x, y - 1, z)] / mg_diag(d, ref, x, y - 1, z);
  if (y < d.ny - 1) s += xb[rb_index(d, x, y + 1, z)] / mg_diag(d, ref, x, y + 1, z);
  if (z > 0) s += xb[rb_index(d, x, y, z - 1)] / mg_diag(d, ref, x, y, z - 1);
  if (z < d.nz - 1) s += xb[rb_index(d, x, y, z + 1)] / mg_diag(d, ref, x, y, z + 1);
  return s;
}
enum { ADJ_SWEEP_FIRST = 0, ADJ_SWEEP_FUSED = 1, ADJ_SWEEP_FINAL = 2 };
// One step of a transposed run of red-black half-sweeps, over the cells of
// colour `color`:
//   FIRST  xb += sum_n xb(n)/diag(n)               (first half of the last
//                                                    half-sweep's transpose)
//   FUSED  bb += -h2 xb/diag; xb = sum_n xb(n)/diag(n)
//   FINAL  bb += -h2 xb/diag; xb = 0
__global__ void __launch_bounds__(256) k_adj_rbgs(Grid d, int color, float h2, int ref, int mode, float* xb, float* bb) {
  pdl_wait();
  pdl_trigger();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (k >= (d.nx >> 1) || y >= d.ny) return;
  const int x = 2 * k + ((y + z + color) & 1);
  const size_t j = rb_index(d, x, y, z);
  if (mode == ADJ_SWEEP_FIRST) {
    xb[j] += nbr_scaled_sum(xb, d, ref, x, y, z);
    return;
  }
  const float diag = mg_diag(d, ref, x, y, z);
  bb[j] += -h2 * xb[j] / diag;
  xb[j] = mode == ADJ_SWEEP_FUSED ? nbr_scaled_sum(xb, d, ref, x, y, z) : 0.0f;
}
// Vectorised form of the transposed half-sweeps for rows with nx % 8 == 0,
// same thread layout as the forward k_rbgs_v4 (four cells of one colour
// per thread, rows packed into warps, branch-free boundaries).  Within a
// transposed run the adjoint is kept scaled by the diagonal, y = xb / diag,
// so most steps need only their own cell's diagonal:
//   FIRST    y = (xb + sum_n xb(n) / diag(n)) / diag   (the other colour is
//            still unscaled: each neighbour is divided by its own diagonal)
//   FUSED    bb += -h2 y;  y = sum_n y(n) / diag
//            (OWN_RAW: the own colour is still unscaled, y = xb / diag first;
//             OUT_RAW: the last step of the run writes xb = sum_n y(n), the
//             unscaled value, since only the own colour is read after it)
//   FINAL    bb += -h2 y;  y = 0
// so the run needs no separate scaling passes.
enum { ADJ4_FIRST = 1, ADJ4_FUSED = 2, ADJ4_FINAL = 3, ADJ4_OWN_RAW = 8, ADJ4_OUT_RAW = 16 };
__device__ __forceinline__ float4 ld4f(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ float f4at(const float4& v, int j) {
  return j == 0 ? v.x : (j == 1 ? v.y : (j == 2 ? v.z : v.w));
}
// 1 / k for a diagonal k in 1..6 (the correctly rounded reciprocals)
__device__ __forceinline__ float rcp_diag(float k) {
  return k == 6.0f ? 1.0f / 6.0f
                   : (k == 5.0f ? 0.2f : (k == 4.0f ? 0.25f : (k == 3.0f ? 1.0f / 3.0f : (k == 2.0f ? 0.5f : 1.0f))));
}
__global__ void __launch_bounds__(256, 5) k_adj_rbgs_v4(Grid d, int color, float h2, int ref, int mode, float* __restrict__ a,
                                                     float* __restrict__ bb) {
  pdl_wait();
  pdl_trigger();
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  const uint32_t hx = (uint32_t)d.nx >> 1;
  const uint32_t k0 = 4u * (uint32_t)q;
  if (k0 >= hx || y >= d.ny) return;
  const int base = mode & 7;
  const int p = (y + z + color) & 1;
  const uint32_t half = (uint32_t)(d.n() >> 1);
  const uint32_t sz = (uint32_t)d.ny * hx;
  const uint32_t r = (uint32_t)z * sz + (uint32_t)y * hx;
  float* own = a + (color ? half : 0u) + r + k0;
  const float* oth = a + (color ? 0u : half);
  const bool has_ym = y > 0, has_yp = y < d.ny - 1, has_zm = z > 0, has_zp = z < d.nz - 1;
  const bool has_ex = p == 0 ? k0 > 0 : k0 + 4 < hx;
  const float wex = has_ex ? 1.0f : 0.0f;
  const float wym = has_ym ? 1.0f : 0.0f, wyp = has_yp ? 1.0f : 0.0f;
  const float wzm = has_zm ? 1.0f : 0.0f, wzp = has_zp ? 1.0f : 0.0f;
  const float dyz = (wym + wzm + wzp) + (ref ? 1.0f : wyp);
  float diag[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const float wxm = (p == 0 && j == 0) ? wex : 1.0f;
    const float wxp = (p == 1 && j == 3) ? wex : 1.0f;
    diag[j] = dyz + (wxm + wxp);
  }
  const float4 ov = ld4f(own);
  float res[4];
  float yo[4];  // the own colour, scaled
#pragma unroll
  for (int j = 0; j < 4; ++j) yo[j] = (mode & ADJ4_OWN_RAW) ? f4at(ov, j) / diag[j] : f4at(ov, j);
  if (base == ADJ4_FINAL) {
    float* bp = bb + (color ? half : 0u) + r + k0;
    const float4 bv = ld4f(bp);
    *reinterpret_cast<float4*>(bp) =
        make_float4(bv.x - h2 * yo[0], bv.y - h2 * yo[1], bv.z - h2 * yo[2], bv.w - h2 * yo[3]);
#pragma unroll
    for (int j = 0; j < 4; ++j) res[j] = 0.0f;
  } else {
    const uint32_t rym = has_ym ? r - hx : r, ryp = has_yp ? r + hx : r;
    const uint32_t rzm = has_zm ? r - sz : r, rzp = has_zp ? r + sz : r;
    float4 cm = ld4f(oth + r + k0);
    float4 ym = ld4f(oth + rym + k0), yp = ld4f(oth + ryp + k0);
    float4 zm = ld4f(oth + rzm + k0), zp = ld4f(oth + rzp + k0);
    const uint32_t kex = p == 0 ? (has_ex ? k0 - 1 : k0) : (has_ex ? k0 + 4 : k0 + 3);
    float ex = oth[r + kex];
    if (base == ADJ4_FIRST) {
      // the other colour is unscaled: divide every neighbour by its diagonal
      // (cells of the other colour at x = 2 (k0 + j) + 1 - p, y +- 1, z +- 1)
      const float fy = (y > 0 ? 1.0f : 0.0f) + (ref ? 1.0f : wyp), fz = wzm + wzp;
      const float fym = (y - 1 > 0 ? 1.0f : 0.0f) + (ref ? 1.0f : (y - 1 < d.ny - 1 ? 1.0f : 0.0f));
      const float fyp = (y + 1 > 0 ? 1.0f : 0.0f) + (ref ? 1.0f : (y + 1 < d.ny - 1 ? 1.0f : 0.0f));
      const float fzm = (z - 1 > 0 ? 1.0f : 0.0f) + (z - 1 < d.nz - 1 ? 1.0f : 0.0f);
      const float fzp = (z + 1 > 0 ? 1.0f : 0.0f) + (z + 1 < d.nz - 1 ? 1.0f : 0.0f);
      auto fx = [&](int xx) { return (xx > 0 ? 1.0f : 0.0f) + (xx < d.nx - 1 ? 1.0f : 0.0f); };
      float c[4], vym[4], vyp[4], vzm[4], vzp[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int xo = 2 * ((int)k0 + j) + p;  // own cell j
        const int xn = 2 * ((int)k0 + j) + 1 - p;  // the other colour's cell of word k0 + j
        c[j] = f4at(cm, j) * rcp_diag(fx(xn) + fy + fz);
        vym[j] = f4at(ym, j) * rcp_diag(fx(xo) + fym + fz);
        vyp[j] = f4at(yp, j) * rcp_diag(fx(xo) + fyp + fz);
        vzm[j] = f4at(zm, j) * rcp_diag(fx(xo) + fy + fzm);
        vzp[j] = f4at(zp, j) * rcp_diag(fx(xo) + fy + fzp);
      }
      cm = make_float4(c[0], c[1], c[2], c[3]);
      ym = make_float4(vym[0], vym[1], vym[2], vym[3]);
      yp = make_float4(vyp[0], vyp[1], vyp[2], vyp[3]);
      zm = make_float4(vzm[0], vzm[1], vzm[2], vzm[3]);
      zp = make_float4(vzp[0], vzp[1], vzp[2], vzp[3]);
      const int xe = 2 * (int)kex + 1 - p;  // the other colour's cell of word kex
      ex = ex * rcp_diag(fx(xe) + fy + fz);
    }
    if (base == ADJ4_FUSED) {
      float* bp = bb + (color ? half : 0u) + r + k0;
      const float4 bv = ld4f(bp);
      *reinterpret_cast<float4*>(bp) =
          make_float4(bv.x - h2 * yo[0], bv.y - h2 * yo[1], bv.z - h2 * yo[2], bv.w - h2 * yo[3]);
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float xm = p == 0 ? (j == 0 ? ex : f4at(cm, j - 1)) : f4at(cm, j);
      const float xp = p == 0 ? f4at(cm, j) : (j == 3 ? ex : f4at(cm, j + 1));
      const float wxm = (p == 0 && j == 0) ? wex : 1.0f;
      const float wxp = (p == 1 && j == 3) ? wex : 1.0f;
      float sumN = base == ADJ4_FIRST ? f4at(ov, j) : 0.0f;
      sumN = fmaf(wxm, xm, sumN);
      sumN = fmaf(wxp, xp, sumN);
      sumN = fmaf(wym, f4at(ym, j), sumN);
      sumN = fmaf(wyp, f4at(yp, j), sumN);
      sumN = fmaf(wzm, f4at(zm, j), sumN);
      sumN = fmaf(wzp, f4at(zp, j), sumN);
      res[j] = (mode & ADJ4_OUT_RAW) ? sumN : sumN / diag[j];
    }
  }
  *reinterpret_cast<float4*>(own) = make_float4(res[0], res[1], res[2], res[3]);
}

// Transposed coarse solve (zero start + `sweeps` red-black sweeps) inside
// one thread-block cluster, the mirror of k_coarse_cluster: CTA r keeps the
// scaled adjoint y and the right-hand-side adjoint of its z-slab in shared
// memory and reads the neighbouring slabs' boundary planes through
// distributed shared memory; one cluster barrier per transposed half-sweep.
// On exit Ebar = 0 (the forward's zero start) and Bbar += its adjoint.
template <int CS>
__global__ void __cluster_dims__(CS, 1, 1) __launch_bounds__(512)
    k_adj_coarse_cluster(Grid d, float h2, int ref, int sweeps, float* __restrict__ eb, float* __restrict__ bb) {
  pdl_wait();
  pdl_trigger();
  cg::cluster_group cl = cg::this_cluster();
  extern __shared__ float asm_[];
  const int rank = (int)cl.block_rank();
  const int pz = d.nz / CS;
  const int plane = d.nx * d.ny;
  const int nloc = pz * plane;
  float* sy = asm_;
  float* sb = asm_ + nloc;
  const int z0 = rank * pz;
  const int K = 2 * sweeps;
  auto color_of = [](int k) { return (k - 1) & 1; };
  auto diag_at = [&](int x, int y, int z) {
    float s = ref ? 1.0f : 0.0f;
    s += (x > 0 ? 1.0f : 0.0f) + (x < d.nx - 1 ? 1.0f : 0.0f) + (y > 0 ? 1.0f : 0.0f);
    s += (!ref && y < d.ny - 1) ? 1.0f : 0.0f;
    s += (z > 0 ? 1.0f : 0.0f) + (z < d.nz - 1 ? 1.0f : 0.0f);
    return s;
  };
  // load: y = Ebar / diag on the colour of the last half-sweep, Ebar elsewhere
  for (int k = threadIdx.x; k < nloc; k += blockDim.x) {
    const int zl = k / plane, rem = k - zl * plane;
    const int y = rem / d.nx, x = rem - y * d.nx;
    const int z = z0 + zl;
    const float v = K > 0 ? eb[rb_index(d, x, y, z)] : 0.0f;
    sy[k] = (K > 0 && ((x + y + z) & 1) == color_of(K)) ? v / diag_at(x, y, z) : v;
    sb[k] = 0.0f;
  }
  const float* below = rank > 0 ? cl.map_shared_rank(sy, rank - 1) + (pz - 1) * plane : nullptr;
  const float* above = rank < CS - 1 ? cl.map_shared_rank(sy, rank + 1) : nullptr;
  cl.sync();
  const int hxc = d.nx >> 1;
  // phases: FIRST over the other colour, FUSED for k = K..2, FINAL for k = 1
  for (int ph = 0; ph <= K && K > 0; ++ph) {
    const int mode = ph == 0 ? 0 : (ph < K ? 1 : 2);  // 0 FIRST, 1 FUSED, 2 FINAL
    const int color = ph == 0 ? 1 - color_of(K) : color_of(K + 1 - ph);
    for (int q = threadIdx.x; q < (nloc >> 1); q += blockDim.x) {
      const int row = q / hxc, kx = q - row * hxc;
      const int zl = row / d.ny, y = row - zl * d.ny;
      const int z = z0 + zl;
      const int x = 2 * kx + ((y + z + color) & 1);
      const int rem = y * d.nx + x;
      const int k = zl * plane + rem;
      const float dg = diag_at(x, y, z);
      const float own = sy[k];
      if (mode != 0) sb[k] += -h2 * own;
      if (mode == 2) { sy[k] = 0.0f; continue; }
      float sumN = mode == 0 ? own : 0.0f;
      if (x > 0) sumN += sy[k - 1];
      if (x < d.nx - 1) sumN += sy[k + 1];
      if (y > 0) sumN += sy[k - d.nx];
      if (y < d.ny - 1) sumN += sy[k + d.nx];
      if (z > 0) sumN += zl > 0 ? sy[k - plane] : below[rem];
      if (z < d.nz - 1) sumN += zl < pz - 1 ? sy[k + plane] : above[rem];
      sy[k] = sumN / dg;
    }
    cl.sync();
  }
  for (int k = threadIdx.x; k < nloc; k += blockDim.x) {
    const int zl = k / plane, rem = k - zl * plane;
    const int y = rem / d.nx, x = rem - y * d.nx;
    const size_t j = rb_index(d, x, y, z0 + zl);
    bb[j] += sb[k];
    eb[j] = 0.0f;
  }
  cl.sync();  // keep this CTA's shared memory alive until its neighbours are done reading it
}

// weight of coarse index J in the cell-centred linear interpolation at fine
// index xf (the forward's clamped taps; 0 above a Dirichlet top when `top0`)
__device__ __forceinline__ float prolong_w(int xf, int nf, int nc, int J, bool top0) {
  const float cx = __fmaf_rn(((float)xf + 0.5f) / (float)nf, (float)nc, -0.5f);  // as k_prolong_add2 forms it
  const float bx = floorf(cx);
  const float fx = cx - bx;
  const int i0 = (int)bx, i1 = i0 + 1;
  float wsum = 0.0f;
  if (dob_clampi(i0, 0, nc - 1) == J && !(top0 && i0 >= nc)) wsum += 1.0f - fx;
  if (dob_clampi(i1, 0, nc - 1) == J && !(top0 && i1 >= nc)) wsum += fx;
  return wsum;
}
// ---- two coarse cells per thread (fine rows with nx % 4 == 0) ------------------------------
// Thread q owns coarse cells X = 2q, 2q+1 of coarse row (Y, Z); in the split
// layout the even fine cells x = 4q, 4q+2 of a fine row are words 2q, 2q+1 of
// one half and the odd cells the same words of the other half (8-byte pairs).
__device__ __forceinline__ float2 ld2f(const float* p) { return *reinterpret_cast<const float2*>(p); }
__device__ __forceinline__ void st2f(float* p, float2 v) { *reinterpret_cast<float2*>(p) = v; }
// coarse split value at (X, Y, Z) (in range)
__device__ __forceinline__ float cval(const float* a, const Grid& c, uint32_t halfc, int X, int Y, int Z) {
  const uint32_t hc = (uint32_t)c.nx >> 1;
  return a[(((X + Y + Z) & 1) ? halfc : 0u) + ((uint32_t)Z * c.ny + Y) * hc + (uint32_t)(X >> 1)];
}
// Transposed residual + restriction, the mirror of k_residual_restrict2.
__global__ void __launch_bounds__(256) k_adj_restrict2(Grid f, Grid c, float inv_h2, int ref, const float* __restrict__ Bb,
                                                       float* __restrict__ xb, float* __restrict__ bb) {
  pdl_wait();
  pdl_trigger();
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int Y = blockIdx.y * blockDim.y + threadIdx.y;
  const int Z = blockIdx.z;
  if (2 * q >= c.nx || Y >= c.ny) return;
  const uint32_t halfc = (uint32_t)(c.n() >> 1);
  const bool has_xm = q > 0, has_xp = 2 * q + 2 < c.nx;
  const int y0 = 2 * Y, z0 = 2 * Z;
  const bool has_ym = y0 > 0, has_yp = y0 + 2 < f.ny, has_zm = z0 > 0, has_zp = z0 + 2 < f.nz;
  // 0.125 * Bbar at the parents: the block row X' = 2q-1..2q+2 and the
  // neighbouring coarse rows X' = 2q, 2q+1 (clamped reads when absent)
  float cr[4], cym[2], cyp[2], czm[2], czp[2];
#pragma unroll
  for (int a = 0; a < 4; ++a) cr[a] = 0.125f * cval(Bb, c, halfc, dob_clampi(2 * q - 1 + a, 0, c.nx - 1), Y, Z);
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    cym[a] = 0.125f * cval(Bb, c, halfc, 2 * q + a, has_ym ? Y - 1 : Y, Z);
    cyp[a] = 0.125f * cval(Bb, c, halfc, 2 * q + a, has_yp ? Y + 1 : Y, Z);
    czm[a] = 0.125f * cval(Bb, c, halfc, 2 * q + a, Y, has_zm ? Z - 1 : Z);
    czp[a] = 0.125f * cval(Bb, c, halfc, 2 * q + a, Y, has_zp ? Z + 1 : Z);
  }
  const float wxm0 = has_xm ? 1.0f : 0.0f, wxp3 = has_xp ? 1.0f : 0.0f;
  const uint32_t hx = (uint32_t)f.nx >> 1, half = (uint32_t)(f.n() >> 1), sz = (uint32_t)f.ny * hx;
  const uint32_t w = 2u * (uint32_t)q;
#pragma unroll
  for (int dz = 0; dz < 2; ++dz)
#pragma unroll
    for (int dy = 0; dy < 2; ++dy) {
      const float wym = (dy == 1 || has_ym) ? 1.0f : 0.0f;
      const float wyp = (dy == 0 || has_yp) ? 1.0f : 0.0f;
      const float wzm = (dz == 1 || has_zm) ? 1.0f : 0.0f;
      const float wzp = (dz == 0 || has_zp) ? 1.0f : 0.0f;
      const float dyz = (wym + wzm + wzp) + (ref ? 1.0f : wyp);
      float dx_[4], db_[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int pi = i >> 1;  // parent among 2q, 2q+1
        const float r0 = cr[1 + pi];
        const float rxm = i > 0 ? cr[1 + ((i - 1) >> 1)] : cr[0];
        const float rxp = i < 3 ? cr[1 + ((i + 1) >> 1)] : cr[3];
        const float rym = dy ? r0 : cym[pi];
        const float ryp = dy ? cyp[pi] : r0;
        const float rzm = dz ? r0 : czm[pi];
        const float rzp = dz ? czp[pi] : r0;
        const float wxm = i == 0 ? wxm0 : 1.0f;
        const float wxp = i == 3 ? wxp3 : 1.0f;
        float sumN = wxm * rxm;
        sumN = fmaf(wxp, rxp, sumN);
        sumN = fmaf(wym, rym, sumN);
        sumN = fmaf(wyp, ryp, sumN);
        sumN = fmaf(wzm, rzm, sumN);
        sumN = fmaf(wzp, rzp, sumN);
        const float diag = dyz + (wxm + wxp);
        dx_[i] = (sumN - diag * r0) * inv_h2;
        db_[i] = r0;
      }
      const int y = y0 + dy, z = z0 + dz, par = (y + z) & 1;
      const uint32_t r = (uint32_t)z * sz + (uint32_t)y * hx + w;
      float* xe = xb + (par ? half : 0u) + r;
      float* xo = xb + (par ? 0u : half) + r;
      float* be = bb + (par ? half : 0u) + r;
      float* bo = bb + (par ? 0u : half) + r;
      const float2 vxe = ld2f(xe), vxo = ld2f(xo), vbe = ld2f(be), vbo = ld2f(bo);
      st2f(xe, make_float2(vxe.x - dx_[0], vxe.y - dx_[2]));
      st2f(xo, make_float2(vxo.x - dx_[1], vxo.y - dx_[3]));
      st2f(be, make_float2(vbe.x + db_[0], vbe.y + db_[2]));
      st2f(bo, make_float2(vbo.x + db_[1], vbo.y + db_[3]));
    }
}
// Transposed prolongation, the mirror of k_prolong_add2: Ebar(X) += sum of
// the interpolation weight on X times xb over the fine cells 2X-1..2X+2 of
// each axis.
// BLACK: the fine level's red cotangents are exactly zero (the transposed
// sweeps that follow a black-only prolongation end with the red cells of
// their input cleared): only the black cells of each fine row are read, the
// red terms enter as the same zeros.
template <bool BLACK>
__global__ void __launch_bounds__(256) k_adj_prolong2(Grid f, Grid c, int ref, const float* __restrict__ xb,
                                                      float* __restrict__ Eb) {
  pdl_wait();
  pdl_trigger();
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int Y = blockIdx.y * blockDim.y + threadIdx.y;
  const int Z = blockIdx.z;
  if (2 * q >= c.nx || Y >= c.ny) return;
  float wx0[4], wx1[4], wy[4], wz[4];
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int x0 = 4 * q - 1 + a, x1 = 4 * q + 1 + a;
    wx0[a] = (x0 >= 0 && x0 < f.nx) ? prolong_w(x0, f.nx, c.nx, 2 * q, false) : 0.0f;
    wx1[a] = (x1 >= 0 && x1 < f.nx) ? prolong_w(x1, f.nx, c.nx, 2 * q + 1, false) : 0.0f;
    const int yf = 2 * Y - 1 + a, zf = 2 * Z - 1 + a;
    wy[a] = (yf >= 0 && yf < f.ny) ? prolong_w(yf, f.ny, c.ny, Y, ref != 0) : 0.0f;
    wz[a] = (zf >= 0 && zf < f.nz) ? prolong_w(zf, f.nz, c.nz, Z, false) : 0.0f;
  }
  const uint32_t hx = (uint32_t)f.nx >> 1, half = (uint32_t)(f.n() >> 1), sz = (uint32_t)f.ny * hx;
  const uint32_t w = 2u * (uint32_t)q;
  const bool has_lo = q > 0, has_hi = 4 * q + 4 < f.nx;
  float acc0 = 0.0f, acc1 = 0.0f;
#pragma unroll
  for (int cz = 0; cz < 4; ++cz) {
    if (wz[cz] == 0.0f) continue;
#pragma unroll
    for (int by = 0; by < 4; ++by) {
      if (wy[by] == 0.0f) continue;
      const int yf = 2 * Y - 1 + by, zf = 2 * Z - 1 + cz, par = (yf + zf) & 1;
      const uint32_t r = (uint32_t)zf * sz + (uint32_t)yf * hx + w;
      const float* pe = xb + (par ? half : 0u) + r;  // even cells 4q, 4q+2 (words 2q, 2q+1)
      const float* po = xb + (par ? 0u : half) + r;  // odd cells 4q+1, 4q+3
      const float2 z2 = make_float2(0.0f, 0.0f);
      // the even cells are black in rows of odd parity, the odd cells in the others
      const float2 e = (!BLACK || par) ? ld2f(pe) : z2, o = (!BLACK || !par) ? ld2f(po) : z2;
      const float lo = (has_lo && (!BLACK || !par)) ? po[-1] : 0.0f;  // x = 4q-1 (odd, word 2q-1)
      const float hi = (has_hi && (!BLACK || par)) ? pe[2] : 0.0f;    // x = 4q+4 (even, word 2q+2)
      const float v[6] = {lo, e.x, o.x, e.y, o.y, hi};
      const float s0 = wx0[0] * v[0] + wx0[1] * v[1] + wx0[2] * v[2] + wx0[3] * v[3];
      const float s1 = wx1[0] * v[2] + wx1[1] * v[3] + wx1[2] * v[4] + wx1[3] * v[5];
      const float wyz = wy[by] * wz[cz];
      acc0 = fmaf(wyz, s0, acc0);
      acc1 = fmaf(wyz, s1, acc1);
    }
  }
  const uint32_t hc = (uint32_t)c.nx >> 1, halfc = (uint32_t)(c.n() >> 1);
  const uint32_t rc = ((uint32_t)Z * c.ny + Y) * hc + (uint32_t)q;
  const int pc = (Y + Z) & 1;
  Eb[(pc ? halfc : 0u) + rc] += acc0;
  Eb[(pc ? 0u : halfc) + rc] += acc1;
}

// ---- CONC_PREDICT (closed box) ------------------------------------------------------------------
// The per-cell adjoints below (dye predictor and resolve, the Casson
// coefficients) and the transposed smoother are capped at 4-5 blocks of 256
// per SM (a few spilled bytes): latency-bound, they gain more from the
// resident warps (192x256x192 backward 4.81 -> 4.67 ms per step).
template <class DS>
__global__ void __launch_bounds__(256, 4) k_adj_conc_predict(Grid gc, Grid g, const StepParams* __restrict__ Pp,
                                                          const float4* __restrict__ cen, const DS* __restrict__ dye,
                                                          const float* __restrict__ apred, float* ac, float4* acen) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= gc.nx || y >= gc.ny) return;
  const size_t i = gc.at(x, y, z);
  const float gout = apred[i];
  if (gout == 0.0f) return;
  const StepParams& P = *Pp;
  const dob_v3 dimsc = v3((float)gc.nx, (float)gc.ny, (float)gc.nz);
  const dob_v3 dimsg = v3((float)g.nx, (float)g.ny, (float)g.nz);
  const float dtv = P.dt;
  const Recip3 dom = dom_recip(P);
  const dob_v3 uvw = (v3((float)x, (float)y, (float)z) + v3(0.5f, 0.5f, 0.5f)) / grid_recip(gc);
  const Taps t0 = make_taps_exact(g, uvw.x, uvw.y, uvw.z);  // the forward's cell-centre sample (dye on the velocity grid)
  const dob_v3 v0 = lerp8x3_fixed(t0, cen);
  const dob_v3 M = uvw - (0.5f * (v0 * dtv)) / dom;
  const dob_v3 Mc = clamp3(M, 0.001f, 0.999f);
  const Taps tM = make_taps_in(g, Mc.x, Mc.y, Mc.z);
  const float4 vmr = lerp8xn<3>(tM, cen);
  const dob_v3 vMid = v3(vmr.x, vmr.y, vmr.z);
  const dob_v3 B = uvw - (vMid * dtv) / dom;
  const dob_v3 Bc = clamp3(B, 0.001f, 0.999f);
  const Taps tB = make_taps_in(gc, Bc.x, Bc.y, Bc.z);
  scatter8(ac, tB, gout);
  const dob_v3 gB = (gout * lerp8_dfrac(tB, node_lo(gc, Bc.x, Bc.y, Bc.z), dye)) * dimsc * pass3(B, 0.001f, 0.999f);
  const dob_v3 gvMid = -(gB * dtv) / dom;
  scatter8v(acen, tM, gvMid);
  const dob_v3 gM = lerp8x3_dfrac(tM, node_lo(g, Mc.x, Mc.y, Mc.z), cen, gvMid) * dimsg * pass3(M, 0.001f, 0.999f);
  const dob_v3 gv0 = -(0.5f * (gM * dtv)) / dom;
  scatter8v(acen, t0, gv0);
}

// ---- CONC_RESOLVE (closed box: MacCormack with the 8-tap limiter) -----------------------------
template <class DS>
__global__ void __launch_bounds__(256, 5) k_adj_dye_resolve(Grid gc, Grid g, const StepParams* __restrict__ Pp,
                                                         const float4* __restrict__ cen, const DS* __restrict__ dye,
                                                         const DS* __restrict__ pred, const float* __restrict__ ac2,
                                                         float* ac, float* apred, float4* acen) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= gc.nx || y >= gc.ny) return;
  const size_t i = gc.at(x, y, z);
  const float gout = ac2[i];
  if (gout == 0.0f) return;
  const StepParams& P = *Pp;
  const dob_v3 dims = v3((float)gc.nx, (float)gc.ny, (float)gc.nz);
  const float dtv = P.dt;
  const Recip3 dom = dom_recip(P);
  const dob_v3 uvw = (v3((float)x, (float)y, (float)z) + v3(0.5f, 0.5f, 0.5f)) / grid_recip(gc);
  const Taps t0 = make_taps_exact(g, uvw.x, uvw.y, uvw.z);  // the forward's cell-centre sample (dye on the velocity grid)
  const dob_v3 v0 = lerp8x3_fixed(t0, cen);
  const dob_v3 uvwMid = clamp3(uvw - (0.5f * (v0 * dtv)) / dom, 0.001f, 0.999f);
  const float4 vmr = lerp8xn<3>(make_taps_in(g, uvwMid.x, uvwMid.y, uvwMid.z), cen);
  const dob_v3 vMid = v3(vmr.x, vmr.y, vmr.z);
  const dob_v3 uvwBack = clamp3(uvw - (vMid * dtv) / dom, 0.001f, 0.999f);
  const dob_v3 Fw = uvw + (v0 * dtv) / dom;
  const dob_v3 uvwFwd = clamp3(Fw, 0.001f, 0.999f);
  const Taps tF = make_taps_in(gc, uvwFwd.x, uvwFwd.y, uvwFwd.z);
  const float gBackEst = lerp8(tF, pred);
  const float kap = 0.45f * P.sharp;
  const float gCorr = __fmaf_rn(kap, ldv(dye + i) - gBackEst, ldv(pred + i));  // as the forward rounds it
  // the limiter's taps: the forward predictor's (make_taps at the departure point)
  const int bx = (int)floorf(texel(uvwBack.x, gc.nx)), by = (int)floorf(texel(uvwBack.y, gc.ny));
  const int bz = (int)floorf(texel(uvwBack.z, gc.nz));
  size_t id[8];
  float s[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    id[k] = gc.at(dob_clampi(bx + (k & 1), 0, gc.nx - 1), dob_clampi(by + ((k >> 1) & 1), 0, gc.ny - 1),
                  dob_clampi(bz + ((k >> 2) & 1), 0, gc.nz - 1));
    s[k] = ldv(dye + id[k]);
  }
  // the forward's min/max trees (dob_minf/dob_maxf keep the second operand on ties)
  auto pick_min = [&](int a, int b) { return s[a] < s[b] ? a : b; };
  auto pick_max = [&](int a, int b) { return s[a] > s[b] ? a : b; };
  const int kmin = pick_min(pick_min(pick_min(0, 1), pick_min(2, 3)), pick_min(pick_min(4, 5), pick_min(6, 7)));
  const int kmax = pick_max(pick_max(pick_max(0, 1), pick_max(2, 3)), pick_max(pick_max(4, 5), pick_max(6, 7)));
  const float minG = s[kmin], maxG = s[kmax];
  if (!(gCorr > minG)) {
    atomicAdd(ac + id[kmin], gout);
  } else if (!(gCorr < maxG)) {
    atomicAdd(ac + id[kmax], gout);
  } else {
    atomicAdd(apred + i, gout);
    atomicAdd(ac + i, kap * gout);
    const float gE = -kap * gout;
    scatter8(apred, tF, gE);
    const dob_v3 gF = (gE * lerp8_dfrac(tF, node_lo(gc, uvwFwd.x, uvwFwd.y, uvwFwd.z), pred)) * dims *
                      pass3(Fw, 0.001f, 0.999f);
    const dob_v3 gv0 = (gF * dtv) / dom;
    scatter8v(acen, t0, gv0);
  }
}

// ---- launchers ----------------------------------------------------------------------------------
static inline dim3 cgrid(const Grid& g) { return dim3((g.nx + 31) / 32, (g.ny + 7) / 8, g.nz); }
static inline dim3 cblock() { return dim3(32, 8, 1); }
static inline dim3 hgrid(const Grid& g) { return dim3((g.nx / 2 + 31) / 32, (g.ny + 7) / 8, g.nz); }

void launch_adj_advect_mac(const DevState& s, const AdjState& a, cudaStream_t st) {
  const dim3 g3(cgrid(s.g).x, cgrid(s.g).y, 3 * s.g.nz);
  k_adj_advect_mac<<<g3, cblock(), 0, st>>>(s.g, s.params, (const float*)s.u, (const float*)s.v,
                                                    (const float*)s.w, (const float4*)s.cen, a.au2, a.av2, a.aw2, a.au,
                                                    a.av, a.aw, a.acen);
}
void launch_adj_mac_to_center(const DevState& s, const AdjState& a, cudaStream_t st) {
  k_adj_mac_to_center<<<cgrid(s.g), cblock(), 0, st>>>(s.g, a.acen, a.au, a.av, a.aw);
}
// The dye and the predictor are read at their storage width: binary16 in
// the mixed mode (the adjoint of the rounding store is the identity, so the
// adjoint arrays stay FP32).
#define ADJ_DYE_DISPATCH(prec, ...)                                \
  do {                                                             \
    if ((prec) == DOB_PREC_MIXED) { using DS = __half; __VA_ARGS__; } \
    else { using DS = float; __VA_ARGS__; }                        \
  } while (0)

void launch_adj_casson(const DevState& s, const AdjState& a, cudaStream_t st) {
  ADJ_DYE_DISPATCH(s.prec, {
    k_adj_casson1<DS><<<cgrid(s.g), cblock(), 0, st>>>(s.g, s.params, (const float*)s.u, (const float*)s.v,
                                                       (const float*)s.w, (const DS*)s.conc, a.au2, a.av2, a.aw2,
                                                       a.alpha, a.gq, a.ac);
  });
  k_adj_casson2<<<cgrid(s.g), cblock(), 0, st>>>(s.g, (const float*)s.u, (const float*)s.v, (const float*)s.w, a.au2,
                                                 a.av2, a.aw2, a.alpha, a.gq, a.au, a.av, a.aw);
}
void launch_adj_mac_rhs(const DevState& s, const AdjState& a, cudaStream_t st) {
  // transpose of the mean removal (a symmetric projection), then D^T
  launch_sum(a.arhs, s.g.n(), a.part, s.num_sms, st);
  launch_sub_mean(a.arhs, s.g.n(), a.part, s.num_sms, st);
  k_adj_mac_rhs<<<cgrid(s.g), cblock(), 0, st>>>(s.g, a.arhs, a.au, a.av, a.aw);
}
void launch_adj_project(const DevState& s, const AdjState& a, cudaStream_t st) {
  k_adj_project<<<cgrid(s.g), cblock(), 0, st>>>(s.g, a.au, a.av, a.aw, a.ap);
}

static inline dim3 qblock(const Grid& d) {
  const int q = d.nx / 8;
  const int bx = q < 256 ? q : 256;
  int by = 256 / bx;
  if (by > d.ny) by = d.ny;
  return dim3(bx, by, 1);
}
static inline dim3 qgrid(const Grid& d, const dim3& b) {
  return dim3((d.nx / 8 + b.x - 1) / b.x, (d.ny + b.y - 1) / b.y, d.nz);
}
// transpose of `sweeps` red-black sweeps (red then black each) on one level
static void adj_smooth(const Grid& d, float h2, int ref, int sweeps, float* xb, float* bb, cudaStream_t st) {
  const int K = 2 * sweeps;
  if (K == 0) return;
  auto color_of = [](int k) { return (k - 1) & 1; };  // half-sweep k = 1..K
  if (d.nx % 8 == 0) {
    const dim3 b = qblock(d), g = qgrid(d, b);
    launch_pdl(k_adj_rbgs_v4, g, b, 0, st, d, 1 - color_of(K), h2, ref, (int)ADJ4_FIRST, xb, bb);
    for (int k = K; k >= 2; --k) {
      const int m = ADJ4_FUSED | (k == K ? ADJ4_OWN_RAW : 0) | (k == 2 ? ADJ4_OUT_RAW : 0);
      launch_pdl(k_adj_rbgs_v4, g, b, 0, st, d, color_of(k), h2, ref, m, xb, bb);
    }
    launch_pdl(k_adj_rbgs_v4, g, b, 0, st, d, color_of(1), h2, ref, (int)ADJ4_FINAL, xb, bb);
    return;
  }
  launch_pdl(k_adj_rbgs, hgrid(d), cblock(), 0, st, d, 1 - color_of(K), h2, ref, (int)ADJ_SWEEP_FIRST, xb, bb);
  for (int k = K; k >= 2; --k)
    launch_pdl(k_adj_rbgs, hgrid(d), cblock(), 0, st, d, color_of(k), h2, ref, (int)ADJ_SWEEP_FUSED, xb, bb);
  launch_pdl(k_adj_rbgs, hgrid(d), cblock(), 0, st, d, color_of(1), h2, ref, (int)ADJ_SWEEP_FINAL, xb, bb);
}
template <int CS>
static void adj_cluster(const MgLevel& L, int ref, int sweeps, float* eb, float* bb, cudaStream_t st) {
  const size_t smem = 2 * (L.d.n() / CS) * sizeof(float);
  launch_pdl(k_adj_coarse_cluster<CS>, dim3(CS), dim3(512), smem, st, L.d, L.h2, ref, sweeps, eb, bb);
}
// Transpose of the exact coarsest solve e = M b (M symmetric):
// Bbar += M Ebar (Ebar is cleared by the caller afterwards).  CTA c forms
// rows 32c..32c+31 like k_coarse_dense: lane l of warp w sums
// M[i][32c + l] Ebar[i] over i = w, w + 32, ..., the 32 warps' partial sums
// are added in shared memory.
__global__ void __launch_bounds__(1024) k_adj_coarse_dense(Grid d, const float* __restrict__ M, int n,
                                                          const float* __restrict__ eb, float* __restrict__ bb) {
  pdl_wait();
  pdl_trigger();
  extern __shared__ float sev[];  // Ebar in natural order (n), then 32 x 32 partial sums
  float* part = sev + n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int x = i % d.nx, y = (i / d.nx) % d.ny, z = i / (d.nx * d.ny);
    sev[i] = eb[rb_index(d, x, y, z)];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int j = blockIdx.x * 32 + lane;
  float acc = 0.0f;
  if (j < n) {
#pragma unroll 8
    for (int i = w; i < n; i += 32) acc = fmaf(M[(size_t)i * n + j], sev[i], acc);
  }
  part[w * 32 + lane] = acc;
  __syncthreads();
  if (w == 0 && j < n) {
    float sum = part[lane];
#pragma unroll
    for (int k = 1; k < 32; ++k) sum += part[k * 32 + lane];
    const int x = j % d.nx, y = (j / d.nx) % d.ny, z = j / (d.nx * d.ny);
    bb[rb_index(d, x, y, z)] += sum;
  }
}
// Transpose of the coarsest-grid solve; Ebar is zero on return.
static void adj_coarse(const DevState& s, const MgLevel& L, int ref, int sweeps, float* eb, float* bb,
                       cudaStream_t st) {
  if (s.coarse_sweeps < 0) {
    launch_pdl(k_adj_coarse_dense, dim3((s.cn + 31) / 32), dim3(1024), (s.cn + 1024) * sizeof(float), st, L.d,
               s.cinv, s.cn, (const float*)eb, bb);
    cudaMemsetAsync(eb, 0, L.d.n() * sizeof(float), st);
    return;
  }
  int cs = 0;
  for (int c : {8, 4, 2, 1})
    if (L.d.nz % c == 0 && 2 * (L.d.n() / c) * sizeof(float) <= 200 * 1024) { cs = c; break; }
  switch (cs) {
    case 8: adj_cluster<8>(L, ref, sweeps, eb, bb, st); break;
    case 4: adj_cluster<4>(L, ref, sweeps, eb, bb, st); break;
    case 2: adj_cluster<2>(L, ref, sweeps, eb, bb, st); break;
    case 1: adj_cluster<1>(L, ref, sweeps, eb, bb, st); break;
    default:
      adj_smooth(L.d, L.h2, ref, sweeps, eb, bb, st);
      cudaMemsetAsync(eb, 0, L.d.n() * sizeof(float), st);
      break;
  }
}
cudaError_t adj_prepare() {
  cudaError_t e = cudaFuncSetAttribute(k_adj_coarse_cluster<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_adj_coarse_cluster<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_adj_coarse_cluster<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_adj_coarse_cluster<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  return e;
}
static inline dim3 pblock(const Grid& c) {
  const int q = c.nx / 2;
  const int bx = q < 256 ? q : 256;
  int by = 256 / bx;
  if (by > c.ny) by = c.ny;
  return dim3(bx, by, 1);
}
static inline dim3 pgrid(const Grid& c, const dim3& b) {
  return dim3((c.nx / 2 + b.x - 1) / b.x, (c.ny + b.y - 1) / b.y, c.nz);
}
static void adj_restrict(const DevState& s, const AdjState& a, int l, float* xb, float* bb, cudaStream_t st) {
  const Grid f = s.lv[l].d, c = s.lv[l + 1].d;  // nx % 4 == 0 on every transfer level
  const dim3 b = pblock(c);
  launch_pdl(k_adj_restrict2, pgrid(c, b), b, 0, st, f, c, 1.0f / s.lv[l].h2, s.ref, a.lb[l + 1], xb, bb);
  cudaMemsetAsync(a.lb[l + 1], 0, c.n() * sizeof(float), st);
}
// black: the level's post-smoothing has sweeps (the forward's prolongation
// then updates only the black cells, and the transposed sweeps leave the
// red cotangents zero)
static void adj_prolong(const DevState& s, const AdjState& a, int l, const float* xb, bool black, cudaStream_t st) {
  const Grid f = s.lv[l].d, c = s.lv[l + 1].d;
  const dim3 b = pblock(c);
  if (black) launch_pdl(k_adj_prolong2<true>, pgrid(c, b), b, 0, st, f, c, s.ref, xb, a.le[l + 1]);
  else launch_pdl(k_adj_prolong2<false>, pgrid(c, b), b, 0, st, f, c, s.ref, xb, a.le[l + 1]);
}
// Transpose of one V-cycle (k_mg.cu vcycle) on (ap, arhs); the coarse
// adjoint arrays are zero on entry and on exit.
static void adj_vcycle(const DevState& s, const AdjState& a, cudaStream_t st) {
  const int L = s.nlev;
  const MgLevel& L0 = s.lv[0];
  if (L == 1) {
    adj_smooth(L0.d, L0.h2, s.ref, s.pre + s.post, a.ap, a.arhs, st);
    return;
  }
  adj_smooth(L0.d, L0.h2, s.ref, s.post0, a.ap, a.arhs, st);
  adj_prolong(s, a, 0, a.ap, s.post0 > 0, st);
  for (int l = 1; l < L - 1; ++l) {
    adj_smooth(s.lv[l].d, s.lv[l].h2, s.ref, s.post, a.le[l], a.lb[l], st);
    adj_prolong(s, a, l, a.le[l], s.post > 0, st);
  }
  const MgLevel& LC = s.lv[L - 1];
  adj_coarse(s, LC, s.ref, s.coarse_sweeps, a.le[L - 1], a.lb[L - 1], st);
  for (int l = L - 2; l >= 1; --l) {
    adj_restrict(s, a, l, a.le[l], a.lb[l], st);
    adj_smooth(s.lv[l].d, s.lv[l].h2, s.ref, s.pre, a.le[l], a.lb[l], st);
    cudaMemsetAsync(a.le[l], 0, s.lv[l].d.n() * sizeof(float), st);
  }
  adj_restrict(s, a, 0, a.ap, a.arhs, st);
  adj_smooth(L0.d, L0.h2, s.ref, s.pre0, a.ap, a.arhs, st);
}
// rhs += lam + lamlo (the adjoint of the right-hand side through an exact
// solve); the solution's adjoint is consumed
__global__ void __launch_bounds__(256) k_adj_take_solution(const float* __restrict__ lam,
                                                           const float* __restrict__ lamlo, float* arhs, float* ap,
                                                           size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    arhs[i] += lam[i] + lamlo[i];
    ap[i] = 0.0f;
  }
}
void launch_adj_pressure_solve(const DevState& s, const AdjState& a, cudaStream_t st) {
  const size_t n = s.g.n();
  if (!s.ref) {
    launch_sum(a.ap, n, a.part + kSumBlocks, s.num_sms, st);
    launch_sub_mean(a.ap, n, a.part + kSumBlocks, s.num_sms, st);
  }
  if (s.prec == DOB_PREC_MIXED) {
    // The mixed forward solves to a tolerance, not a fixed number of cycles:
    // its pressure is A^+ b up to that tolerance, whatever the warm start, so
    // its adjoint is the same solve: A lam = ap (A symmetric, ap zero-mean),
    // by the mixed solver itself to ||ap - A lam|| <= kAdjRelTol ||ap||, then
    // rhs adjoint += lam and no adjoint reaches the warm start.  The solve
    // starts from the previous (later) step's lam, which the reverse sweep
    // leaves in place: the adjoint pressures of neighbouring steps are close,
    // so fewer V-cycles reach the tolerance.
    DevState t = s;
    t.p = a.lam;
    t.plo = a.lamlo;
    t.rhs = a.ap;
    t.rel_tol = kAdjRelTol;
    t.div_tol_r = 0.0f;
    t.max_outer = kMixedMaxRounds;
    t.cycles = 0;
    launch_pressure_solve(t, st);
    k_adj_take_solution<<<s.num_sms * 4, 256, 0, st>>>(a.lam, a.lamlo, a.arhs, a.ap, n);
    return;
  }
  for (int c = 0; c < s.cycles; ++c) adj_vcycle(s, a, st);
}
void launch_adj_conc_predict(const DevState& s, const AdjState& a, cudaStream_t st) {
  ADJ_DYE_DISPATCH(s.prec, {
    k_adj_conc_predict<DS><<<cgrid(s.gc), cblock(), 0, st>>>(s.gc, s.g, s.params, (const float4*)s.cen,
                                                             (const DS*)s.conc, a.apred, a.ac, a.acen);
  });
}
void launch_adj_conc_resolve(const DevState& s, const AdjState& a, cudaStream_t st) {
  ADJ_DYE_DISPATCH(s.prec, {
    k_adj_dye_resolve<DS><<<cgrid(s.gc), cblock(), 0, st>>>(s.gc, s.g, s.params, (const float4*)s.cen,
                                                            (const DS*)s.conc, (const DS*)s.pred, a.ac2, a.ac,
                                                            a.apred, a.acen);
  });
}

}  // namespace dob
