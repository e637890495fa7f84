// k_box.cu — the closed-box stencil kernels of the step (Casson viscosity,
// divergence, projection + centre velocity) on z-columns.
//
// Column addressing (dob_column.cuh): block 32 x 8, every thread walks ZC
// planes of its (x, y) column with the z-neighbours in registers, the
// x-neighbours from warp shuffles and the y-neighbours from the adjacent
// rows.
//
// Each kernel computes exactly the expressions of its general counterpart in
// k_fluid.cu (k_casson's closed-box branch, k_mac_rhs, k_project followed by
// k_mac_to_center), in the same order, so the results are the same bits;
// the step graph of the closed box uses these, the stage-level interface the
// general kernels.
#include "dob_column.cuh"
#include "dob_kernels.cuh"

namespace dob {
namespace {

using column_detail::kFull;

template <class VS> __device__ __forceinline__ float vs_round(float v);
template <> __device__ __forceinline__ float vs_round<float>(float v) { return v; }
template <> __device__ __forceinline__ float vs_round<__half>(float v) { return __half2float(__float2half_rn(v)); }

// ---- Casson viscosity, closed box (k_casson's closed-box branch) -------------------------
template <class VS, class DS, int ZC>
__global__ void __launch_bounds__(256) k_casson_box(Grid g, const StepParams* __restrict__ Pp,
                                                    const VS* __restrict__ u, const VS* __restrict__ v,
                                                    const VS* __restrict__ w, const DS* __restrict__ dye,
                                                    VS* __restrict__ uo, VS* __restrict__ vo, VS* __restrict__ wo) {
  const Col c = column<ZC>(g);
  if (c.z0 >= g.nz) return;  // uniform over the block
  const StepParams& P = *Pp;
  const float dtv = P.dt, dxv = P.dx;
  const float sqrtMu = dob_sqrt(P.mu_p);
  // the two divisions by launch constants, correctly rounded from their
  // reciprocals (div_by: the IEEE quotients, so the general kernel's bits)
  const float twoDx = 2.0f * dxv, dx2 = dxv * dxv;
  const float rTwoDx = 1.0f / twoDx, rDx2 = 1.0f / dx2;
  const int dym = c.y > 0 ? -(int)c.sy : 0, dyp = c.y < g.ny - 1 ? (int)c.sy : 0;
  uint32_t i = c.i;
  dob_v3 mZn = ld3(u, v, w, c.z0 > 0 ? i - c.sz : i);
  dob_v3 mac = ld3(u, v, w, i);
  // a rolled loop: unrolled over its 8 planes it takes 58 registers and
  // runs slower (93 -> 107 us at 192x256x192)
  for (int z = c.z0; z < c.zend; ++z) {
    const dob_v3 mZp = ld3(u, v, w, z < g.nz - 1 ? i + c.sz : i);
    const dob_v3 mXn = v3(x_minus(c, mac.x, u, i), x_minus(c, mac.y, v, i), x_minus(c, mac.z, w, i));
    const dob_v3 mXp = v3(x_plus(c, g, mac.x, u, i), x_plus(c, g, mac.y, v, i), x_plus(c, g, mac.z, w, i));
    const dob_v3 mYp = ld3(u, v, w, i + dyp), mYn = ld3(u, v, w, i + dym);
    const dob_v3 du = mXp - mXn, dv = mYp - mYn, dw = mZp - mZn;
    const dob_v3 lapMac = (mXp + mXn + mYp + mYn + mZp + mZn) - 6.0f * mac;
    const float cval = ldf(dye + i);
    const float cc = dob_clampf(cval, 0.0f, 1.5f);
    const float ssq = dot3(du, du) + dot3(dv, dv) + dot3(dw, dw);
    // clear water (cc = +0) with a finite shear and yield stress: the yield
    // term is sqrt(+-0 / (gdot + 0.4)), a zero that leaves sqrtMu + it
    // unchanged, so its square roots and division are not formed
    float sqrtYield = 0.0f;
    if (!(cc == 0.0f && ssq <= 3.4e38f && fabsf(P.tau_y) <= 3.4e38f)) {
      const float gdot = div_by(dob_sqrt(ssq), twoDx, rTwoDx);
      sqrtYield = dob_sqrt(P.tau_y * cc * cc / (gdot + 0.4f));
    }
    const float nu = (sqrtMu + sqrtYield) * (sqrtMu + sqrtYield);
    const float alpha = dob_minf(div_by(nu * dtv, dx2, rDx2), 0.125f);
    dob_v3 out = mac + alpha * lapMac;
    if (c.x >= g.nx - 1) out.x = 0.0f;
    if (z >= g.nz - 1) out.z = 0.0f;
    if (c.y >= g.ny - 1) out.y = 0.0f;
    if (c.valid) { stf(uo + i, out.x); stf(vo + i, out.y); stf(wo + i, out.z); }
    mZn = mac;
    mac = mZp;
    i += c.sz;
  }
}

// ---- divergence into the split right-hand side (k_mac_rhs, closed box) ------------------
template <class VS, int ZC, bool FULL>
__global__ void __launch_bounds__(256) k_rhs_box(Grid g, const VS* __restrict__ u, const VS* __restrict__ v,
                                                 const VS* __restrict__ w, float* __restrict__ rhs) {
  const Col c = column<ZC>(g);
  if (c.z0 >= g.nz) return;
  const uint32_t half = (uint32_t)(g.n() >> 1), hx = (uint32_t)g.nx >> 1;
  uint32_t i = c.i;
  float wBack = c.z0 > 0 ? ldf(w + i - c.sz) : 0.0f;
#pragma unroll
  for (int k = 0; k < ZC; ++k) {
    const int z = c.z0 + k;
    if (!FULL && z >= c.zend) break;
    const float uo_ = ldf(u + i), vo_ = ldf(v + i), wo_ = ldf(w + i);
    const float uL = x_minus(c, uo_, u, i);
    const float uRight = c.x >= g.nx - 1 ? 0.0f : uo_;
    const float uLeft = c.x == 0 ? 0.0f : uL;
    const float vTop = c.y >= g.ny - 1 ? 0.0f : vo_;
    const float vBot = c.y == 0 ? 0.0f : ldf(v + i - c.sy);
    const float wFront = z >= g.nz - 1 ? 0.0f : wo_;
    const float r = (uRight - uLeft) + (vTop - vBot) + (wFront - wBack);
    if (c.valid) {
      const uint32_t k = ((uint32_t)(c.x + c.y + z) & 1u) * half + ((uint32_t)z * (uint32_t)g.ny + c.y) * hx +
                         ((uint32_t)c.x >> 1);
      rhs[k] = r;
    }
    wBack = wo_;
    i += c.sz;
  }
}

// ---- projection + centre velocity (k_project then k_mac_to_center, closed box) ----------
// The projected faces go to uo/vo/wo (each cell also reads the old faces
// below it); each cell forms its lower faces' projected values with the
// arithmetic of the cell below, stored with the velocity storage's rounding.
// Bound by the latency of the split-layout pressure loads: capped at 32
// registers (8 blocks per SM, a 24-byte spill), 114.8 -> 102.5 us at
// 192x256x192.
// FULL (nz % ZC == 0): the plane loop has a fixed trip count and is
// unrolled, so the loads of the next planes issue ahead of this plane's
// stores (102 -> 86 us at 192x256x192).  Blocks per SM of the register cap
// (8: 32 registers) as measured against 6 and 4 (97 and 108 us).
#ifndef DOB_PROJECT_MIN_BLOCKS
#define DOB_PROJECT_MIN_BLOCKS 8
#endif
template <class VS, int ZC, bool FULL>
__global__ void __launch_bounds__(256, DOB_PROJECT_MIN_BLOCKS) k_project_center_box(Grid g, const VS* __restrict__ u,
                                                            const VS* __restrict__ v, const VS* __restrict__ w,
                                                            const float* __restrict__ p,
                                                            const float* __restrict__ plo, VS* __restrict__ uo,
                                                            VS* __restrict__ vo, VS* __restrict__ wo,
                                                            typename Vec4Of<VS>::type* __restrict__ cen,
                                                            float scale, unsigned int* __restrict__ maxbits,
                                                            unsigned int* __restrict__ speedbits) {
  const Col c = column<ZC>(g);
  if (c.z0 >= g.nz) return;  // uniform over the block
  const uint32_t half = (uint32_t)(g.n() >> 1), hx = (uint32_t)g.nx >> 1;
  const bool df = plo != nullptr;
  float mdiv = 0.0f;  // max |div| dt/dx of the projected faces (maxbits: statistics)
  unsigned int smax = 0u;  // bits of max |component| of the stored centre velocity (speedbits)
  auto pidx = [&](int x, int y, int z) {  // rb_index in 32 bits
    return ((uint32_t)(x + y + z) & 1u) * half + ((uint32_t)z * (uint32_t)g.ny + (uint32_t)y) * hx + ((uint32_t)x >> 1);
  };
  auto ldp = [&](uint32_t k, float& pv, float& lv) {
    pv = __ldg(p + k);
    lv = df ? __ldg(plo + k) : 0.0f;
  };
  const bool has_ym = c.y > 0, has_yp = c.y < g.ny - 1, has_xm = c.x > 0, has_xp = c.x < g.nx - 1;
  uint32_t i = c.i;
  float pZn = 0.0f, lZn = 0.0f, wBold = 0.0f;  // column at z - 1
  if (c.z0 > 0) {
    ldp(pidx(c.x, c.y, c.z0 - 1), pZn, lZn);
    wBold = ldf(w + i - c.sz);
  }
  float pC, lC;
  ldp(pidx(c.x, c.y, c.z0), pC, lC);
#pragma unroll
  for (int k = 0; k < ZC; ++k) {
    const int z = c.z0 + k;
    if (!FULL && z >= c.zend) break;
    const bool has_zp = z < g.nz - 1;
    float pZp = 0.0f, lZp = 0.0f;
    if (has_zp) ldp(pidx(c.x, c.y, z + 1), pZp, lZp);
    // x neighbours from the neighbouring lanes; the edge lanes of a warp load them
    float pXp = __shfl_down_sync(kFull, pC, 1), lXp = __shfl_down_sync(kFull, lC, 1);
    float pXn = __shfl_up_sync(kFull, pC, 1), lXn = __shfl_up_sync(kFull, lC, 1);
    if (c.lane == 31 && has_xp) ldp(pidx(c.x + 1, c.y, z), pXp, lXp);
    if (c.lane == 0 && has_xm) ldp(pidx(c.x - 1, c.y, z), pXn, lXn);
    float pYp = 0.0f, lYp = 0.0f, pYn = 0.0f, lYn = 0.0f;
    if (has_yp) ldp(pidx(c.x, c.y + 1, z), pYp, lYp);
    if (has_ym) ldp(pidx(c.x, c.y - 1, z), pYn, lYn);
    const float uOwn = ldf(u + i), vOwn = ldf(v + i), wOwn = ldf(w + i);
    const float uSh = __shfl_up_sync(kFull, uOwn, 1);
    const float uLold = has_xm ? (c.lane == 0 ? ldf(u + i - 1) : uSh) : 0.0f;
    const float vDold = has_ym ? ldf(v + i - c.sy) : 0.0f;
    // upper faces: p(hi) - p(this) (+ low parts), as k_project
    auto dp_up = [&](float ph, float lh) { return df ? (ph - pC) + (lh - lC) : (ph - pC); };
    // lower faces: p(this) - p(lo), as the cell below forms it
    auto dp_dn = [&](float pl, float ll) { return df ? (pC - pl) + (lC - ll) : (pC - pl); };
    const float mx = has_xp ? uOwn - dp_up(pXp, lXp) : 0.0f;
    const float my = has_yp ? vOwn - dp_up(pYp, lYp) : 0.0f;
    const float mz = has_zp ? wOwn - dp_up(pZp, lZp) : 0.0f;
    const float uL = has_xm ? vs_round<VS>(uLold - dp_dn(pXn, lXn)) : 0.0f;
    const float vD = has_ym ? vs_round<VS>(vDold - dp_dn(pYn, lYn)) : 0.0f;
    const float wB = z > 0 ? vs_round<VS>(wBold - dp_dn(pZn, lZn)) : 0.0f;
    if (c.valid) {
      stf(uo + i, mx); stf(vo + i, my); stf(wo + i, mz);
      const float uR = vs_round<VS>(mx), vU = vs_round<VS>(my), wF = vs_round<VS>(mz);
      const float cx = 0.5f * (uL + uR), cy = 0.5f * (vD + vU), cz = 0.5f * (wB + wF);
      st4(cen + i, make_float4(cx, cy, cz, 0.0f));
      if (speedbits)  // of the values as stored (binary16 rounds them); NaN orders above every float
        smax = max(smax, max(__float_as_uint(fabsf(vs_round<VS>(cx))),
                             max(__float_as_uint(fabsf(vs_round<VS>(cy))), __float_as_uint(fabsf(vs_round<VS>(cz))))));
      // k_divergence's expression on the stored faces (walls are 0)
      if (maxbits) mdiv = dob_maxf(mdiv, fabsf((uR - uL) + (vU - vD) + (wF - wB)) * scale);
    }
    pZn = pC; lZn = lC;
    pC = pZp; lC = lZp;
    wBold = wOwn;
    i += c.sz;
  }
  if (maxbits) block_max_atomic(mdiv, maxbits);
  if (speedbits) block_max_u32(smax, speedbits);
}

template <int ZC>
inline dim3 col_grid(const Grid& g) { return dim3((g.nx + 31) / 32, (g.ny + 7) / 8, (g.nz + ZC - 1) / ZC); }
constexpr int kCassonZ = 8, kRhsZ = 8, kProjectZ = 4;  // planes per thread (measured at 192x256x192)

}  // namespace

bool box_casson_applies(const DevState& s) {
  return !s.ref && s.gc.nx == s.g.nx && s.gc.ny == s.g.ny && s.gc.nz == s.g.nz;
}

void launch_casson_box(const DevState& s, cudaStream_t st) {
  DOB_VEL_DISPATCH(s.prec, {
    k_casson_box<VS, DS, kCassonZ><<<col_grid<kCassonZ>(s.g), dim3(32, 8), 0, st>>>(
        s.g, s.params, (const VS*)s.u, (const VS*)s.v, (const VS*)s.w, (const DS*)s.conc, (VS*)s.u2, (VS*)s.v2,
        (VS*)s.w2);
  });
}

void launch_mac_rhs_box(const DevState& s, cudaStream_t st, double* sumsq) {
  DOB_VEL_DISPATCH(s.prec, {
    if (s.g.nz % kRhsZ == 0)
      k_rhs_box<VS, kRhsZ, true><<<col_grid<kRhsZ>(s.g), dim3(32, 8), 0, st>>>(s.g, (const VS*)s.u, (const VS*)s.v,
                                                                             (const VS*)s.w, s.rhs);
    else
      k_rhs_box<VS, kRhsZ, false><<<col_grid<kRhsZ>(s.g), dim3(32, 8), 0, st>>>(s.g, (const VS*)s.u, (const VS*)s.v,
                                                                              (const VS*)s.w, s.rhs);
  });
  launch_sum(s.rhs, s.g.n(), s.part + PART_RHS * kSumBlocks, s.num_sms, st);
  launch_sub_mean(s.rhs, s.g.n(), s.part + PART_RHS * kSumBlocks, s.num_sms, st, sumsq);
}

void launch_project_center_box(const DevState& s, cudaStream_t st, float scale, unsigned int* maxbits,
                               unsigned int* speedbits) {
  DOB_VEL_DISPATCH(s.prec, {
    if (s.g.nz % kProjectZ == 0)
      k_project_center_box<VS, kProjectZ, true><<<col_grid<kProjectZ>(s.g), dim3(32, 8), 0, st>>>(
          s.g, (const VS*)s.u, (const VS*)s.v, (const VS*)s.w, s.p, s.plo, (VS*)s.u2, (VS*)s.v2, (VS*)s.w2,
          (typename Vec4Of<VS>::type*)s.cen, scale, maxbits, speedbits);
    else
      k_project_center_box<VS, kProjectZ, false><<<col_grid<kProjectZ>(s.g), dim3(32, 8), 0, st>>>(
          s.g, (const VS*)s.u, (const VS*)s.v, (const VS*)s.w, s.p, s.plo, (VS*)s.u2, (VS*)s.v2, (VS*)s.w2,
          (typename Vec4Of<VS>::type*)s.cen, scale, maxbits, speedbits);
  });
}

}  // namespace dob
