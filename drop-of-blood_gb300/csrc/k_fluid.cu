// k_fluid.cu — velocity-grid kernels of the step: initial field, MAC
// advection, MAC->centre, curl, Casson viscosity + forces, divergence,
// projection, and the dye/conc transport kernels.
//
// Each kernel is one HBM-bound pass over the grid (one thread per cell,
// x-fastest warps so every field access is a coalesced row segment; the
// trilinear gathers of the centre field are 16 B AoS loads).
#include "dob_kernels.cuh"

namespace dob {

// ---- evalTopDirichletPressure (fluid.ts:16-77) ------------------------------------
__device__ float top_pressure(const Grid& g, const StepParams& P, const float4* wave, int ix, int iz) {
  const float halfXZ = P.U[52];
  const float fx = ((float)ix + 0.5f) / (float)g.nx;
  const float fz = ((float)iz + 0.5f) / (float)g.nz;
  const float wx = dob_mix(-halfXZ, halfXZ, fx), wz = dob_mix(-halfXZ, halfXZ, fz);
  const float dtv = P.dt;
  const float cellH = (2.0f * halfXZ) / (float)g.nx;
  const float dtOverH = dtv / cellH;
  const float4 ws = sample_wave(wave, wx, wz, 0.002f, 0.998f);
  const float eta = ws.x, lap = ws.z;
  const float capTerm = -18.4f * lap;
  float pK = 2.45f * (0.155f * eta + 0.00095f * capTerm);
  for (int d = 0; d < kMaxDrops; ++d) {
    const float signedSeed = drop(P, d, 7), drain = drop(P, d, 6);
    if (signedSeed > 0.0f && drain > 0.0005f) {
      const float rx = wx - drop(P, d, 0), rz = wz - drop(P, d, 2);
      const float r = length2f(rx, rz);
      const float theta = dob_atan2(rz, rx);
      const float seed = signedSeed;
      const float azim = 1.0f + 0.022f * dob_cos(4.0f * theta + seed * 1.73f) +
                         0.016f * dob_cos(6.0f * theta - seed * 2.31f) + 0.010f * dob_sin(8.0f * theta + seed * 0.89f);
      const float slugPhase = dob_smoothstep(0.32f, 0.92f, drain);
      const float rOrifice =
          dob_clampf(drop(P, d, 3) * 1.12f + dob_mix(0.018f, 0.032f, slugPhase), 0.030f, 0.090f) * azim;
      const float rNorm = r / dob_maxf(rOrifice, 1e-4f);
      const float speedY = dob_clampf(-drop(P, d, 4), 0.08f, 0.65f);
      const float neck = (0.28f + 1.05f * rNorm * rNorm) * dob_exp(-0.92f * rNorm * rNorm) * (1.0f - 0.38f * rNorm * rNorm);
      pK = pK + drain * (0.014f + 0.048f * speedY) * neck;
    }
  }
  const float wallTaper = 1.0f - dob_smoothstep(halfXZ * 0.72f, halfXZ * 0.96f, dob_maxf(fabsf(wx), fabsf(wz)));
  return pK * dtOverH * wallTaper;
}

#define CELL_INDEX                                   \
  const int x = blockIdx.x * blockDim.x + threadIdx.x; \
  const int y = blockIdx.y * blockDim.y + threadIdx.y; \
  const int z = blockIdx.z;                          \
  if (x >= g.nx || y >= g.ny) return;                \
  const size_t i = g.at(x, y, z);

// ---- FLUID_INIT_VEL (fluid.ts:80-121) --------------------------------------------------
template <class VS>
__global__ void k_init_vel(Grid g, const StepParams* __restrict__ Pp, VS* u, VS* v, VS* w,
                           typename Vec4Of<VS>::type* cen, typename Vec4Of<VS>::type* curl) {
  CELL_INDEX
  const StepParams& P = *Pp;
  const dob_v3 dims = v3((float)g.nx, (float)g.ny, (float)g.nz);
  const float seed = P.U[43], surfY = P.U[40], halfXZ = P.U[52];
  const dob_v3 pX = to_world(P, v3((float)x + 1.0f, (float)y + 0.5f, (float)z + 0.5f) / dims);
  const dob_v3 pY = to_world(P, v3((float)x + 0.5f, (float)y + 1.0f, (float)z + 0.5f) / dims);
  const dob_v3 pZ = to_world(P, v3((float)x + 0.5f, (float)y + 0.5f, (float)z + 1.0f) / dims);
  auto fade = [&](dob_v3 q) {
    return (1.0f - dob_smoothstep(halfXZ * 0.55f, halfXZ * 0.96f, dob_maxf(fabsf(q.x), fabsf(q.z)))) *
           (1.0f - dob_smoothstep(surfY - 0.12f, surfY, q.y)) * dob_smoothstep(0.06f, 0.24f, length2f(q.x, q.z));
  };
  float vx = 0.00045f * dob_sin(pX.x * 6.5f) * dob_cos(pX.z * 6.5f) * dob_sin(pX.y * 5.2f + seed * 1.3f) * fade(pX);
  float vy = 0.00030f * dob_cos(pY.x * 6.5f) * dob_sin(pY.z * 6.5f) * dob_cos(pY.y * 5.2f + seed * 0.7f) * fade(pY);
  float vz = -0.00045f * dob_cos(pZ.x * 6.5f) * dob_sin(pZ.z * 6.5f) * dob_sin(pZ.y * 5.2f + seed * 1.3f) * fade(pZ);
  if (x >= g.nx - 1) vx = 0.0f;
  if (z >= g.nz - 1) vz = 0.0f;
  stf(u + i, vx); stf(v + i, vy); stf(w + i, vz);
  st4(cen + i, make_float4(vx, vy, vz, 0.0f));
  st4(curl + i, make_float4(vx, vy, vz, 0.0f));
}

// ---- FLUID_ADVECT_MAC (fluid.ts:144-329) ------------------------------------------------
// The semi-Lagrangian kernels (advection, dye predictor and resolve) are
// bound by the latency of their gathers: their register caps (5, 8 and 8
// blocks of 256 per SM, a few spilled bytes) buy resident warps, measured
// at 192x256x192: 336 -> 327, 150 -> 131 and 94 -> 86 us.
template <class VS>
__device__ __forceinline__ float sample_mac(const Grid& g, const VS* a, dob_v3 uvw, int comp) {
  // 0.5 / n is half the host-formed 1 / n (the same quotient: scaling by a
  // power of two commutes with rounding)
  if (comp == 0) uvw.x = uvw.x - 0.5f * g.rx;
  if (comp == 1) uvw.y = uvw.y - 0.5f * g.ry;
  if (comp == 2) uvw.z = uvw.z - 0.5f * g.rz;
  uvw = clamp3(uvw, 0.001f, 0.999f);
  const Taps t = make_taps_in(g, uvw.x, uvw.y, uvw.z);
  return lerp8(t, a);
}
// midpoint trace from the face centre uvwF, whose centre velocity is v0
template <class V4>
__device__ __forceinline__ dob_v3 trace_back(const Grid& g, const V4* cen, dob_v3 uvwF, dob_v3 v0, float dtv,
                                             const Recip3& dom) {
  const dob_v3 uvwMid = clamp3(uvwF - (0.5f * (v0 * dtv)) / dom, 0.002f, 0.998f);
  const dob_v3 vMid = sample_center_in(g, cen, uvwMid);
  return clamp3(uvwF - (vMid * dtv) / dom, 0.002f, 0.998f);
}
__device__ __forceinline__ float azim_neck(float theta, float seed) {
  return 1.0f + 0.036f * dob_cos(4.0f * theta + seed * 1.73f) + 0.026f * dob_cos(6.0f * theta - seed * 2.31f) +
         0.018f * dob_sin(8.0f * theta + seed * 0.89f);
}

template <class VS>
__global__ void __launch_bounds__(256, 5) k_advect_mac(Grid g, const StepParams* __restrict__ Pp, int ref, int flags,
                                                    const VS* __restrict__ u, const VS* __restrict__ v,
                                                    const VS* __restrict__ w,
                                                    const typename Vec4Of<VS>::type* __restrict__ cen,
                                                    const float4* __restrict__ wave, VS* __restrict__ uo,
                                                    VS* __restrict__ vo, VS* __restrict__ wo) {
  CELL_INDEX
  const StepParams& P = *Pp;
  const Recip3 dimr = grid_recip(g), dom = dom_recip(P);
  const float dtv = P.dt;
  const float damp = P.damp;
  // a: the cell centre, b: the upper faces; face X is (b.x, a.y, a.z) etc.
  const dob_v3 a = v3((float)x + 0.5f, (float)y + 0.5f, (float)z + 0.5f) / dimr;
  const dob_v3 b = v3((float)x + 1.0f, (float)y + 1.0f, (float)z + 1.0f) / dimr;
  const dob_v3 uvwX = v3(b.x, a.y, a.z), uvwY = v3(a.x, b.y, a.z), uvwZ = v3(a.x, a.y, b.z);
  // start samples at the (clamped) face centres: where the texel coordinates
  // are exact the interpolation is the mean of the two cells the face joins
  const dob_v3 ca = clamp3(a, 0.002f, 0.998f), cb = clamp3(b, 0.002f, 0.998f);
  const bool ax = texel_exact(ca.x, g.nx) == (float)x, bx = texel_exact(cb.x, g.nx) == (float)x + 0.5f;
  const bool ay = texel_exact(ca.y, g.ny) == (float)y, by = texel_exact(cb.y, g.ny) == (float)y + 0.5f;
  const bool az = texel_exact(ca.z, g.nz) == (float)z, bz = texel_exact(cb.z, g.nz) == (float)z + 0.5f;
  const size_t sy = (size_t)g.nx, sz = (size_t)g.nx * g.ny;
  const dob_v3 v0X = bx && ay && az ? face_mean(cen, i, 1) : sample_center_exact(g, cen, v3(cb.x, ca.y, ca.z));
  const dob_v3 v0Y = ax && by && az ? face_mean(cen, i, sy) : sample_center_exact(g, cen, v3(ca.x, cb.y, ca.z));
  const dob_v3 v0Z = ax && ay && bz ? face_mean(cen, i, sz) : sample_center_exact(g, cen, v3(ca.x, ca.y, cb.z));
  float vx = sample_mac(g, u, trace_back(g, cen, uvwX, v0X, dtv, dom), 0) * damp;
  float vy = sample_mac(g, v, trace_back(g, cen, uvwY, v0Y, dtv, dom), 1) * damp;
  float vz = sample_mac(g, w, trace_back(g, cen, uvwZ, v0Z, dtv, dom), 2) * damp;
  if (ref) {
    const float surfY = P.U[40];
    const dob_v3 pCell = to_world(P, (v3((float)x, (float)y, (float)z) + v3(0.5f, 0.5f, 0.5f)) / dimr);
    const dob_v3 pFaceY = to_world(P, uvwY);
    float activeNeckMask = 0.0f;
    if (flags & DOB_PHYS_NECK) {
      for (int d = 0; d < kMaxDrops; ++d) {
        const float signedSeed = drop(P, d, 7), drain = drop(P, d, 6);
        if (!(signedSeed > 0.0f && drain > 0.0005f)) continue;
        const float dX = drop(P, d, 0), dZ = drop(P, d, 2);
        const float relx = pFaceY.x - dX, relz = pFaceY.z - dZ;
        const float r = length2f(relx, relz);
        const float seed = signedSeed;
        const float sp = dob_smoothstep(0.14f, 0.76f, drain);
        const float rNeckBase =
            dob_clampf(drop(P, d, 3) * dob_mix(0.80f, 1.08f, sp) + dob_mix(0.012f, 0.030f, sp), 0.018f, 0.088f);
        // The azimuthal factor lies in [0.92, 1.08] and both radial profiles
        // vanish exactly from rRatio = 1.15 on, so at r >= 1.25 rNeckBase the
        // profile, the mask and this drop's share of activeNeckMask are
        // exactly 0; at or below surfY - 0.058 the vertical mask is exactly 0,
        // and activeNeckMask is read only in the top two layers.  The angle
        // and its harmonics are formed only where they can change a result.
        if (r < rNeckBase * 1.25f && (y >= g.ny - 2 || pFaceY.y > surfY - 0.058f)) {
          const float theta = dob_atan2(relz, relx);
          const float azim = azim_neck(theta, seed);
          const float rNeck = rNeckBase * azim;
          const float rRatio = r / dob_maxf(rNeck, 1e-4f);
          const float slugRadial = (0.14f + 1.00f * dob_minf(rRatio * rRatio, 1.20f)) * (1.0f - dob_smoothstep(0.78f, 1.15f, rRatio));
          const float stemRadial = (0.68f + 0.32f * dob_minf(rRatio * rRatio, 1.0f)) * (1.0f - dob_smoothstep(0.74f, 1.10f, rRatio));
          const float radialProfile = dob_mix(stemRadial, slugRadial, sp);
          const float vertMask = dob_smoothstep(surfY - 0.058f, surfY - 0.014f, pFaceY.y);
          const float meniscusShear = dob_mix(1.0f, 0.36f, dob_smoothstep(surfY - 0.024f, surfY - 0.002f, pFaceY.y));
          const float mask = radialProfile * vertMask;
          activeNeckMask = dob_maxf(activeNeckMask, radialProfile);
          if (mask > 0.001f) {
            const float lobeMod = 1.0f + 0.036f * dob_cos(4.0f * theta + seed * 1.73f) + 0.026f * dob_cos(6.0f * theta - seed * 2.31f);
            const float impactSpeed = dob_clampf(-drop(P, d, 4), 0.10f, 0.65f);
            const float slugDrive = dob_clampf(dob_pow(dob_maxf(drain, 0.0f), 0.66f) * 0.84f, 0.0f, 1.24f);
            const float stemDrive = dob_clampf(0.045f + drain * 0.22f, 0.0f, 0.20f) * dob_smoothstep(0.0f, 0.05f, drain);
            const float fluxDrive = dob_mix(stemDrive, slugDrive, sp);
            const float targetVy = -dob_clampf(0.14f + 0.64f * impactSpeed, 0.15f, 0.39f) * fluxDrive * lobeMod * meniscusShear;
            const float blend = dob_clampf(dtv * dob_mix(14.0f, 22.0f, sp) * mask, 0.0f, 1.0f);
            vy = dob_mix(vy, targetVy, blend);
          }
        }
        const float vertMaskXZ = dob_smoothstep(surfY - 0.058f, surfY - 0.014f, pCell.y);
        if (vertMaskXZ > 0.001f) {
          const float flare = dob_mix(0.104f * (0.35f + 0.65f * sp), -0.020f, dob_smoothstep(surfY - 0.066f, surfY - 0.012f, pCell.y)) *
                              dob_clampf(drain, 0.0f, 1.3f);
          for (int comp = 0; comp < 2; ++comp) {
            const dob_v3 fw = to_world(P, comp == 0 ? uvwX : uvwZ);
            const float ax = fw.x - dX, az = fw.z - dZ;
            const float rF = length2f(ax, az);
            if (rF > 1e-4f && rF < rNeckBase * 1.34f) {
              const float thF = dob_atan2(az, ax);
              const float azF = azim_neck(thF, seed);
              const float rR = rF / dob_maxf(rNeckBase * azF, 1e-4f);
              if (rR < 1.22f) {
                const float slugR = (0.14f + 1.00f * dob_minf(rR * rR, 1.20f)) * (1.0f - dob_smoothstep(0.78f, 1.15f, rR));
                const float stemR = (0.68f + 0.32f * dob_minf(rR * rR, 1.0f)) * (1.0f - dob_smoothstep(0.74f, 1.10f, rR));
                const float maskF = dob_mix(stemR, slugR, sp) * vertMaskXZ;
                const float blendF = dob_clampf(dtv * dob_mix(14.0f, 22.0f, sp) * maskF, 0.0f, 1.0f);
                if (comp == 0) vx = dob_mix(vx, (ax / rF) * flare, blendF * 0.65f);
                else vz = dob_mix(vz, (az / rF) * flare, blendF * 0.65f);
              }
            }
          }
        }
      }
    }
    if ((flags & DOB_PHYS_SURFACE) && y >= g.ny - 3) {
      const float topFade = (float)(y - (g.ny - 3) + 1) / 3.0f;
      const float epsW = 0.015f;
      const float4 wc = sample_wave(wave, pCell.x, pCell.z, 0.002f, 0.998f);
      const float wC = wc.w;
      const float wXp = sample_wave(wave, pCell.x + epsW, pCell.z, 0.002f, 0.998f).w;
      const float wXn = sample_wave(wave, pCell.x - epsW, pCell.z, 0.002f, 0.998f).w;
      const float wZp = sample_wave(wave, pCell.x, pCell.z + epsW, 0.002f, 0.998f).w;
      const float wZn = sample_wave(wave, pCell.x, pCell.z - epsW, 0.002f, 0.998f).w;
      const float cmcWindow = 1.0f - dob_smoothstep(0.45f, 0.88f, wC);
      const float gx = (wXp - wXn) / (2.0f * epsW), gz = (wZp - wZn) / (2.0f * epsW);
      const float sc = -P.U[41] * 0.026f * cmcWindow;
      vx = vx + (sc * gx * topFade) * dtv;
      vz = vz + (sc * gz * topFade) * dtv;
      if (y >= g.ny - 2 && activeNeckMask < 0.02f) {
        const float calmGate = 1.0f - dob_smoothstep(0.020f, 0.14f, fabsf(wc.y));
        const float layerWeight = (y == g.ny - 1) ? 0.72f : 0.26f;
        vy = dob_mix(vy, dob_clampf(wc.y * 0.35f, -0.045f, 0.045f), calmGate * layerWeight);
      }
    }
    if (flags & DOB_PHYS_SPONGE) {
      const float halfXZ = P.U[52], yMin = P.U[53];
      const float rCellXZ = length2f(pCell.x, pCell.z);
      // inside the inner radius and above the floor band the fade is exactly
      // 1 and the factor exactly 1: the smoothsteps are formed only outside
      if (!(rCellXZ <= halfXZ * 0.68f && pCell.y >= yMin + 0.052f)) {
        const float wallFade = (1.0f - dob_smoothstep(halfXZ * 0.68f, halfXZ * 0.94f, rCellXZ)) *
                               dob_smoothstep(yMin + 0.004f, yMin + 0.052f, pCell.y);
        const float spongeMul = dob_mix(0.84f, 1.0f, wallFade);
        vx = vx * spongeMul; vy = vy * spongeMul; vz = vz * spongeMul;
      }
    }
  }
  if (x >= g.nx - 1) vx = 0.0f;
  if (z >= g.nz - 1) vz = 0.0f;
  if (!ref && y >= g.ny - 1) vy = 0.0f;
  stf(uo + i, vx); stf(vo + i, vy); stf(wo + i, vz);
}

// ---- FLUID_MAC_TO_CENTER (fluid.ts:917-962) -----------------------------------------------
// Reference mode: a downward centre velocity in the top two layers is
// damped near the surface except inside an active drop's neck.
__device__ __forceinline__ float surface_stagnation(const Grid& g, const StepParams& P, int flags, int x, int y, int z,
                                                    float cy) {
  if (!((flags & DOB_PHYS_SURFACE) && y >= g.ny - 2 && cy < 0.0f)) return cy;
  const Recip3 dims = grid_recip(g);
  const dob_v3 pCell = to_world(P, (v3((float)x, (float)y, (float)z) + v3(0.5f, 0.5f, 0.5f)) / dims);
  float activeNeck = 0.0f;
  for (int d = 0; d < kMaxDrops; ++d) {
    if (drop(P, d, 7) > 0.0f && drop(P, d, 6) > 0.008f) {
      const float rActive = dob_clampf(drop(P, d, 3) * 1.15f + 0.032f, 0.046f, 0.092f);
      const float rDist = length2f(pCell.x - drop(P, d, 0), pCell.z - drop(P, d, 2));
      const float drainGate = dob_smoothstep(0.008f, 0.065f, drop(P, d, 6));
      activeNeck = dob_maxf(activeNeck, (1.0f - dob_smoothstep(rActive * 0.78f, rActive * 1.20f, rDist)) * drainGate);
    }
  }
  const float stagGate = dob_mix(0.45f, 1.0f, dob_smoothstep(0.002f, 0.018f, dob_maxf(0.0f, P.U[40] - pCell.y)));
  return cy * dob_mix(stagGate, 1.0f, activeNeck);
}
template <class VS>
__global__ void __launch_bounds__(256) k_mac_to_center(Grid g, const StepParams* __restrict__ Pp, int ref, int flags,
                                                       const VS* __restrict__ u, const VS* __restrict__ v,
                                                       const VS* __restrict__ w,
                                                       typename Vec4Of<VS>::type* __restrict__ cen) {
  CELL_INDEX
  const float uR = x >= g.nx - 1 ? 0.0f : ldf(u + i);
  const float uL = x == 0 ? 0.0f : ldf(u + i - 1);
  const float vU = (!ref && y >= g.ny - 1) ? 0.0f : ldf(v + i);
  const float vD = y == 0 ? 0.0f : ldf(v + i - g.nx);
  const float wF = z >= g.nz - 1 ? 0.0f : ldf(w + i);
  const float wB = z == 0 ? 0.0f : ldf(w + i - (size_t)g.nx * g.ny);
  const float cx = 0.5f * (uL + uR), cz = 0.5f * (wB + wF);
  float cy = 0.5f * (vD + vU);
  if (ref) cy = surface_stagnation(g, *Pp, flags, x, y, z, cy);
  st4(cen + i, make_float4(cx, cy, cz, 0.0f));
}

// ---- FLUID_CURL (fluid.ts:331-369) ----------------------------------------------------------
template <class V4>
__device__ __forceinline__ float4 ldc4(const Grid& g, const V4* a, int x, int y, int z) {
  return ld4(a + g.at(dob_clampi(x, 0, g.nx - 1), dob_clampi(y, 0, g.ny - 1), dob_clampi(z, 0, g.nz - 1)));
}
template <class VS>
__global__ void __launch_bounds__(256) k_curl(Grid g, const typename Vec4Of<VS>::type* __restrict__ cen,
                                              typename Vec4Of<VS>::type* __restrict__ curl) {
  CELL_INDEX
  const float4 vR = ldc4(g, cen, x + 1, y, z), vL = ldc4(g, cen, x - 1, y, z);
  const float4 vU = ldc4(g, cen, x, y + 1, z), vD = ldc4(g, cen, x, y - 1, z);
  const float4 vF = ldc4(g, cen, x, y, z + 1), vB = ldc4(g, cen, x, y, z - 1);
  const dob_v3 om = 0.5f * v3((vU.z - vD.z) - (vF.y - vB.y), (vF.x - vB.x) - (vR.z - vL.z), (vR.y - vL.y) - (vU.x - vD.x));
  const float mag = length3(om);
  st4(curl + i, make_float4(om.x, om.y, om.z, mag));
}

// ---- FLUID_CASSON_FORCES (fluid.ts:377-511) ------------------------------------------------
template <class VS>
__device__ __forceinline__ dob_v3 ldmac(const Grid& g, const VS* u, const VS* v, const VS* w, int x, int y, int z) {
  const size_t j = g.at(dob_clampi(x, 0, g.nx - 1), dob_clampi(y, 0, g.ny - 1), dob_clampi(z, 0, g.nz - 1));
  return v3(ldf(u + j), ldf(v + j), ldf(w + j));
}
template <class V4>
__device__ __forceinline__ dob_v3 vort_conf(const Grid& g, const V4* curl, int ix, int iy, int iz, float vc) {
  if (ix <= 1 || ix >= g.nx - 2 || iy <= 1 || iy >= g.ny - 3 || iz <= 1 || iz >= g.nz - 2) return v3(0.0f, 0.0f, 0.0f);
  const float4 c = ld4(curl + g.at(ix, iy, iz));
  const dob_v3 omega = v3(c.x, c.y, c.z);
  const float omegaMag = c.w;
  if (omegaMag <= 0.18f) return v3(0.0f, 0.0f, 0.0f);
  const float ringGate = dob_smoothstep(0.18f, 0.95f, omegaMag) / (1.0f + 0.28f * omegaMag);
  const dob_v3 eta = 0.5f * v3(ldc4(g, curl, ix + 1, iy, iz).w - ldc4(g, curl, ix - 1, iy, iz).w,
                               ldc4(g, curl, ix, iy + 1, iz).w - ldc4(g, curl, ix, iy - 1, iz).w,
                               ldc4(g, curl, ix, iy, iz + 1).w - ldc4(g, curl, ix, iy, iz - 1).w);
  const float etaLen = length3(eta);
  if (etaLen <= 1e-5f) return v3(0.0f, 0.0f, 0.0f);
  return (vc * ringGate) * cross3(eta / etaLen, omega);
}
template <class DS>
__device__ __forceinline__ dob_v3 sample_conc_rg(const Grid& gc, const typename Vec4Of<DS>::type* conc4, dob_v3 uvw) {
  const Taps t = make_taps(gc, uvw.x, uvw.y, uvw.z);
  const float4 r = lerp8x4(t, conc4);
  return v3(r.x, r.y, 0.0f);
}

template <class VS, class DS>
__global__ void __launch_bounds__(256) k_casson(Grid g, Grid gc, const StepParams* __restrict__ Pp, int ref, int flags,
                                                const VS* __restrict__ u, const VS* __restrict__ v,
                                                const VS* __restrict__ w,
                                                const typename Vec4Of<VS>::type* __restrict__ curl,
                                                const typename Vec4Of<DS>::type* __restrict__ conc4,
                                                const DS* __restrict__ dye, VS* __restrict__ uo, VS* __restrict__ vo,
                                                VS* __restrict__ wo) {
  CELL_INDEX
  const StepParams& P = *Pp;
  const Recip3 dims = grid_recip(g);
  const float dtv = P.dt;
  dob_v3 mac = v3(ldf(u + i), ldf(v + i), ldf(w + i));
  const dob_v3 mXp = ldmac(g, u, v, w, x + 1, y, z), mXn = ldmac(g, u, v, w, x - 1, y, z);
  const dob_v3 mYp = ldmac(g, u, v, w, x, y + 1, z), mYn = ldmac(g, u, v, w, x, y - 1, z);
  const dob_v3 mZp = ldmac(g, u, v, w, x, y, z + 1), mZn = ldmac(g, u, v, w, x, y, z - 1);
  const dob_v3 uvwCell = (v3((float)x, (float)y, (float)z) + v3(0.5f, 0.5f, 0.5f)) / dims;
  const dob_v3 du = mXp - mXn, dv = mYp - mYn, dw = mZp - mZn;
  const dob_v3 lapMac = (mXp + mXn + mYp + mYn + mZp + mZn) - 6.0f * mac;
  if (ref) {
    const dob_v3 concCell = sample_conc_rg<DS>(gc, conc4, uvwCell);
    const float cRbc = dob_clampf(concCell.x, 0.0f, 1.5f);
    const float cassonScale = P.U[58];
    const float sqrtMuInf = dob_sqrt(0.00010f * (1.0f + 1.35f * cRbc));
    // without red cells (cRbc = +0) and with a finite scale the yield term
    // is sqrt(+-0 / max(shearRate + 0.4, 0.4)), a zero that leaves
    // sqrtMuInf + it unchanged: the shear rate's root and the division are
    // not formed
    float sqrtYieldTerm = 0.0f;
    if (!(cRbc == 0.0f && fabsf(cassonScale) <= 3.4e38f)) {
      const float shearRate = 50.0f * dob_sqrt(dot3(du, du) + dot3(dv, dv) + dot3(dw, dw) + 1e-6f);
      const float tauYield = 0.0036f * cassonScale * cRbc * cRbc;
      sqrtYieldTerm = dob_sqrt(tauYield / dob_maxf(shearRate + 0.40f, 0.40f));
    }
    const float alpha = dob_clampf((sqrtMuInf + sqrtYieldTerm) * (sqrtMuInf + sqrtYieldTerm), 0.00010f, 0.0044f);
    mac = mac + alpha * lapMac;
    if (flags & DOB_PHYS_VORT_CONF) {
      const float vcs = P.U[44];
      const dob_v3 vc0 = vort_conf(g, curl, x, y, z, vcs);
      const float vcX = 0.5f * (vc0.x + vort_conf(g, curl, min(x + 1, g.nx - 1), y, z, vcs).x);
      const float vcY = 0.5f * (vc0.y + vort_conf(g, curl, x, min(y + 1, g.ny - 1), z, vcs).y);
      const float vcZ = 0.5f * (vc0.z + vort_conf(g, curl, x, y, min(z + 1, g.nz - 1), vcs).z);
      mac = mac + v3(vcX, vcY, vcZ) * dtv;
    }
    if (flags & DOB_PHYS_BUOYANCY) {
      const dob_v3 uvwFaceY = v3((float)x + 0.5f, (float)y + 1.0f, (float)z + 0.5f) / dims;
      const dob_v3 cf = sample_conc_rg<DS>(gc, conc4, clamp3(uvwFaceY, 0.001f, 0.999f));
      const float buoyDensity = 1.24f * cf.x + 0.26f * cf.y;
      if (buoyDensity > 0.0008f) {
        const dob_v3 pFaceY = to_world(P, uvwFaceY);
        const float surfBuoyGate = dob_smoothstep(0.002f, 0.024f, dob_maxf(0.0f, P.U[40] - pFaceY.y));
        const float effBuoyConc = 1.24f * dob_tanh(buoyDensity / 1.24f);
        const float buoyAccel = -P.U[45] * 0.345f * effBuoyConc * surfBuoyGate;
        mac.y = mac.y + buoyAccel * dtv;
      }
    }
    if (flags & DOB_PHYS_SOLENOIDAL) {
      const dob_v3 pc = to_world(P, uvwCell);
      const float depthBelow = P.U[40] - pc.y;
      const float unfurlGate = dob_smoothstep(0.11f, 0.36f, depthBelow) * dob_smoothstep(0.0008f, 0.015f, cRbc + 0.45f * concCell.y);
      if (unfurlGate > 0.001f) {
        const float tSwirl = P.U[35] * 0.36f + P.U[60] * 1.7f;
        const float q1 = 6.4f * pc.x + 4.0f * pc.y + 5.2f * pc.z + tSwirl;
        const float q2 = -5.6f * pc.x + 4.8f * pc.y + 7.2f * pc.z - tSwirl * 0.77f;
        const float q3 = 9.0f * pc.x - 6.0f * pc.y - 6.4f * pc.z + tSwirl * 1.13f;
        const float c1 = dob_cos(q1), c2 = dob_cos(q2), s3 = 0.42f * dob_sin(q3);
        const dob_v3 sf = v3(-6.25f, 2.85f, 5.50f) * c1 + v3(-6.30f, -1.26f, -4.06f) * c2 + v3(6.40f, -0.96f, 9.90f) * s3;
        const float vertMod = dob_smoothstep(0.16f, 0.42f, depthBelow);
        mac = mac + v3(sf.x, sf.y * vertMod, sf.z) * (0.0028f * unfurlGate * dtv);
      }
    }
    mac = clamp3(mac, -1.8f, 1.8f);
  } else {
    // Closed box: nu = (sqrt(mu_p) + sqrt(tau_y c^2 / (gdot + 0.4)))^2, explicit
    // u += min(nu dt / dx^2, 1/8) lap u.
    const float cval = gc.nx == g.nx ? ldf(dye + i) : lerp8(make_taps(gc, uvwCell.x, uvwCell.y, uvwCell.z), dye);
    const float c = dob_clampf(cval, 0.0f, 1.5f);
    const float dxv = P.dx;
    const float gdot = dob_sqrt(dot3(du, du) + dot3(dv, dv) + dot3(dw, dw)) / (2.0f * dxv);
    const float sqrtMu = dob_sqrt(P.mu_p);
    const float sqrtYield = dob_sqrt(P.tau_y * c * c / (gdot + 0.4f));
    const float nu = (sqrtMu + sqrtYield) * (sqrtMu + sqrtYield);
    const float alpha = dob_minf(nu * dtv / (dxv * dxv), 0.125f);
    mac = mac + alpha * lapMac;
  }
  if (x >= g.nx - 1) mac.x = 0.0f;
  if (z >= g.nz - 1) mac.z = 0.0f;
  if (!ref && y >= g.ny - 1) mac.y = 0.0f;
  stf(uo + i, mac.x); stf(vo + i, mac.y); stf(wo + i, mac.z);
}

// ---- FLUID_MAC_RHS (fluid.ts:517-555) with the FP64 compatibility sum ---------------------
template <class VS>
__global__ void __launch_bounds__(256) k_mac_rhs(Grid g, const StepParams* __restrict__ Pp, int ref,
                                                 const VS* __restrict__ u, const VS* __restrict__ v,
                                                 const VS* __restrict__ w, const float4* __restrict__ wave,
                                                 float* __restrict__ rhs, double* __restrict__ sum) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  double part = 0.0;
  if (x < g.nx && y < g.ny) {
    const size_t i = g.at(x, y, z);
    const float uRight = x >= g.nx - 1 ? 0.0f : ldf(u + i);
    const float uLeft = x == 0 ? 0.0f : ldf(u + i - 1);
    const float vTop = (!ref && y >= g.ny - 1) ? 0.0f : ldf(v + i);
    const float vBot = y == 0 ? 0.0f : ldf(v + i - g.nx);
    const float wFront = z >= g.nz - 1 ? 0.0f : ldf(w + i);
    const float wBack = z == 0 ? 0.0f : ldf(w + i - (size_t)g.nx * g.ny);
    float r = (uRight - uLeft) + (vTop - vBot) + (wFront - wBack);
    if (ref && y == g.ny - 1) r = r - top_pressure(g, *Pp, wave, x, z);
    rhs[rb_index(g, x, y, z)] = r;
    part = (double)r;
  }
  if (sum) block_sum_atomic(part, sum);
}

// ---- FLUID_MAC_PROJECT (fluid.ts:863-911), in place ----------------------------------------
template <class VS>
__global__ void __launch_bounds__(256) k_project(Grid g, const StepParams* __restrict__ Pp, int ref, VS* u, VS* v, VS* w,
                                                 const float* __restrict__ p, const float* __restrict__ plo,
                                                 const float4* __restrict__ wave) {
  CELL_INDEX
  float mx = ldv(u + i), my = ldv(v + i), mz = ldv(w + i);
  // p is red-black split: the +x, +y, +z neighbours are in the other half.
  // With a double-float pressure (p + plo) the differences of the high parts
  // are taken first, then the low parts added.
  const size_t ic = rb_index(g, x, y, z);
  const float pC = __ldg(p + ic);
  const float lC = plo ? __ldg(plo + ic) : 0.0f;
  auto dp = [&](size_t j) { return plo ? (__ldg(p + j) - pC) + (__ldg(plo + j) - lC) : (__ldg(p + j) - pC); };
  if (x < g.nx - 1) mx = mx - dp(rb_index(g, x + 1, y, z)); else mx = 0.0f;
  if (y < g.ny - 1) my = my - dp(rb_index(g, x, y + 1, z));
  else if (ref) my = my - (top_pressure(g, *Pp, wave, x, z) - pC);
  else my = 0.0f;
  if (z < g.nz - 1) mz = mz - dp(rb_index(g, x, y, z + 1)); else mz = 0.0f;
  if (ref) {
    mx = dob_clampf(mx, -2.0f, 2.0f); my = dob_clampf(my, -2.0f, 2.0f); mz = dob_clampf(mz, -2.0f, 2.0f);
  }
  stf(u + i, mx); stf(v + i, my); stf(w + i, mz);
}

// FLUID_MAC_PROJECT and the MAC_TO_CENTER that follows it (reference mode)
// in one pass, out of place: the projected faces go to uo/vo/wo (the caller
// swaps the buffers); each cell forms its lower faces' projected values with
// k_project's arithmetic for the cell below, then the centre velocity from
// the faces as stored (binary16 rounds them) with k_mac_to_center's.
template <class VS> __device__ __forceinline__ float as_stored_vs(float v);
template <> __device__ __forceinline__ float as_stored_vs<float>(float v) { return v; }
template <> __device__ __forceinline__ float as_stored_vs<__half>(float v) { return __half2float(__float2half_rn(v)); }
template <class VS>
__global__ void __launch_bounds__(256) k_project_center_ref(Grid g, const StepParams* __restrict__ Pp, int flags,
                                                            const VS* __restrict__ u, const VS* __restrict__ v,
                                                            const VS* __restrict__ w, const float* __restrict__ p,
                                                            const float* __restrict__ plo,
                                                            const float4* __restrict__ wave, VS* __restrict__ uo,
                                                            VS* __restrict__ vo, VS* __restrict__ wo,
                                                            typename Vec4Of<VS>::type* __restrict__ cen) {
  CELL_INDEX
  const size_t ic = rb_index(g, x, y, z);
  const float pC = __ldg(p + ic);
  const float lC = plo ? __ldg(plo + ic) : 0.0f;
  // the face between a lower cell (pl, ll) and an upper one (ph, lh)
  auto dpf = [&](size_t jl, size_t jh) {
    return plo ? (__ldg(p + jh) - __ldg(p + jl)) + (__ldg(plo + jh) - __ldg(plo + jl)) : (__ldg(p + jh) - __ldg(p + jl));
  };
  float mx = ldf(u + i), my = ldf(v + i), mz = ldf(w + i);
  if (x < g.nx - 1) mx = mx - dpf(ic, rb_index(g, x + 1, y, z)); else mx = 0.0f;
  if (y < g.ny - 1) my = my - dpf(ic, rb_index(g, x, y + 1, z));
  else my = my - (top_pressure(g, *Pp, wave, x, z) - pC);
  if (z < g.nz - 1) mz = mz - dpf(ic, rb_index(g, x, y, z + 1)); else mz = 0.0f;
  mx = dob_clampf(mx, -2.0f, 2.0f); my = dob_clampf(my, -2.0f, 2.0f); mz = dob_clampf(mz, -2.0f, 2.0f);
  stf(uo + i, mx); stf(vo + i, my); stf(wo + i, mz);
  float uL = 0.0f, vD = 0.0f, wB = 0.0f;
  if (x > 0) uL = as_stored_vs<VS>(dob_clampf(ldf(u + i - 1) - dpf(rb_index(g, x - 1, y, z), ic), -2.0f, 2.0f));
  if (y > 0) vD = as_stored_vs<VS>(dob_clampf(ldf(v + i - g.nx) - dpf(rb_index(g, x, y - 1, z), ic), -2.0f, 2.0f));
  if (z > 0)
    wB = as_stored_vs<VS>(dob_clampf(ldf(w + i - (size_t)g.nx * g.ny) - dpf(rb_index(g, x, y, z - 1), ic), -2.0f, 2.0f));
  const float uR = x >= g.nx - 1 ? 0.0f : as_stored_vs<VS>(mx);
  const float vU = as_stored_vs<VS>(my);
  const float wF = z >= g.nz - 1 ? 0.0f : as_stored_vs<VS>(mz);
  const float cx = 0.5f * (uL + uR), cz = 0.5f * (wB + wF);
  const float cy = surface_stagnation(g, *Pp, flags, x, y, z, 0.5f * (vD + vU));
  st4(cen + i, make_float4(cx, cy, cz, 0.0f));
}

// ---- divergence field and its max (statistics) -----------------------------------------
template <class VS>
__global__ void __launch_bounds__(256) k_divergence(Grid g, int ref, const VS* __restrict__ u, const VS* __restrict__ v,
                                                    const VS* __restrict__ w, float* __restrict__ out,
                                                    float scale, unsigned int* __restrict__ maxbits) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  float m = 0.0f;
  if (x < g.nx && y < g.ny) {
    const size_t i = g.at(x, y, z);
    const float uRight = x >= g.nx - 1 ? 0.0f : ldf(u + i);
    const float uLeft = x == 0 ? 0.0f : ldf(u + i - 1);
    const float vTop = (!ref && y >= g.ny - 1) ? 0.0f : ldf(v + i);
    const float vBot = y == 0 ? 0.0f : ldf(v + i - g.nx);
    const float wFront = z >= g.nz - 1 ? 0.0f : ldf(w + i);
    const float wBack = z == 0 ? 0.0f : ldf(w + i - (size_t)g.nx * g.ny);
    const float d = (uRight - uLeft) + (vTop - vBot) + (wFront - wBack);
    if (out) out[i] = d;
    if (!(ref && y == g.ny - 1)) m = fabsf(d) * scale;
  }
  if (maxbits) block_max_atomic(m, maxbits);
}

// ---- sparse dye bricks (reference mode) ------------------------------------------------------
// Most of the 192x256x192 dye grid is clear water.  Per 8x8x8 brick of the
// dye grid the predictor records whether any of its values is nonzero, and
// the resolve whether any lysed value (.y, the only channel the predictor
// reads) of its output is.  Inside a step the predictor skips a block whose
// departure points can only reach bricks without lysed dye (its result
// there is exactly +0), and the resolve skips the voxels of a block that
// sees no predictor value within one voxel and no splat (its early-out
// writes exactly zeros there).  Flags are plain stores of 1 (a race between
// writers of the same value is harmless); the launchers clear them first.
constexpr int kDyeBrick = 8;
// |centre velocity| per axis inside a step: the projection clamps the faces
// to +-2 (fluid.ts:908) and the centre is their mean (with a margin)
constexpr float kDyeSpeedBound = 2.0f * 1.0001f;
constexpr int kDyeResolveZ = 4;  // voxels per thread along z in the reference-mode resolve
__host__ __device__ __forceinline__ Grid brick_grid(const Grid& gc) {
  return Grid{(gc.nx + kDyeBrick - 1) / kDyeBrick, (gc.ny + kDyeBrick - 1) / kDyeBrick,
              (gc.nz + kDyeBrick - 1) / kDyeBrick};
}
__device__ __forceinline__ void mark_brick(const Grid& gc, uint32_t* flags, int x, int y, int z) {
  flags[brick_grid(gc).at(x / kDyeBrick, y / kDyeBrick, z / kDyeBrick)] = 1u;
}
// Whether any brick overlapping the block's voxels (x and y from the block
// index, planes zlo..zhi), widened by rx, ry, rz voxels per axis, is flagged
// (block-uniform; every thread must call it).
__device__ __forceinline__ bool block_any_brick(const Grid& gc, const uint32_t* flags, int rx, int ry, int rz,
                                                int zlo, int zhi) {
  __shared__ int any;
  const int tid = threadIdx.x + blockDim.x * threadIdx.y;
  if (tid == 0) any = 0;
  __syncthreads();
  const int x0 = max((int)(blockIdx.x * blockDim.x) - rx, 0);
  const int x1 = min((int)(blockIdx.x * blockDim.x + blockDim.x) - 1 + rx, gc.nx - 1);
  const int y0 = max((int)(blockIdx.y * blockDim.y) - ry, 0);
  const int y1 = min((int)(blockIdx.y * blockDim.y + blockDim.y) - 1 + ry, gc.ny - 1);
  const int z0 = max(zlo - rz, 0), z1 = min(zhi + rz, gc.nz - 1);
  const Grid b = brick_grid(gc);
  const int bx0 = x0 / kDyeBrick, by0 = y0 / kDyeBrick, bz0 = z0 / kDyeBrick;
  const int nbx = x1 / kDyeBrick - bx0 + 1, nby = y1 / kDyeBrick - by0 + 1, nbz = z1 / kDyeBrick - bz0 + 1;
  const int count = nbx * nby * nbz;
  for (int k = tid; k < count; k += blockDim.x * blockDim.y) {
    const int ix = k % nbx, iy = (k / nbx) % nby, iz = k / (nbx * nby);
    if (__ldg(flags + b.at(bx0 + ix, by0 + iy, bz0 + iz))) any = 1;
  }
  __syncthreads();
  return any != 0;
}
// The predictor's reach: RK2 departures move at most `speed` dt per axis in
// world units, plus one voxel for the interpolation's taps (a reach of the
// whole grid or more, or a non-finite speed, covers the whole grid).
__device__ __forceinline__ int reach_voxels(float d, int n, float size) {
  const float r = ceilf(d * (float)n / size);
  return (r < (float)n ? (int)r : n) + 1;
}
__device__ __forceinline__ bool block_reaches_dye(const Grid& gc, const StepParams& P, const uint32_t* cbrick,
                                                  float speed, int zlo, int zhi) {
  const float d = speed * P.dt;
  const int rx = reach_voxels(d, gc.nx, P.dsize[0]);
  const int ry = reach_voxels(d, gc.ny, P.dsize[1]);
  const int rz = reach_voxels(d, gc.nz, P.dsize[2]);
  return block_any_brick(gc, cbrick, rx, ry, rz, zlo, zhi);
}

// ---- CONC_PREDICT (advect.ts:28-72) -----------------------------------------------------------
template <class VS, class DS>
__device__ __forceinline__ void predict_cell(const Grid& gc, const Grid& g, const StepParams& P, int ref,
                                             const typename Vec4Of<VS>::type* __restrict__ cen,
                                             const typename Vec4Of<DS>::type* __restrict__ conc4,
                                             const DS* __restrict__ dye, DS* __restrict__ pred, DS* __restrict__ lim,
                                             uint32_t* __restrict__ pbrick, int x, int y, int z) {
  const size_t i = gc.at(x, y, z);
  const Recip3 dims = grid_recip(gc);
  const float dtv = P.dt;
  const Recip3 dom = dom_recip(P);
  const dob_v3 uvw = (v3((float)x, (float)y, (float)z) + v3(0.5f, 0.5f, 0.5f)) / dims;
  if (ref) {
    if (x == 0 || x >= gc.nx - 1 || z == 0 || z >= gc.nz - 1 || y >= gc.ny - 1) { stf(pred + i, 0.0f); return; }
    const dob_v3 v0 = sample_center(g, cen, uvw);
    const float speed2 = dot3(v0, v0);
    if (speed2 < 2.5e-5f) {
      const float pv = ld4(conc4 + i).y;
      stf(pred + i, pv);
      if (pbrick && pv != 0.0f) mark_brick(gc, pbrick, x, y, z);
      return;
    }
    dob_v3 back;
    if (speed2 < 0.012f) {
      back = clamp3(uvw - (v0 * dtv) / dom, 0.001f, 0.999f);
    } else {
      const dob_v3 mid = clamp3(uvw - (0.5f * (v0 * dtv)) / dom, 0.001f, 0.999f);
      const dob_v3 vMid = sample_center_in(g, cen, mid);
      back = clamp3(uvw - (vMid * dtv) / dom, 0.001f, 0.999f);
    }
    const Taps t = make_taps_in(gc, back.x, back.y, back.z);
    const float pv = lerp8x4(t, conc4).y;
    stf(pred + i, pv);
    if (pbrick && pv != 0.0f) mark_brick(gc, pbrick, x, y, z);
  } else {
    const dob_v3 v0 = gc.nx == g.nx ? center_at_cell(g, cen, uvw, x, y, z, i) : sample_center(g, cen, uvw);
    const dob_v3 mid = clamp3(uvw - (0.5f * (v0 * dtv)) / dom, 0.001f, 0.999f);
    const dob_v3 vMid = sample_center_in(g, cen, mid);
    const dob_v3 back = clamp3(uvw - (vMid * dtv) / dom, 0.001f, 0.999f);
    const Taps tb = make_taps_in(gc, back.x, back.y, back.z);
    if (lim) {  // also the limiter's bracket for k_dye_resolve_lim
      float c[8];
      load8(tb, dye, c);
      stf(pred + i, tri(c[0], c[1], c[2], c[3], c[4], c[5], c[6], c[7], tb));
      stf(lim + 2 * i, min8(c));
      stf(lim + 2 * i + 1, max8(c));
    } else {
      stf(pred + i, lerp8(tb, dye));
    }
  }
}

// ZP voxels per thread along z (grid z = nz / ZP): with the brick flags
// (reference mode inside a step, ZP = kDyeResolveZ) one reach test serves
// ZP planes; the closed box runs one voxel per thread.
template <class VS, class DS, int ZP>
__global__ void __launch_bounds__(256, ZP == 1 ? 8 : 4) k_conc_predict(Grid gc, Grid g, const StepParams* __restrict__ Pp, int ref,
                                                      const typename Vec4Of<VS>::type* __restrict__ cen,
                                                      const typename Vec4Of<DS>::type* __restrict__ conc4,
                                                      const DS* __restrict__ dye, DS* __restrict__ pred,
                                                      DS* __restrict__ lim, const uint32_t* __restrict__ cbrick,
                                                      uint32_t* __restrict__ pbrick,
                                                      const unsigned int* __restrict__ speedbits) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z0 = blockIdx.z * ZP;
  const int z1 = min(z0 + ZP, gc.nz);
  const StepParams& P = *Pp;
  // inside a step: a block whose departure points can only reach dye bricks
  // holding nothing but +0 (reference mode: no lysed dye) writes the zeros
  // the trace would give without tracing.  The centre velocity is bounded
  // per axis by the projection's clamp to +-2 in reference mode, by the
  // projection's own maximum (speedbits, a margin of 1e-4 for the
  // departure's rounding) in the closed box.
  if (cbrick) {
    const float speed = speedbits ? __uint_as_float(*speedbits) * 1.0001f : kDyeSpeedBound;
    if (!block_reaches_dye(gc, P, cbrick, speed, z0, z1 - 1)) {
      if (x < gc.nx && y < gc.ny)
        for (int z = z0; z < z1; ++z) {
          const size_t i = gc.at(x, y, z);
          stf(pred + i, 0.0f);
          if (lim) { stf(lim + 2 * i, 0.0f); stf(lim + 2 * i + 1, 0.0f); }
        }
      return;
    }
  }
  if (x >= gc.nx || y >= gc.ny) return;
#pragma unroll 1
  for (int z = z0; z < z1; ++z) predict_cell<VS, DS>(gc, g, P, ref, cen, conc4, dye, pred, lim, pbrick, x, y, z);
}

// ---- CONC_RESOLVE (advect.ts:81-298) ------------------------------------------------------------
template <class S>
__device__ __forceinline__ float ldcs(const Grid& gc, const S* a, int x, int y, int z) {
  return ldf(a + gc.at(dob_clampi(x, 0, gc.nx - 1), dob_clampi(y, 0, gc.ny - 1), dob_clampi(z, 0, gc.nz - 1)));
}
template <class V4>
__device__ __forceinline__ float4 ldc4v(const Grid& gc, const V4* a, int x, int y, int z) {
  return ld4(a + gc.at(dob_clampi(x, 0, gc.nx - 1), dob_clampi(y, 0, gc.ny - 1), dob_clampi(z, 0, gc.nz - 1)));
}
__device__ __forceinline__ float intact_raw(const Grid& gc, const uint32_t* s, int x, int y, int z) {
  return (float)__ldg(s + gc.at(dob_clampi(x, 0, gc.nx - 1), dob_clampi(y, 0, gc.ny - 1), dob_clampi(z, 0, gc.nz - 1))) * kSplatInv;
}

// One interior voxel of the resolve (the boundary shell and the clear-water
// early-out are the kernel's).
template <class VS, class DS>
__device__ __forceinline__ void resolve_ref_cell(const Grid& gc, const Grid& g, const StepParams& P,
                                                 const typename Vec4Of<VS>::type* __restrict__ cen,
                                                 const typename Vec4Of<DS>::type* __restrict__ conc,
                                                 const DS* __restrict__ pred, const uint32_t* __restrict__ splatI,
                                                 const uint32_t* __restrict__ splatL,
                                                 typename Vec4Of<DS>::type* __restrict__ out,
                                                 uint32_t* __restrict__ cbrick_out, int x, int y, int z) {
  const size_t i = gc.at(x, y, z);
  const dob_v3 dims = v3((float)gc.nx, (float)gc.ny, (float)gc.nz);
  const Recip3 dimr = grid_recip(gc);
  const bool inFloorZone = y <= 7;
  const uint32_t rawIntact = __ldg(splatI + i), rawLysed = __ldg(splatL + i);
  if (rawIntact == 0u && rawLysed == 0u) {
    const dob_v3 g0 = v3((float)x, (float)y, (float)z) / dimr;
    const dob_v3 g1 = (v3((float)x, (float)y, (float)z) + v3(1.0f, 1.0f, 1.0f)) / dimr;
    const float oct0 = lerp8(make_taps(gc, g0.x, g0.y, g0.z), pred);
    const float oct1 = lerp8(make_taps(gc, g1.x, g1.y, g1.z), pred);
    float bedActive = 0.0f;
    if (inFloorZone) {
      const dob_v3 gh = (v3((float)x, (float)y, (float)z) + v3(0.5f, 0.5f, 0.5f)) / dimr;
      bedActive = lerp8x4(make_taps(gc, gh.x, gh.y, gh.z), conc).w;
    }
    if (oct0 + oct1 <= 1.0e-7f && bedActive <= 1.0e-6f) {
      st4(out + i, make_float4(0.f, 0.f, 0.f, 0.f));
      return;
    }
  }
  const float gPred = ldf(pred + i);
  const float lapNeighborsG = (ldcs(gc, pred, x + 1, y, z) + ldcs(gc, pred, x - 1, y, z) + ldcs(gc, pred, x, y + 1, z) +
                               ldcs(gc, pred, x, y - 1, z) + ldcs(gc, pred, x, y, z + 1) + ldcs(gc, pred, x, y, z - 1)) *
                              (1.0f / 6.0f);
  if (!inFloorZone && rawIntact == 0u && rawLysed == 0u && gPred <= 1.2e-6f && lapNeighborsG <= 1.2e-6f) {
    st4(out + i, make_float4(0.f, 0.f, 0.f, 0.f));
    return;
  }
  float lapIntact = 0.0f;
  if (rawIntact > 0u || gPred > 8.0e-5f || lapNeighborsG > 8.0e-5f)
    lapIntact = (intact_raw(gc, splatI, x + 1, y, z) + intact_raw(gc, splatI, x - 1, y, z) + intact_raw(gc, splatI, x, y + 1, z) +
                 intact_raw(gc, splatI, x, y - 1, z) + intact_raw(gc, splatI, x, y, z + 1) + intact_raw(gc, splatI, x, y, z - 1)) *
                (1.0f / 6.0f);
  const dob_v3 uvw = (v3((float)x, (float)y, (float)z) + v3(0.5f, 0.5f, 0.5f)) / dimr;
  const float dtv = P.dt;
  const Recip3 dom = dom_recip(P);
  const dob_v3 pw = to_world(P, uvw);
  const float halfXZ = P.U[52], yMin = P.U[53];
  const dob_v3 v0 = sample_center(g, cen, uvw);
  const dob_v3 uvwMid = clamp3(uvw - (0.5f * (v0 * dtv)) / dom, 0.001f, 0.999f);
  const dob_v3 vMid = sample_center_in(g, cen, uvwMid);
  const dob_v3 uvwBack = clamp3(uvw - (vMid * dtv) / dom, 0.001f, 0.999f);
  const dob_v3 uvwFwd = clamp3(uvw + (v0 * dtv) / dom, 0.001f, 0.999f);
  const float gBackEst = lerp8(make_taps_in(gc, uvwFwd.x, uvwFwd.y, uvwFwd.z), pred);
  const float4 orig = ld4(conc + i);
  const float gOrig = orig.y;
  const float gCorr = gPred + (0.45f * P.U[47]) * (gOrig - gBackEst);
  const dob_v3 tc = uvwBack * dims - v3(0.5f, 0.5f, 0.5f);
  const int bx = (int)floorf(tc.x), by = (int)floorf(tc.y), bz = (int)floorf(tc.z);
  const float s000 = ldc4v(gc, conc, bx, by, bz).y, s100 = ldc4v(gc, conc, bx + 1, by, bz).y;
  const float s010 = ldc4v(gc, conc, bx, by + 1, bz).y, s110 = ldc4v(gc, conc, bx + 1, by + 1, bz).y;
  const float s001 = ldc4v(gc, conc, bx, by, bz + 1).y, s101 = ldc4v(gc, conc, bx + 1, by, bz + 1).y;
  const float s011 = ldc4v(gc, conc, bx, by + 1, bz + 1).y, s111 = ldc4v(gc, conc, bx + 1, by + 1, bz + 1).y;
  const float minG = dob_minf(dob_minf(dob_minf(s000, s100), dob_minf(s010, s110)), dob_minf(dob_minf(s001, s101), dob_minf(s011, s111)));
  const float maxG = dob_maxf(dob_maxf(dob_maxf(s000, s100), dob_maxf(s010, s110)), dob_maxf(dob_maxf(s001, s101), dob_maxf(s011, s111)));
  float cLysed = dob_clampf(gCorr, minG, maxG);
  const float diffBlend = dob_clampf(dtv * 5.60f, 0.0f, 0.105f);
  cLysed = dob_mix(cLysed, lapNeighborsG, diffBlend);
  const float upperDilute = dob_exp(-dtv * dob_mix(0.016f, 0.034f, dob_smoothstep(yMin + 0.045f, yMin + 0.26f, pw.y)));
  cLysed = cLysed * upperDilute;
  const float dmTransfer = (float)rawLysed * kSplatInv;
  const float floorBedCapture = 1.0f - dob_smoothstep(yMin + 0.018f, yMin + 0.058f, pw.y);
  cLysed = cLysed + dmTransfer * (1.0f - floorBedCapture * 0.72f);
  if (cLysed < 2.5e-6f) cLysed = 0.0f;
  const float rHoriz = length2f(pw.x, pw.z);
  float cBed = 0.0f;
  if (inFloorZone) {
    const float bCenter = orig.w;
    const float bHoriz = 0.25f * (ldc4v(gc, conc, x + 1, y, z).w + ldc4v(gc, conc, x - 1, y, z).w +
                                  ldc4v(gc, conc, x, y, z + 1).w + ldc4v(gc, conc, x, y, z - 1).w);
    const float bAbove = ldc4v(gc, conc, x, y + 1, z).w;
    const float bBelow = ldc4v(gc, conc, x, max(0, y - 1), z).w;
    const float spreadAlpha = dob_clampf(dtv * (3.20f + 6.50f * dob_minf(bCenter, 0.65f)), 0.0f, 0.165f);
    const float vertDiffuse = dob_clampf(dtv * 0.75f, 0.0f, 0.026f);
    const float settleAlpha = dob_clampf(dtv * 2.80f, 0.0f, 0.090f);
    const float bedDecay = dob_exp(-dtv * dob_mix(0.095f, 0.28f, dob_smoothstep(halfXZ * 0.35f, halfXZ * 0.78f, rHoriz)));
    const float drainedSelf = (y == 0 ? bCenter : bCenter * (1.0f - settleAlpha)) * bedDecay;
    const float settledFromAbove = y >= 7 ? 0.0f : bAbove * settleAlpha;
    const float advectedBed = drainedSelf + settledFromAbove;
    const float smoothedBed = dob_mix(dob_mix(advectedBed, bHoriz, spreadAlpha), 0.5f * (bAbove + bBelow), vertDiffuse);
    const float topBedFade = 1.0f - 0.38f * dob_smoothstep(3.5f, 7.0f, (float)y);
    cBed = (smoothedBed + dmTransfer * floorBedCapture * 0.68f) * topBedFade;
    if (cBed < 1.0e-6f) cBed = 0.0f;
  }
  const float wallSponge = 1.0f - dob_smoothstep(halfXZ * 0.68f, halfXZ * 0.94f, rHoriz);
  const float floorRadialTaper = 1.0f - dob_smoothstep(halfXZ * 0.52f, halfXZ * 0.88f, rHoriz);
  const float maxBedProfile = 0.54f * dob_exp(-0.56f * (float)y) * floorRadialTaper;
  cBed = dob_minf(cBed * wallSponge, maxBedProfile);
  const float cParcelRaw = (float)rawIntact * kSplatInv;
  const float shoulderFeather = rawIntact > 0u ? 0.36f : 0.18f;
  const float cParcelIntact = dob_mix(cParcelRaw, lapIntact, shoulderFeather) * wallSponge;
  const float cIntact = cParcelIntact + cBed;
  cLysed = cLysed * wallSponge;
  const float cTotal = cIntact + cLysed;
  float vOx = 0.0f;
  if (cTotal > 1.0e-5f) {
    const float fLysis = dob_clampf(cLysed / dob_maxf(cTotal, 1.0e-5f), 0.0f, 1.0f);
    const float intactFrac = 1.0f - fLysis;
    const float bedFrac = dob_smoothstep(0.0f, 0.85f, cBed / dob_maxf(cTotal, 1.0e-5f));
    const float flowSpeed = length3(v0);
    const float convShear = length3(v0 - vMid) / dob_maxf(0.5f * dtv, 1.0e-3f);
    const float shearDispersion = dob_smoothstep(0.014f, 0.135f, flowSpeed + 0.38f * convShear);
    const float thinIntactSheet = (1.0f - dob_smoothstep(0.024f, 0.24f, cIntact)) * dob_smoothstep(0.0006f, 0.0065f, cIntact);
    const float activeSheet = thinIntactSheet * (0.38f + 0.62f * shearDispersion) * intactFrac;
    const float rawOx = dob_clampf(0.08f + 0.62f * activeSheet + 0.36f * shearDispersion * intactFrac, 0.0f, 1.0f);
    vOx = rawOx * (1.0f - 0.82f * bedFrac);
  }
  st4(out + i, make_float4(cIntact, cLysed, vOx, cBed));
  if (cLysed != 0.0f) mark_brick(gc, cbrick_out, x, y, z);
}

// Each thread resolves kDyeResolveZ voxels along z: their splat sums are
// loaded before the block's brick test, so in clear water (most of the dye
// grid) the flag loads, the barrier and the splat loads overlap and one
// test serves kDyeResolveZ planes; the voxels that need the full resolve
// then run it one after another.
template <class VS, class DS>
__global__ void __launch_bounds__(256, 3) k_conc_resolve_ref(Grid gc, Grid g, const StepParams* __restrict__ Pp,
                                                          const typename Vec4Of<VS>::type* __restrict__ cen,
                                                          const typename Vec4Of<DS>::type* __restrict__ conc,
                                                          const DS* __restrict__ pred,
                                                          const uint32_t* __restrict__ splatI,
                                                          const uint32_t* __restrict__ splatL,
                                                          typename Vec4Of<DS>::type* __restrict__ out,
                                                          const uint32_t* __restrict__ pbrick,
                                                          uint32_t* __restrict__ cbrick_out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z0 = blockIdx.z * kDyeResolveZ;
  const bool inside = x < gc.nx && y < gc.ny;
  uint32_t rI[kDyeResolveZ], rL[kDyeResolveZ];
#pragma unroll
  for (int k = 0; k < kDyeResolveZ; ++k) {
    const bool ok = inside && z0 + k < gc.nz;
    const size_t i = ok ? gc.at(x, y, z0 + k) : 0;
    rI[k] = ok ? __ldg(splatI + i) : 0u;
    rL[k] = ok ? __ldg(splatL + i) : 0u;
  }
  // inside a step: no predictor value within one voxel of the block
  const bool clear = pbrick && !block_any_brick(gc, pbrick, 1, 1, 1, z0, z0 + kDyeResolveZ - 1);
  if (!inside) return;
  const bool shellXY = x == 0 || x >= gc.nx - 1 || y >= gc.ny - 1;
  const bool inFloorZone = y <= 7;
  unsigned need = 0u;
#pragma unroll
  for (int k = 0; k < kDyeResolveZ; ++k) {
    const int z = z0 + k;
    if (z >= gc.nz) break;
    // the boundary shell, and clear water's early-out (every predictor tap
    // +0, so oct0 = oct1 = 0 below) outside the floor zone
    if (shellXY || z == 0 || z >= gc.nz - 1 || (clear && !inFloorZone && rI[k] == 0u && rL[k] == 0u))
      st4(out + gc.at(x, y, z), make_float4(0.f, 0.f, 0.f, 0.f));
    else
      need |= 1u << k;
  }
  const StepParams& P = *Pp;
  while (need) {
    const int k = __ffs(need) - 1;
    need &= need - 1u;
    resolve_ref_cell<VS, DS>(gc, g, P, cen, conc, pred, splatI, splatL, out, cbrick_out, x, y, z0 + k);
  }
}

// Closed box: MacCormack correction of the single dye, 8-tap min/max limiter.
template <class VS, class DS>
__global__ void __launch_bounds__(256) k_dye_resolve_box(Grid gc, Grid g, const StepParams* __restrict__ Pp,
                                                         const typename Vec4Of<VS>::type* __restrict__ cen,
                                                         const DS* __restrict__ dye, const DS* __restrict__ pred,
                                                         DS* __restrict__ out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= gc.nx || y >= gc.ny) return;
  const size_t i = gc.at(x, y, z);
  const StepParams& P = *Pp;
  const float dtv = P.dt;
  const Recip3 dom = dom_recip(P);
  const dob_v3 uvw = (v3((float)x, (float)y, (float)z) + v3(0.5f, 0.5f, 0.5f)) / grid_recip(gc);
  const dob_v3 v0 = gc.nx == g.nx ? center_at_cell(g, cen, uvw, x, y, z, i) : sample_center(g, cen, uvw);
  const dob_v3 uvwMid = clamp3(uvw - (0.5f * (v0 * dtv)) / dom, 0.001f, 0.999f);
  const dob_v3 vMid = sample_center_in(g, cen, uvwMid);
  const dob_v3 uvwBack = clamp3(uvw - (vMid * dtv) / dom, 0.001f, 0.999f);
  const dob_v3 uvwFwd = clamp3(uvw + (v0 * dtv) / dom, 0.001f, 0.999f);
  const float gBackEst = lerp8(make_taps_in(gc, uvwFwd.x, uvwFwd.y, uvwFwd.z), pred);
  const float gOrig = ldf(dye + i);
  // one explicit FMA, so the step's and the stage's resolve (and the
  // adjoint's replay of it) round the correction alike
  const float gCorr = __fmaf_rn(0.45f * P.sharp, gOrig - gBackEst, ldf(pred + i));
  // the limiter's bracket: the 8 dye taps around the departure point (the
  // predictor's taps)
  float c[8];
  load8(make_taps_in(gc, uvwBack.x, uvwBack.y, uvwBack.z), dye, c);
  stf(out + i, dob_clampf(gCorr, min8(c), max8(c)));
}

// The same resolve in the step: the predictor (k_conc_predict with `lim`)
// has already bracketed its 8 taps, so only the forward sample is traced.
// cbrick_out (the flags of `out`): a brick is marked when it receives a
// value whose bits are not those of +0.
template <class VS, class DS>
__global__ void __launch_bounds__(256, 8) k_dye_resolve_lim(Grid gc, Grid g, const StepParams* __restrict__ Pp,
                                                         const typename Vec4Of<VS>::type* __restrict__ cen,
                                                         const DS* __restrict__ dye, const DS* __restrict__ pred,
                                                         const DS* __restrict__ lim, DS* __restrict__ out,
                                                         uint32_t* __restrict__ cbrick_out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= gc.nx || y >= gc.ny) return;
  const size_t i = gc.at(x, y, z);
  // A bracket of two zeros clamps every correction to its upper end: min(max(g,
  // lo), hi) is hi whenever lo and hi are zeros of either sign (max gives g > 0
  // or lo, min of either with hi is hi), so the trace is not needed.
  const float lo = ldf(lim + 2 * i), hi = ldf(lim + 2 * i + 1);
  if (lo == 0.0f && hi == 0.0f) {
    stf(out + i, hi);
    if (cbrick_out && __float_as_uint(hi) != 0u) mark_brick(gc, cbrick_out, x, y, z);
    return;
  }
  const StepParams& P = *Pp;
  const float dtv = P.dt;
  const Recip3 dom = dom_recip(P);
  const dob_v3 uvw = (v3((float)x, (float)y, (float)z) + v3(0.5f, 0.5f, 0.5f)) /
                     grid_recip(gc);
  const dob_v3 v0 = gc.nx == g.nx ? center_at_cell(g, cen, uvw, x, y, z, i) : sample_center(g, cen, uvw);
  const dob_v3 uvwFwd = clamp3(uvw + (v0 * dtv) / dom, 0.001f, 0.999f);
  const float gBackEst = lerp8(make_taps_in(gc, uvwFwd.x, uvwFwd.y, uvwFwd.z), pred);
  const float gOrig = ldf(dye + i);
  // one explicit FMA, so the step's and the stage's resolve (and the
  // adjoint's replay of it) round the correction alike
  const float gCorr = __fmaf_rn(0.45f * P.sharp, gOrig - gBackEst, ldf(pred + i));
  const float r = dob_clampf(gCorr, lo, hi);
  stf(out + i, r);
  if (cbrick_out && __float_as_uint(r) != 0u) mark_brick(gc, cbrick_out, x, y, z);
}

// ---- host launchers ------------------------------------------------------------------------------
static inline dim3 cell_grid(const Grid& g) { return dim3((g.nx + 31) / 32, (g.ny + 7) / 8, g.nz); }
static inline dim3 cell_block() { return dim3(32, 8, 1); }



void launch_init_vel(const DevState& s, cudaStream_t st) {
  DOB_VEL_DISPATCH(s.prec, {
    k_init_vel<VS><<<cell_grid(s.g), cell_block(), 0, st>>>(s.g, s.params, (VS*)s.u, (VS*)s.v, (VS*)s.w,
                                                            (typename Vec4Of<VS>::type*)s.cen,
                                                            (typename Vec4Of<VS>::type*)s.curl);
  });
}

void launch_advect_mac(const DevState& s, cudaStream_t st) {
  DOB_VEL_DISPATCH(s.prec, {
    k_advect_mac<VS><<<cell_grid(s.g), cell_block(), 0, st>>>(
        s.g, s.params, s.ref, s.flags, (const VS*)s.u, (const VS*)s.v, (const VS*)s.w,
        (const typename Vec4Of<VS>::type*)s.cen, s.wave, (VS*)s.u2, (VS*)s.v2, (VS*)s.w2);
  });
}

void launch_mac_to_center(const DevState& s, cudaStream_t st) {
  DOB_VEL_DISPATCH(s.prec, {
    k_mac_to_center<VS><<<cell_grid(s.g), cell_block(), 0, st>>>(s.g, s.params, s.ref, s.flags, (const VS*)s.u,
                                                                 (const VS*)s.v, (const VS*)s.w,
                                                                 (typename Vec4Of<VS>::type*)s.cen);
  });
}

void launch_curl(const DevState& s, cudaStream_t st) {
  DOB_VEL_DISPATCH(s.prec, {
    k_curl<VS><<<cell_grid(s.g), cell_block(), 0, st>>>(s.g, (const typename Vec4Of<VS>::type*)s.cen,
                                                        (typename Vec4Of<VS>::type*)s.curl);
  });
}

void launch_casson(const DevState& s, cudaStream_t st) {
  DOB_VEL_DISPATCH(s.prec, {
    k_casson<VS, DS><<<cell_grid(s.g), cell_block(), 0, st>>>(
        s.g, s.gc, s.params, s.ref, s.flags, (const VS*)s.u, (const VS*)s.v, (const VS*)s.w,
        (const typename Vec4Of<VS>::type*)s.curl, (const typename Vec4Of<DS>::type*)s.conc, (const DS*)s.conc,
        (VS*)s.u2, (VS*)s.v2, (VS*)s.w2);
  });
}

void launch_mac_rhs(const DevState& s, cudaStream_t st) {
  DOB_VEL_DISPATCH(s.prec, {
    k_mac_rhs<VS><<<cell_grid(s.g), cell_block(), 0, st>>>(s.g, s.params, s.ref, (const VS*)s.u, (const VS*)s.v,
                                                           (const VS*)s.w, s.wave, s.rhs, nullptr);
  });
  if (!s.ref) {  // compatibility of the pure-Neumann problem: zero-mean right-hand side
    launch_sum(s.rhs, s.g.n(), s.part + PART_RHS * kSumBlocks, s.num_sms, st);
    launch_sub_mean(s.rhs, s.g.n(), s.part + PART_RHS * kSumBlocks, s.num_sms, st);
  }
}

void launch_project(const DevState& s, cudaStream_t st) {
  DOB_VEL_DISPATCH(s.prec, {
    k_project<VS><<<cell_grid(s.g), cell_block(), 0, st>>>(s.g, s.params, s.ref, (VS*)s.u, (VS*)s.v, (VS*)s.w, s.p,
                                                           s.plo, s.wave);
  });
}

void launch_project_center_ref(const DevState& s, cudaStream_t st) {
  DOB_VEL_DISPATCH(s.prec, {
    k_project_center_ref<VS><<<cell_grid(s.g), cell_block(), 0, st>>>(
        s.g, s.params, s.flags, (const VS*)s.u, (const VS*)s.v, (const VS*)s.w, s.p, s.plo, s.wave, (VS*)s.u2,
        (VS*)s.v2, (VS*)s.w2, (typename Vec4Of<VS>::type*)s.cen);
  });
}

void launch_divergence(const DevState& s, float* out, float scale, unsigned int* maxbits, cudaStream_t st) {
  DOB_VEL_DISPATCH(s.prec, {
    k_divergence<VS><<<cell_grid(s.g), cell_block(), 0, st>>>(s.g, s.ref, (const VS*)s.u, (const VS*)s.v,
                                                              (const VS*)s.w, out, scale, maxbits);
  });
}

// the dye-brick flags of one of the context's two dye buffers (none for
// other dye arrays, such as the adjoint's tape)
static uint32_t* brick_flags_of(const DevState& s, const void* conc) {
  return conc == s.concA ? s.cbrickA : conc == s.concB ? s.cbrickB : nullptr;
}
void launch_dye_bricks_unknown(const DevState& s, cudaStream_t st) {
  const size_t nb = brick_grid(s.gc).n() * sizeof(uint32_t);
  if (s.cbrickA) cudaMemsetAsync(s.cbrickA, 1, nb, st);
  if (s.cbrickB) cudaMemsetAsync(s.cbrickB, 1, nb, st);
}
size_t dye_brick_count(const Grid& gc) { return brick_grid(gc).n(); }

void launch_conc_predict(const DevState& s, cudaStream_t st, bool bracket, bool sparse) {
  uint32_t* pb = s.ref ? s.pbrick : nullptr;
  if (pb) cudaMemsetAsync(pb, 0, brick_grid(s.gc).n() * sizeof(uint32_t), st);
  const uint32_t* cb = sparse ? brick_flags_of(s, s.conc) : nullptr;
  DOB_VEL_DISPATCH(s.prec, {
    if (cb && s.ref) {
      dim3 gr = cell_grid(s.gc);
      gr.z = (s.gc.nz + kDyeResolveZ - 1) / kDyeResolveZ;
      k_conc_predict<VS, DS, kDyeResolveZ><<<gr, cell_block(), 0, st>>>(
          s.gc, s.g, s.params, s.ref, (const typename Vec4Of<VS>::type*)s.cen,
          (const typename Vec4Of<DS>::type*)s.conc, (const DS*)s.conc, (DS*)s.pred, nullptr, cb, pb, nullptr);
    } else {
      // the closed box's bound on the centre velocity comes from the projection
      k_conc_predict<VS, DS, 1><<<cell_grid(s.gc), cell_block(), 0, st>>>(
          s.gc, s.g, s.params, s.ref, (const typename Vec4Of<VS>::type*)s.cen,
          (const typename Vec4Of<DS>::type*)s.conc, (const DS*)s.conc, (DS*)s.pred,
          bracket && !s.ref ? (DS*)s.lim : nullptr, cb, pb, cb ? s.redu + REDU_SPEED : nullptr);
    }
  });
}

void launch_dye_resolve_lim(const DevState& s, cudaStream_t st) {
  uint32_t* cb = brick_flags_of(s, s.conc2);
  if (cb) cudaMemsetAsync(cb, 0, brick_grid(s.gc).n() * sizeof(uint32_t), st);
  DOB_VEL_DISPATCH(s.prec, {
    k_dye_resolve_lim<VS, DS><<<cell_grid(s.gc), cell_block(), 0, st>>>(
        s.gc, s.g, s.params, (const typename Vec4Of<VS>::type*)s.cen, (const DS*)s.conc, (const DS*)s.pred,
        (const DS*)s.lim, (DS*)s.conc2, cb);
  });
}

void launch_conc_resolve(const DevState& s, cudaStream_t st, bool sparse) {
  uint32_t* cb = brick_flags_of(s, s.conc2);
  // reference mode: the resolve rewrites its output's flags; the closed box's
  // tracing resolve does not, so its output's flags say "may hold dye"
  if (cb) cudaMemsetAsync(cb, s.ref ? 0 : 1, brick_grid(s.gc).n() * sizeof(uint32_t), st);
  DOB_VEL_DISPATCH(s.prec, {
    if (s.ref) {
      dim3 gr = cell_grid(s.gc);
      gr.z = (s.gc.nz + kDyeResolveZ - 1) / kDyeResolveZ;
      k_conc_resolve_ref<VS, DS><<<gr, cell_block(), 0, st>>>(
          s.gc, s.g, s.params, (const typename Vec4Of<VS>::type*)s.cen, (const typename Vec4Of<DS>::type*)s.conc,
          (const DS*)s.pred, s.splatI, s.splatL, (typename Vec4Of<DS>::type*)s.conc2, sparse ? s.pbrick : nullptr,
          cb);
    } else {
      k_dye_resolve_box<VS, DS><<<cell_grid(s.gc), cell_block(), 0, st>>>(
          s.gc, s.g, s.params, (const typename Vec4Of<VS>::type*)s.cen, (const DS*)s.conc, (const DS*)s.pred,
          (DS*)s.conc2);
    }
  });
}

}  // namespace dob
