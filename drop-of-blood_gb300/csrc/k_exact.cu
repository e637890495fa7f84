// k_exact.cu — kernels whose results must be reproducible bit for bit by a
// host build of the same arithmetic: Lagrangian parcel emission, advection
// and fixed-point splatting (particles.ts:53-462), sphere injection, and the
// device evaluation of the library's elementary functions.
//
// This translation unit is compiled with -fmad=false (no multiply-add
// contraction) and uses only IEEE-rounded + - * / sqrt, floor/rint and the
// library's own transcendentals, so a parcel's position, and therefore its
// splat cell (floor(uvw * dims - 0.5), particles.ts:239-247), is the same on
// the host and the device for the same inputs.  Splat sums are unsigned
// integer atomics: their order does not change the result.  DOB_UNFUSED
// keeps the shared sampling helpers in that unfused form here.
#define DOB_UNFUSED 1
#include "dob_kernels.cuh"

namespace dob {

// Mark the 8x8x8 brick of dye voxel (x, y, z) as holding a splat: a plain
// store of 1 (writers of the same value may race harmlessly), left out when
// the flag already reads 1 (most splats land in bricks already marked, and
// a stale 0 only costs a redundant store).
__device__ __forceinline__ void mark_splat(const Grid& gc, uint32_t* sbrick, int x, int y, int z) {
  if (!sbrick) return;
  const int bnx = (gc.nx + 7) >> 3, bny = (gc.ny + 7) >> 3;
  uint32_t* f = sbrick + ((z >> 3) * bny + (y >> 3)) * bnx + (x >> 3);
  if (*f == 0u) *f = 1u;
}
__device__ __forceinline__ void splat_trilinear(const Grid& gc, uint32_t* dst, dob_v3 uvw, float mass, float minMass,
                                                uint32_t* sbrick) {
  if (mass <= minMass) return;
  const dob_v3 dims = v3((float)gc.nx, (float)gc.ny, (float)gc.nz);
  const dob_v3 coord = uvw * dims - v3(0.5f, 0.5f, 0.5f);
  const int bx = (int)floorf(coord.x), by = (int)floorf(coord.y), bz = (int)floorf(coord.z);
  const dob_v3 f = clamp3(coord - v3((float)bx, (float)by, (float)bz), 0.0f, 1.0f);
  const dob_v3 omf = v3(1.0f, 1.0f, 1.0f) - f;
  const int x0 = dob_clampi(bx, 0, gc.nx - 1), y0 = dob_clampi(by, 0, gc.ny - 1), z0 = dob_clampi(bz, 0, gc.nz - 1);
  const int x1 = dob_clampi(bx + 1, 0, gc.nx - 1), y1 = dob_clampi(by + 1, 0, gc.ny - 1), z1 = dob_clampi(bz + 1, 0, gc.nz - 1);
  const float scale = mass * kSplatScale;
  const uint32_t w000 = (uint32_t)rintf(scale * omf.x * omf.y * omf.z);
  const uint32_t w100 = (uint32_t)rintf(scale * f.x * omf.y * omf.z);
  const uint32_t w010 = (uint32_t)rintf(scale * omf.x * f.y * omf.z);
  const uint32_t w110 = (uint32_t)rintf(scale * f.x * f.y * omf.z);
  const uint32_t w001 = (uint32_t)rintf(scale * omf.x * omf.y * f.z);
  const uint32_t w101 = (uint32_t)rintf(scale * f.x * omf.y * f.z);
  const uint32_t w011 = (uint32_t)rintf(scale * omf.x * f.y * f.z);
  const uint32_t w111 = (uint32_t)rintf(scale * f.x * f.y * f.z);
  if (w000 > 0u) atomicAdd(dst + gc.at(x0, y0, z0), w000);
  if (w100 > 0u) atomicAdd(dst + gc.at(x1, y0, z0), w100);
  if (w010 > 0u) atomicAdd(dst + gc.at(x0, y1, z0), w010);
  if (w110 > 0u) atomicAdd(dst + gc.at(x1, y1, z0), w110);
  if (w001 > 0u) atomicAdd(dst + gc.at(x0, y0, z1), w001);
  if (w101 > 0u) atomicAdd(dst + gc.at(x1, y0, z1), w101);
  if (w011 > 0u) atomicAdd(dst + gc.at(x0, y1, z1), w011);
  if (w111 > 0u) atomicAdd(dst + gc.at(x1, y1, z1), w111);
  // the eight taps are the corners x0|x1 x y0|y1 x z0|z1: mark each distinct
  // brick among them once (usually all eight share one)
  if (sbrick && (w000 | w100 | w010 | w110 | w001 | w101 | w011 | w111)) {
    const bool dx = (x0 >> 3) != (x1 >> 3), dy = (y0 >> 3) != (y1 >> 3), dz = (z0 >> 3) != (z1 >> 3);
    mark_splat(gc, sbrick, x0, y0, z0);
    if (dx) mark_splat(gc, sbrick, x1, y0, z0);
    if (dy) mark_splat(gc, sbrick, x0, y1, z0);
    if (dx && dy) mark_splat(gc, sbrick, x1, y1, z0);
    if (dz) {
      mark_splat(gc, sbrick, x0, y0, z1);
      if (dx) mark_splat(gc, sbrick, x1, y0, z1);
      if (dy) mark_splat(gc, sbrick, x0, y1, z1);
      if (dx && dy) mark_splat(gc, sbrick, x1, y1, z1);
    }
  }
}

__device__ __forceinline__ float azim_modes(float theta, float seed) {
  return 1.0f + 0.036f * dob_cos(4.0f * theta + seed * 1.73f) + 0.026f * dob_cos(6.0f * theta - seed * 2.31f) +
         0.018f * dob_sin(8.0f * theta + seed * 0.89f);
}

// hash33 (common.ts:79-83)
__device__ __forceinline__ dob_v3 hash33(dob_v3 p3in) {
  dob_v3 p3 = v3(dob_fract(p3in.x * 0.1031f), dob_fract(p3in.y * 0.1030f), dob_fract(p3in.z * 0.0973f));
  const float dd = dot3(p3, v3(p3.y + 33.33f, p3.x + 33.33f, p3.z + 33.33f));
  p3 = v3(p3.x + dd, p3.y + dd, p3.z + dd);
  const dob_v3 a = v3(p3.x + p3.y, p3.x + p3.x, p3.y + p3.x);
  const dob_v3 b = v3(p3.z, p3.y, p3.x);
  const dob_v3 q = a * b;
  return v3(dob_fract(q.x), dob_fract(q.y), dob_fract(q.z));
}

// ---- PARTICLE_EMIT (particles.ts:53-181) ---------------------------------------------
__global__ void __launch_bounds__(256) k_parcel_emit(Grid gc, const StepParams* __restrict__ Pp, float4* parcels,
                                                     uint32_t cap, const float4* __restrict__ wave,
                                                     uint32_t* __restrict__ splatL, uint32_t* __restrict__ sbrick) {
  const StepParams& P = *Pp;
  const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t spawnCount = P.spawn_count;
  if (gid >= spawnCount) return;
  float totalDrain = 0.0f;
  for (int d = 0; d < kMaxDrops; ++d)
    if (drop(P, d, 7) > 0.0f && drop(P, d, 6) > 0.0001f) totalDrain = totalDrain + drop(P, d, 6);
  if (totalDrain <= 1e-6f) return;
  const float targetFrac = ((float)gid + 0.5f) / (float)(spawnCount > 1u ? spawnCount : 1u) * totalDrain;
  float accum = 0.0f;
  int chosen = 0;
  for (int d = 0; d < kMaxDrops; ++d) {
    if (drop(P, d, 7) > 0.0f && drop(P, d, 6) > 0.0001f) {
      accum = accum + drop(P, d, 6);
      chosen = d;
      if (accum >= targetFrac) break;
    }
  }
  const float dX = drop(P, chosen, 0), dY = drop(P, chosen, 1), dZ = drop(P, chosen, 2), dRad = drop(P, chosen, 3);
  const float dDrain = drop(P, chosen, 6);
  const float seed = dob_maxf(drop(P, chosen, 7), 0.5f);
  const float surfY = P.U[40];
  const uint32_t ringIdx = (uint32_t)(((uint64_t)P.cursor + gid) % cap);
  const float4 o0 = parcels[2 * (size_t)ringIdx];
  if (o0.w > 1e-6f) {
    const dob_v3 settle = o0.y < surfY - 0.32f ? v3(o0.x, P.U[53] + 0.012f, o0.z) : v3(o0.x, o0.y, o0.z);
    const dob_v3 oldUvw = to_uvw(P, settle);
    if (oldUvw.x > 0.002f && oldUvw.y > 0.002f && oldUvw.z > 0.002f && oldUvw.x < 0.998f && oldUvw.y < 0.998f &&
        oldUvw.z < 0.998f) {
      const dob_v3 cd = oldUvw * v3((float)gc.nx, (float)gc.ny, (float)gc.nz);
      const int cx = dob_clampi((int)floorf(cd.x), 0, gc.nx - 1), cy = dob_clampi((int)floorf(cd.y), 0, gc.ny - 1),
                cz = dob_clampi((int)floorf(cd.z), 0, gc.nz - 1);
      const uint32_t fpOld = (uint32_t)rintf(o0.w * kSplatScale);
      if (fpOld > 0u) {
        atomicAdd(splatL + gc.at(cx, cy, cz), fpOld);
        mark_splat(gc, sbrick, cx, cy, cz);
      }
    }
  }
  const float seqIdx = (float)ringIdx + seed * 137.0f;
  const dob_v3 hsh = hash33(v3((float)gid, P.U[35] * 60.0f, seed));
  const dob_v3 r3 = v3(dob_fract(seqIdx * 0.8191725134f + hsh.x * 0.032f), dob_fract(seqIdx * 0.6710436067f + hsh.y * 0.032f),
                       dob_fract(seqIdx * 0.5497004779f + hsh.z * 0.032f));
  const float theta = 6.28318530718f * r3.x;
  const float azim = azim_modes(theta, seed);
  const float rDrop = dob_maxf(dRad, 0.010f);
  const float emergNorm = (dY - surfY) / dob_maxf(rDrop, 0.018f);
  const float nascentCoreFill = dob_smoothstep(-0.32f, 0.18f, emergNorm);
  const float slugWeight = dob_smoothstep(0.26f, 0.85f, dDrain);
  const float wakeThin = dob_mix(0.46f, 1.0f, dob_smoothstep(0.018f, 0.26f, dDrain));
  const float rNeck = dob_mix(0.013f * wakeThin, dob_clampf(rDrop * 0.84f + 0.014f, 0.020f, 0.056f), slugWeight) * azim;
  const float innerRing = 0.37f * slugWeight;
  const bool isCapVeil = slugWeight > 0.08f && r3.z < 0.16f;
  const float radFracAnnular = dob_mix(innerRing, 1.0f, dob_pow(r3.y, dob_mix(0.50f, 0.44f, slugWeight)));
  const float radFracCap = dob_mix(0.14f * slugWeight, dob_maxf(innerRing * 1.32f, 0.08f), dob_sqrt(r3.y));
  const float radFracTorus = isCapVeil ? radFracCap : radFracAnnular;
  const float radFrac = dob_mix(radFracTorus, dob_sqrt(r3.y), nascentCoreFill * 0.82f);
  const float r = rNeck * radFrac;
  const float wakeDriftAngle = P.U[35] * 1.85f + seed * 3.17f;
  const float driftS = 0.0038f * (1.0f - slugWeight) * (1.0f - wakeThin * 0.45f);
  const float wdx = dob_cos(wakeDriftAngle) * driftS, wdz = dob_sin(wakeDriftAngle * 0.83f + seed) * driftS;
  const float ct = dob_cos(theta), stt = dob_sin(theta);
  const float posX = dX + wdx + ct * r, posZ = dZ + wdz + stt * r;
  const float4 ws = sample_wave(wave, posX, posZ, 0.002f, 0.998f);
  const float localEta = dob_clampf(ws.x, -0.085f, 0.015f);
  const float neckTopY = surfY + dob_minf(0.0f, localEta) - 0.0038f;
  const float cavitySag = (1.0f - radFrac * radFrac) * (0.0085f * slugWeight + 0.0045f * nascentCoreFill);
  const float zStrat =
      isCapVeil ? r3.z * 3.6f : (r3.z - 0.16f * slugWeight) / dob_maxf(1.0f - 0.16f * slugWeight, 0.5f);
  const float posY = neckTopY - cavitySag - dob_mix(0.0014f, 0.0135f, dob_clampf(zStrat, 0.0f, 1.0f));
  const float smallDropFragility = 1.0f - dob_smoothstep(0.022f, 0.056f, rDrop);
  const float rimExposure = dob_smoothstep(0.58f, 1.0f, radFrac);
  const float initLysis =
      dob_clampf(0.14f * rimExposure + 0.28f * smallDropFragility * (0.45f + 0.55f * radFrac), 0.0f, 0.44f);
  const float rf = dob_maxf(radFrac, 0.25f);
  const dob_v3 tangentDir = v3(-stt * rf, -0.80f, ct * rf);
  const dob_v3 initStretch = normalize3(tangentDir) * 0.0036f;
  parcels[2 * (size_t)ringIdx] = make_float4(posX, posY, posZ, kParcelMass);
  parcels[2 * (size_t)ringIdx + 1] = make_float4(initStretch.x, initStretch.y, initStretch.z, initLysis);
}

// ---- sampleVelWorld (particles.ts:201-232) ---------------------------------------------
template <class V4>
__device__ __forceinline__ dob_v3 sample_vel_world(const Grid& g, const StepParams& P, const V4* cen, dob_v3 pp,
                                                   float rouleauxMaturity, float meniscusHold) {
  const float depth = P.U[40] - pp.y;
  const dob_v3 uvw = clamp3(to_uvw(P, pp), 0.002f, 0.998f);
  const float settleGate = dob_mix(0.38f, 1.0f, dob_smoothstep(0.002f, 0.055f, depth));
  const float rouleauxFall = dob_mix(0.020f, 0.046f, dob_smoothstep(0.04f, 0.42f, depth));
  const float monoSettle = rouleauxFall * settleGate;
  const float stackSettle = dob_mix(0.032f, 0.062f, dob_smoothstep(0.04f, 0.48f, depth));
  const float surfTailHold = meniscusHold * (1.0f - dob_smoothstep(0.003f, 0.034f, dob_maxf(0.0f, depth)));
  const float effSettle = dob_mix(monoSettle, stackSettle, rouleauxMaturity) * dob_mix(1.0f, 0.035f, surfTailHold);
  const float deepUnfurl = dob_smoothstep(0.035f, 0.24f, depth);
  dob_v3 sub = v3(0.0f, 0.0f, 0.0f);
  if (deepUnfurl > 0.001f) {
    const float tPhase = P.U[35] * 0.42f;
    const float a1 = 8.4f * pp.x + 5.2f * pp.y + 6.6f * pp.z + tPhase;
    const float a2 = -7.2f * pp.x + 6.0f * pp.y + 9.4f * pp.z - tPhase * 0.81f;
    const float a3 = 11.5f * pp.x - 7.5f * pp.y - 8.5f * pp.z + tPhase * 1.13f;
    const float c1 = dob_cos(a1), c2 = dob_cos(a2), s3 = 0.45f * dob_sin(a3);
    const dob_v3 raw = v3(-8.16f, 3.84f, 7.36f) * c1 + v3(-8.20f, -1.38f, -5.40f) * c2 + v3(8.30f, -1.10f, 12.20f) * s3;
    const float vertTaper = dob_smoothstep(0.06f, 0.24f, depth);
    sub = v3(raw.x, raw.y * vertTaper, raw.z) * (0.00028f * deepUnfurl);
  }
  dob_v3 vg = sample_center(g, cen, uvw);
  vg.y = vg.y * dob_mix(1.0f, 0.045f, surfTailHold);
  return vg + v3(0.0f, -effSettle, 0.0f) + sub;
}

// ---- PARTICLE_ADVECT_SPLAT (particles.ts:303-462) ---------------------------------------
template <class VS, class DS>
__global__ void __launch_bounds__(256) k_parcel_advect_ref(Grid g, Grid gc, const StepParams* __restrict__ Pp,
                                                           const typename Vec4Of<VS>::type* __restrict__ cen,
                                                           const typename Vec4Of<DS>::type* __restrict__ conc,
                                                           float4* __restrict__ parcels,
                                                           uint32_t* __restrict__ splatI, uint32_t* __restrict__ splatL,
                                                           uint32_t* __restrict__ sbrick) {
  const StepParams& P = *Pp;
  const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= P.advect_count) return;
  const float4 q0 = parcels[2 * (size_t)gid];
  const float4 q1 = parcels[2 * (size_t)gid + 1];
  float mass = q0.w;
  if (mass <= 1e-6f) return;
  const float dtv = P.dt;
  const float halfXZ = P.U[52], yMin = P.U[53], surfY = P.U[40];
  dob_v3 pos = v3(q0.x, q0.y, q0.z);
  dob_v3 stretch = v3(q1.x, q1.y, q1.z);
  const float rawW = dob_maxf(0.0f, q1.w);
  float ageTicks = floorf(rawW);
  float lysis = dob_clampf(rawW - ageTicks, 0.0f, 0.98f);
  const float parcelAge = ageTicks * (1.0f / 240.0f);
  const float rouleauxMaturity = dob_smoothstep(8.5f, 18.0f, parcelAge);
  const float tailRank = dob_fract((float)gid * 0.7548776662f);
  const float meniscusHold =
      dob_pow(dob_smoothstep(0.36f, 0.995f, tailRank), 1.65f) * (1.0f - dob_smoothstep(5.2f, 10.2f, parcelAge));
  const dob_v3 v1 = sample_vel_world(g, P, cen, pos, rouleauxMaturity, meniscusHold);
  const float speed2 = dot3(v1, v1);
  if (dtv > 0.0f) {
    ageTicks = dob_minf(8191.0f, ageTicks + dob_maxf(1.0f, rintf(dtv * 240.0f)));
    const dob_v3 v2 = sample_vel_world(g, P, cen, pos + 0.5f * v1 * dtv, rouleauxMaturity, meniscusHold);
    dob_v3 vAdv = v2;
    if (speed2 > 0.0025f) {
      const dob_v3 v3v = sample_vel_world(g, P, cen, pos + 0.75f * v2 * dtv, rouleauxMaturity, meniscusHold);
      vAdv = (float)(2.0 / 9.0) * v1 + (float)(3.0 / 9.0) * v2 + (float)(4.0 / 9.0) * v3v;
    }
    const float floorSlip = dob_smoothstep(yMin + 0.005f, yMin + 0.042f, pos.y);
    const float rXZFloor = length2f(pos.x, pos.z);
    float fox = 0.0f, foz = 0.0f;
    if (rXZFloor > 1e-4f) {
      const float k = 0.016f * (1.0f - floorSlip) * dob_smoothstep(0.01f, 0.22f, rXZFloor);
      fox = (pos.x / dob_maxf(rXZFloor, 1e-4f)) * k;
      foz = (pos.z / dob_maxf(rXZFloor, 1e-4f)) * k;
    }
    vAdv = v3(vAdv.x * dob_mix(0.45f, 1.0f, floorSlip) + fox, vAdv.y * dob_mix(0.15f, 1.0f, floorSlip),
              vAdv.z * dob_mix(0.45f, 1.0f, floorSlip) + foz);
    pos = pos + vAdv * dtv;
    pos.y = dob_clampf(pos.y, yMin + 0.0055f, surfY - 0.0018f);
    if (speed2 > 2.5e-7f && floorSlip > 0.15f) {
      const float sLen = dob_maxf(length3(stretch), 1e-5f);
      const dob_v3 sDir = stretch / sLen;
      const float probeStep = 0.0065f;
      const dob_v3 vPlus = sample_vel_world(g, P, cen, pos + sDir * probeStep, rouleauxMaturity, meniscusHold);
      const dob_v3 vMinus = sample_vel_world(g, P, cen, pos - sDir * probeStep, rouleauxMaturity, meniscusHold);
      const dob_v3 dVel = (vPlus - vMinus) * (sLen / (2.0f * probeStep));
      stretch = stretch + dVel * dtv;
      const float vMag = dob_sqrt(speed2);
      if (vMag > 0.001f && sLen < 0.006f) stretch = stretch + (v1 / vMag) * (0.0022f * dtv);
      const float maxThreadLen =
          dob_mix(0.0270f, 0.0420f, meniscusHold * (1.0f - dob_smoothstep(0.005f, 0.065f, dob_maxf(0.0f, surfY - pos.y))));
      const float nextLen = dob_clampf(length3(stretch), 0.0026f, maxThreadLen);
      stretch = (stretch / dob_maxf(length3(stretch), 1e-5f)) * nextLen;
    } else if (floorSlip <= 0.15f) {
      stretch.y = stretch.y * dob_exp(-dtv * 5.0f);
    }
  }
  const dob_v3 uvw = to_uvw(P, pos);
  const float rHoriz = length2f(pos.x, pos.z);
  const float wallSponge = 1.0f - dob_smoothstep(halfXZ * 0.68f, halfXZ * 0.94f, rHoriz);
  mass = mass * dob_mix(1.0f, wallSponge, dob_clampf(dtv * 6.0f, 0.0f, 1.0f));
  if (mass <= 1e-5f || rHoriz >= halfXZ * 0.95f || uvw.x <= 0.002f || uvw.x >= 0.998f || uvw.z <= 0.002f ||
      uvw.z >= 0.998f || uvw.y >= 0.998f) {
    parcels[2 * (size_t)gid] = make_float4(q0.x, q0.y, q0.z, 0.0f);
    return;
  }
  if (dtv > 0.0f && pos.y < yMin + 0.026f) {
    const float settleWeight = 1.0f - dob_smoothstep(yMin + 0.005f, yMin + 0.026f, pos.y);
    const float dmBed = mass * dob_clampf(settleWeight * dtv * 1.65f, 0.0f, 0.095f);
    if (dmBed > 1e-7f) {
      mass = dob_maxf(0.0f, mass - dmBed);
      splat_trilinear(gc, splatL, clamp3(uvw, 0.002f, 0.998f), dmBed * 0.68f, 1e-7f, sbrick);
    }
    if (mass <= 1e-5f) {
      parcels[2 * (size_t)gid] = make_float4(q0.x, q0.y, q0.z, 0.0f);
      return;
    }
  }
  const float cellRes = dob_fract((float)gid * 0.6180339887f + 0.17f);
  const dob_v3 cu = clamp3(uvw, 0.002f, 0.998f);
  const float4 cs = lerp8x4(make_taps(gc, cu.x, cu.y, cu.z), conc);
  const float cNeighborhood = cs.x + cs.y;
  const float diluteExposure = 1.0f - dob_smoothstep(0.012f, 0.22f, cNeighborhood);
  const float ageDispersion = dob_smoothstep(1.1f, 7.8f, parcelAge + diluteExposure * 2.2f + lysis * 2.5f);
  const float lateDiluteFade = dob_smoothstep(7.2f, 16.0f, parcelAge) * diluteExposure;
  const float midResid = dob_mix(0.07f, 0.20f, cellRes);
  const float lateResid = dob_mix(0.014f, 0.052f, cellRes);
  const float minIntactMass =
      kParcelMass * dob_mix(dob_mix(0.46f, 0.64f, cellRes), dob_mix(midResid, lateResid, lateDiluteFade), ageDispersion);
  const float lysableHeadroom = mass - minIntactMass;
  const float floorShelter = dob_smoothstep(yMin + 0.024f, yMin + 0.062f, pos.y);
  if (dtv > 0.0f && lysableHeadroom > 1e-7f && floorShelter > 0.02f) {
    const float shearActivity = dob_mix(0.22f, 1.0f, dob_smoothstep(0.0005f, 0.0120f, speed2));
    const float waterExposure = (1.0f - 0.72f * dob_smoothstep(0.016f, 0.30f, cNeighborhood)) * floorShelter * shearActivity;
    const float kLysis = P.U[59];
    lysis = dob_clampf(lysis + kLysis * (1.85f * waterExposure) * dtv, 0.0f, 0.98f);
    const float fragility = dob_smoothstep(0.04f, 0.48f, lysis) * waterExposure;
    const float dmLysed = dob_minf(lysableHeadroom, mass * dob_clampf(fragility * kLysis * 1.95f * dtv, 0.0f, 0.16f));
    if (dmLysed > 1e-7f) {
      mass = dob_maxf(0.0f, mass - dmLysed);
      splat_trilinear(gc, splatL, clamp3(uvw, 0.002f, 0.998f), dmLysed, 1e-7f, sbrick);
    }
  }
  parcels[2 * (size_t)gid] = make_float4(pos.x, pos.y, pos.z, mass);
  parcels[2 * (size_t)gid + 1] = make_float4(stretch.x, stretch.y, stretch.z, ageTicks + dob_clampf(lysis, 0.0f, 0.98f));
  const float sLenNow = length3(stretch);
  if (sLenNow < 0.0038f) {
    splat_trilinear(gc, splatI, clamp3(uvw, 0.002f, 0.998f), mass, 1e-6f, sbrick);
  } else {
    const float sxz = length2f(stretch.x, stretch.z);
    const dob_v3 horiz = sxz > 1e-4f ? v3(-stretch.z, 0.0f, stretch.x) / dob_maxf(sxz, 1e-5f) : v3(1.0f, 0.0f, 0.0f);
    const dob_v3 sheetCross = cross3(stretch, horiz);
    const float scl = length3(sheetCross);
    const dob_v3 crossChoice = scl > 1e-4f ? sheetCross / dob_maxf(scl, 1e-5f) : horiz;
    const float horizMix = dob_smoothstep(0.35f, 0.85f, fabsf(stretch.y) / dob_maxf(sLenNow, 1e-5f));
    const dob_v3 sheetNorm = normalize3(mix3(crossChoice, horiz, horizMix));
    const float sheetSpan = dob_clampf(sLenNow * 0.62f, 0.0032f, 0.0085f);
    const dob_v3 sheetVec = sheetNorm * sheetSpan;
    const dob_v3 uvw0 = clamp3(to_uvw(P, pos - 0.42f * stretch), 0.002f, 0.998f);
    const dob_v3 uvw1 = clamp3(to_uvw(P, pos - 0.14f * stretch + sheetVec), 0.002f, 0.998f);
    const dob_v3 uvw2 = clamp3(to_uvw(P, pos + 0.14f * stretch - sheetVec), 0.002f, 0.998f);
    const dob_v3 uvw3 = clamp3(to_uvw(P, pos + 0.42f * stretch), 0.002f, 0.998f);
    splat_trilinear(gc, splatI, uvw0, 0.21f * mass, 1e-6f, sbrick);
    splat_trilinear(gc, splatI, uvw1, 0.29f * mass, 1e-6f, sbrick);
    splat_trilinear(gc, splatI, uvw2, 0.29f * mass, 1e-6f, sbrick);
    splat_trilinear(gc, splatI, uvw3, 0.21f * mass, 1e-6f, sbrick);
  }
}

// Closed box: Ralston RK3 tracer on the centre velocity, clamped inside the
// box, 1-point trilinear fixed-point splat of its mass.
template <class VS>
__global__ void __launch_bounds__(256) k_parcel_advect_box(Grid g, Grid gc, const StepParams* __restrict__ Pp,
                                                           const typename Vec4Of<VS>::type* __restrict__ cen,
                                                           float4* __restrict__ parcels, uint32_t* __restrict__ splatI,
                                                           uint32_t* __restrict__ sbrick) {
  const StepParams& P = *Pp;
  const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= P.advect_count) return;
  const float4 q0 = parcels[2 * (size_t)gid];
  const float mass = q0.w;
  if (mass <= 1e-6f) return;
  const float dtv = P.dt;
  dob_v3 pos = v3(q0.x, q0.y, q0.z);
  const dob_v3 v1 = sample_center(g, cen, clamp3(to_uvw(P, pos), 0.002f, 0.998f));
  const dob_v3 v2 = sample_center(g, cen, clamp3(to_uvw(P, pos + 0.5f * v1 * dtv), 0.002f, 0.998f));
  const dob_v3 v3v = sample_center(g, cen, clamp3(to_uvw(P, pos + 0.75f * v2 * dtv), 0.002f, 0.998f));
  const dob_v3 vAdv = (float)(2.0 / 9.0) * v1 + (float)(3.0 / 9.0) * v2 + (float)(4.0 / 9.0) * v3v;
  pos = pos + vAdv * dtv;
  const dob_v3 lo = dmin_of(P) + dsize_of(P) * 0.002f;
  const dob_v3 hi = v3(P.dmax[0], P.dmax[1], P.dmax[2]) - dsize_of(P) * 0.002f;
  pos = v3(dob_clampf(pos.x, lo.x, hi.x), dob_clampf(pos.y, lo.y, hi.y), dob_clampf(pos.z, lo.z, hi.z));
  parcels[2 * (size_t)gid] = make_float4(pos.x, pos.y, pos.z, mass);
  splat_trilinear(gc, splatI, clamp3(to_uvw(P, pos), 0.002f, 0.998f), mass, 1e-6f, sbrick);
}

__global__ void k_count_alive(const float4* __restrict__ parcels, uint32_t cap, unsigned int* __restrict__ out) {
  unsigned int c = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += gridDim.x * blockDim.x)
    c += parcels[2 * (size_t)i].w > 1e-6f ? 1u : 0u;
  c = __reduce_add_sync(0xffffffffu, c);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

// ---- sphere injection (closed box) ------------------------------------------------------------
template <class VS, class DS>
__global__ void __launch_bounds__(256) k_inject_sphere(Grid g, Grid gc, const StepParams* __restrict__ Pp, VS* u, VS* v,
                                                       VS* w, DS* dye, float cx, float cy, float cz, float rr,
                                                       float dyev, float vx, float vy, float vz, float sigma,
                                                       uint64_t seed) {
  const StepParams& P = *Pp;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  const dob_v3 cc = v3(cx, cy, cz);
  if (x < gc.nx && y < gc.ny && z < gc.nz) {
    const dob_v3 cdm = v3((float)gc.nx, (float)gc.ny, (float)gc.nz);
    const dob_v3 pw = to_world(P, (v3((float)x, (float)y, (float)z) + v3(0.5f, 0.5f, 0.5f)) / cdm);
    if (length3(pw - cc) <= rr) stf(dye + gc.at(x, y, z), dyev);
  }
  if (x < g.nx && y < g.ny && z < g.nz) {
    const size_t i = g.at(x, y, z);
    const dob_v3 dims = v3((float)g.nx, (float)g.ny, (float)g.nz);
    const dob_v3 fx = to_world(P, v3((float)x + 1.0f, (float)y + 0.5f, (float)z + 0.5f) / dims);
    const dob_v3 fy = to_world(P, v3((float)x + 0.5f, (float)y + 1.0f, (float)z + 0.5f) / dims);
    const dob_v3 fz = to_world(P, v3((float)x + 0.5f, (float)y + 0.5f, (float)z + 1.0f) / dims);
    if (x < g.nx - 1 && length3(fx - cc) <= rr) stf(u + i, vx + sigma * dob_sphere_noise(seed, i, 0));
    if (y < g.ny - 1 && length3(fy - cc) <= rr) stf(v + i, vy + sigma * dob_sphere_noise(seed, i, 1));
    if (z < g.nz - 1 && length3(fz - cc) <= rr) stf(w + i, vz + sigma * dob_sphere_noise(seed, i, 2));
  }
}

// d loss / d s for injected face velocities s * vel: the sum of the face
// adjoints times vel over exactly the faces k_inject_sphere writes (same
// FMA-free predicate).
__global__ void __launch_bounds__(256) k_sphere_impulse(Grid g, const StepParams* __restrict__ Pp,
                                                        const float* __restrict__ au, const float* __restrict__ av,
                                                        const float* __restrict__ aw, float cx, float cy, float cz,
                                                        float rr, float vx, float vy, float vz, double* out) {
  const StepParams& P = *Pp;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  double part = 0.0;
  if (x < g.nx && y < g.ny) {
    const dob_v3 cc = v3(cx, cy, cz);
    const size_t i = g.at(x, y, z);
    const dob_v3 dims = v3((float)g.nx, (float)g.ny, (float)g.nz);
    const dob_v3 fx = to_world(P, v3((float)x + 1.0f, (float)y + 0.5f, (float)z + 0.5f) / dims);
    const dob_v3 fy = to_world(P, v3((float)x + 0.5f, (float)y + 1.0f, (float)z + 0.5f) / dims);
    const dob_v3 fz = to_world(P, v3((float)x + 0.5f, (float)y + 0.5f, (float)z + 1.0f) / dims);
    if (x < g.nx - 1 && length3(fx - cc) <= rr) part += (double)au[i] * (double)vx;
    if (y < g.ny - 1 && length3(fy - cc) <= rr) part += (double)av[i] * (double)vy;
    if (z < g.nz - 1 && length3(fz - cc) <= rr) part += (double)aw[i] * (double)vz;
  }
  block_sum_atomic(part, out);
}

// Soft-edged drop (dob_soft_sphere weight w): dye += w dyev on the dye grid
// and face += w (vel + sigma noise) on the MAC faces below the upper walls.
// Additive, so the result does not depend on what the faces held before and
// the derivative in the centre needs no earlier state.
template <class VS, class DS>
__global__ void __launch_bounds__(256) k_inject_sphere_soft(Grid g, Grid gc, const StepParams* __restrict__ Pp, VS* u,
                                                            VS* v, VS* w, DS* dye, float cx, float cy, float cz,
                                                            float rr, float hh, float dyev, float vx, float vy,
                                                            float vz, float sigma, uint64_t seed) {
  const StepParams& P = *Pp;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  const dob_v3 cc = v3(cx, cy, cz);
  dob_v3 gw;
  if (x < gc.nx && y < gc.ny && z < gc.nz) {
    const dob_v3 cdm = v3((float)gc.nx, (float)gc.ny, (float)gc.nz);
    const dob_v3 pw = to_world(P, (v3((float)x, (float)y, (float)z) + v3(0.5f, 0.5f, 0.5f)) / cdm);
    const float wt = dob_soft_sphere(pw, cc, rr, hh, &gw);
    if (wt > 0.0f) {
      const size_t k = gc.at(x, y, z);
      stf(dye + k, ldv(dye + k) + wt * dyev);
    }
  }
  if (x < g.nx && y < g.ny && z < g.nz) {
    const size_t i = g.at(x, y, z);
    const dob_v3 dims = v3((float)g.nx, (float)g.ny, (float)g.nz);
    const dob_v3 fx = to_world(P, v3((float)x + 1.0f, (float)y + 0.5f, (float)z + 0.5f) / dims);
    const dob_v3 fy = to_world(P, v3((float)x + 0.5f, (float)y + 1.0f, (float)z + 0.5f) / dims);
    const dob_v3 fz = to_world(P, v3((float)x + 0.5f, (float)y + 0.5f, (float)z + 1.0f) / dims);
    float wt = dob_soft_sphere(fx, cc, rr, hh, &gw);
    if (x < g.nx - 1 && wt > 0.0f) stf(u + i, ldv(u + i) + wt * (vx + sigma * dob_sphere_noise(seed, i, 0)));
    wt = dob_soft_sphere(fy, cc, rr, hh, &gw);
    if (y < g.ny - 1 && wt > 0.0f) stf(v + i, ldv(v + i) + wt * (vy + sigma * dob_sphere_noise(seed, i, 1)));
    wt = dob_soft_sphere(fz, cc, rr, hh, &gw);
    if (z < g.nz - 1 && wt > 0.0f) stf(w + i, ldv(w + i) + wt * (vz + sigma * dob_sphere_noise(seed, i, 2)));
  }
}

// Gradient of the loss in the soft drop's parameters from the adjoints of
// the fields right after the injection: out[0] = sum over faces of
// w (adj . vel) (d loss / d s for injected velocity s vel, at s = 1), out[1..3]
// = d loss / d centre = sum over cells of adj_dye dyev dw/dc plus sum over
// faces of adj_face (vel + sigma noise) dw/dc.  Per-thread FP64 sums, one
// FP64 atomic per block and output.
__global__ void __launch_bounds__(256) k_sphere_soft_grad(Grid g, Grid gc, const StepParams* __restrict__ Pp,
                                                          const float* __restrict__ au, const float* __restrict__ av,
                                                          const float* __restrict__ aw, const float* __restrict__ ac,
                                                          float cx, float cy, float cz, float rr, float hh,
                                                          float dyev, float vx, float vy, float vz, float sigma,
                                                          uint64_t seed, double* out) {
  const StepParams& P = *Pp;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  const dob_v3 cc = v3(cx, cy, cz);
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
  dob_v3 gw;
  if (x < gc.nx && y < gc.ny && z < gc.nz) {
    const dob_v3 cdm = v3((float)gc.nx, (float)gc.ny, (float)gc.nz);
    const dob_v3 pw = to_world(P, (v3((float)x, (float)y, (float)z) + v3(0.5f, 0.5f, 0.5f)) / cdm);
    dob_soft_sphere(pw, cc, rr, hh, &gw);
    const double a = (double)ac[gc.at(x, y, z)] * (double)dyev;
    s1 += a * gw.x; s2 += a * gw.y; s3 += a * gw.z;
  }
  if (x < g.nx && y < g.ny && z < g.nz) {
    const size_t i = g.at(x, y, z);
    const dob_v3 dims = v3((float)g.nx, (float)g.ny, (float)g.nz);
    const dob_v3 fp[3] = {to_world(P, v3((float)x + 1.0f, (float)y + 0.5f, (float)z + 0.5f) / dims),
                          to_world(P, v3((float)x + 0.5f, (float)y + 1.0f, (float)z + 0.5f) / dims),
                          to_world(P, v3((float)x + 0.5f, (float)y + 0.5f, (float)z + 1.0f) / dims)};
    const bool inside[3] = {x < g.nx - 1, y < g.ny - 1, z < g.nz - 1};
    const float* adj[3] = {au, av, aw};
    const float vel[3] = {vx, vy, vz};
    for (int k = 0; k < 3; ++k) {
      if (!inside[k]) continue;
      const float wt = dob_soft_sphere(fp[k], cc, rr, hh, &gw);
      if (!(wt > 0.0f)) continue;
      const double a = (double)adj[k][i];
      s0 += a * (double)wt * (double)vel[k];
      const double val = (double)(vel[k] + sigma * dob_sphere_noise(seed, i, k));
      s1 += a * val * gw.x; s2 += a * val * gw.y; s3 += a * val * gw.z;
    }
  }
  block_sum_atomic(s0, out + 0);
  block_sum_atomic(s1, out + 1);
  block_sum_atomic(s2, out + 2);
  block_sum_atomic(s3, out + 3);
}

__global__ void k_eval_math(int fn, const float* __restrict__ x, const float* __restrict__ y, float* __restrict__ out,
                            uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float a = x[i], b = y ? y[i] : 0.0f;
  float r = 0.0f;
  switch (fn) {
    case 0: r = dob_sin(a); break;
    case 1: r = dob_cos(a); break;
    case 2: r = dob_exp(a); break;
    case 3: r = dob_log(a); break;
    case 4: r = dob_pow(a, b); break;
    case 5: r = dob_atan2(a, b); break;
    case 6: r = dob_tanh(a); break;
    case 7: r = __half2float(__float2half_rn(a)); break;
    case 8: r = __bfloat162float(__float2bfloat16_rn(a)); break;
    case 9: r = div_by(a, b, 1.0f / b); break;
    default: break;
  }
  out[i] = r;
}

// ---- host launchers ---------------------------------------------------------------------------


void launch_parcel_emit(const DevState& s, cudaStream_t st) {
  if (!s.ref) return;
  k_parcel_emit<<<8192 / 256, 256, 0, st>>>(s.gc, s.params, (float4*)s.parcels, s.cap, s.wave, s.splatL, s.sbrick);
}

void launch_parcel_advect(const DevState& s, cudaStream_t st) {
  const unsigned blocks = (s.cap + 255u) / 256u;
  DOB_VEL_DISPATCH(s.prec, {
    if (s.ref)
      k_parcel_advect_ref<VS, DS><<<blocks, 256, 0, st>>>(s.g, s.gc, s.params, (const typename Vec4Of<VS>::type*)s.cen,
                                                          (const typename Vec4Of<DS>::type*)s.conc, (float4*)s.parcels,
                                                          s.splatI, s.splatL, s.sbrick);
    else
      k_parcel_advect_box<VS><<<blocks, 256, 0, st>>>(s.g, s.gc, s.params, (const typename Vec4Of<VS>::type*)s.cen,
                                                      (float4*)s.parcels, s.splatI, s.sbrick);
  });
}

// One warp per brick of the dye grid: a marked brick's accumulators in both
// arrays are zeroed (8-voxel rows, 16-byte stores where the rows allow) and
// its mark cleared; unmarked bricks hold zeros already.
__global__ void __launch_bounds__(256) k_clear_splat_bricks(Grid gc, uint32_t* __restrict__ splatI,
                                                            uint32_t* __restrict__ splatL,
                                                            uint32_t* __restrict__ sbrick) {
  const int bnx = (gc.nx + 7) >> 3, bny = (gc.ny + 7) >> 3, bnz = (gc.nz + 7) >> 3;
  const int nb = bnx * bny * bnz, lane = threadIdx.x & 31;
  const bool vec = (gc.nx & 3) == 0;
  const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
  for (int b = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); b < nb; b += (int)((gridDim.x * blockDim.x) >> 5)) {
    if (sbrick[b] == 0u) continue;  // the same b in every lane
    const int bx = b % bnx, by = (b / bnx) % bny, bz = b / (bnx * bny);
    const int x0 = bx << 3, nxr = min(8, gc.nx - x0);
    for (int r = lane; r < 64; r += 32) {  // 8 rows in y by 8 planes
      const int y = (by << 3) + (r & 7), z = (bz << 3) + (r >> 3);
      if (y >= gc.ny || z >= gc.nz) continue;
      const size_t base = gc.at(x0, y, z);
      if (vec && nxr == 8) {
        reinterpret_cast<uint4*>(splatI + base)[0] = zero;
        reinterpret_cast<uint4*>(splatI + base)[1] = zero;
        reinterpret_cast<uint4*>(splatL + base)[0] = zero;
        reinterpret_cast<uint4*>(splatL + base)[1] = zero;
      } else {
        for (int k = 0; k < nxr; ++k) { splatI[base + k] = 0u; splatL[base + k] = 0u; }
      }
    }
    __syncwarp();
    if (lane == 0) sbrick[b] = 0u;
  }
}

void launch_clear_splats(const DevState& s, cudaStream_t st) {
  if (!s.sbrick) {
    cudaMemsetAsync(s.splatI, 0, s.gc.n() * 4, st);
    cudaMemsetAsync(s.splatL, 0, s.gc.n() * 4, st);
    return;
  }
  k_clear_splat_bricks<<<s.num_sms * 8, 256, 0, st>>>(s.gc, s.splatI, s.splatL, s.sbrick);
}

void launch_count_alive(const DevState& s, unsigned int* out, cudaStream_t st) {
  cudaMemsetAsync(out, 0, sizeof(unsigned int), st);
  k_count_alive<<<s.num_sms * 2, 256, 0, st>>>((const float4*)s.parcels, s.cap, out);
}

void launch_inject_sphere(const DevState& s, const float c[3], float r, float dye, const float vel[3], float sigma,
                          uint64_t seed, cudaStream_t st) {
  const int nx = s.gc.nx > s.g.nx ? s.gc.nx : s.g.nx;
  const int ny = s.gc.ny > s.g.ny ? s.gc.ny : s.g.ny;
  const int nz = s.gc.nz > s.g.nz ? s.gc.nz : s.g.nz;
  const dim3 grid((nx + 31) / 32, (ny + 7) / 8, nz);
  DOB_VEL_DISPATCH(s.prec, {
    k_inject_sphere<VS, DS><<<grid, dim3(32, 8, 1), 0, st>>>(s.g, s.gc, s.params, (VS*)s.u, (VS*)s.v, (VS*)s.w,
                                                            (DS*)s.conc, c[0], c[1], c[2], r, dye, vel[0], vel[1],
                                                            vel[2], sigma, seed);
  });
}

void launch_sphere_impulse(const DevState& s, const float* a_u, const float* a_v, const float* a_w, const float c[3],
                           float r, const float vel[3], double* out, cudaStream_t st) {
  const dim3 grid((s.g.nx + 31) / 32, (s.g.ny + 7) / 8, s.g.nz);
  cudaMemsetAsync(out, 0, sizeof(double), st);
  k_sphere_impulse<<<grid, dim3(32, 8, 1), 0, st>>>(s.g, s.params, a_u, a_v, a_w, c[0], c[1], c[2], r, vel[0], vel[1],
                                                    vel[2], out);
}

void launch_inject_sphere_soft(const DevState& s, const float c[3], float r, float h, float dye, const float vel[3],
                               float sigma, uint64_t seed, cudaStream_t st) {
  const int nx = s.gc.nx > s.g.nx ? s.gc.nx : s.g.nx;
  const int ny = s.gc.ny > s.g.ny ? s.gc.ny : s.g.ny;
  const int nz = s.gc.nz > s.g.nz ? s.gc.nz : s.g.nz;
  const dim3 grid((nx + 31) / 32, (ny + 7) / 8, nz);
  DOB_VEL_DISPATCH(s.prec, {
    k_inject_sphere_soft<VS, DS><<<grid, dim3(32, 8, 1), 0, st>>>(s.g, s.gc, s.params, (VS*)s.u, (VS*)s.v,
                                                                 (VS*)s.w, (DS*)s.conc, c[0], c[1], c[2], r, h, dye,
                                                                 vel[0], vel[1], vel[2], sigma, seed);
  });
}

void launch_sphere_soft_grad(const DevState& s, const float* a_u, const float* a_v, const float* a_w,
                             const float* a_c, const float c[3], float r, float h, float dye, const float vel[3],
                             float sigma, uint64_t seed, double* out, cudaStream_t st) {
  const int nx = s.gc.nx > s.g.nx ? s.gc.nx : s.g.nx;
  const int ny = s.gc.ny > s.g.ny ? s.gc.ny : s.g.ny;
  const int nz = s.gc.nz > s.g.nz ? s.gc.nz : s.g.nz;
  const dim3 grid((nx + 31) / 32, (ny + 7) / 8, nz);
  cudaMemsetAsync(out, 0, 4 * sizeof(double), st);
  k_sphere_soft_grad<<<grid, dim3(32, 8, 1), 0, st>>>(s.g, s.gc, s.params, a_u, a_v, a_w, a_c, c[0], c[1], c[2], r,
                                                      h, dye, vel[0], vel[1], vel[2], sigma, seed, out);
}

cudaError_t eval_math_device(int fn, const float* x, const float* y, float* out, uint32_t n) {
  float *dx = nullptr, *dy = nullptr, *dout = nullptr;
  cudaError_t e = cudaMalloc(&dx, n * sizeof(float));
  if (e == cudaSuccess && y) e = cudaMalloc(&dy, n * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&dout, n * sizeof(float));
  if (e == cudaSuccess) e = cudaMemcpy(dx, x, n * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && y) e = cudaMemcpy(dy, y, n * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_eval_math<<<(n + 255) / 256, 256>>>(fn, dx, dy, dout, n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(out, dout, n * sizeof(float), cudaMemcpyDeviceToHost);
  cudaFree(dx);
  cudaFree(dy);
  cudaFree(dout);
  return e;
}

}  // namespace dob
