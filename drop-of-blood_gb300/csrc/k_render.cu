// k_render.cu — the volumetric plume march of the reference renderer
// (marchPlume, src/shaders/render.ts:1593-2109), driven per pixel as the
// submerged camera's primary ray (evalSubmergedBranch,
// render.ts:2411-2434, with fsMain's camera ray, render.ts:2659-2688), into
// a headless image: per pixel the plume's radiance, its spectral
// transmittance and its two optical depths, as the composite consumes them
// (render.ts:2632: behind * transmittance + radiance).
//
// Restated with the reference's constants and arithmetic order, with the
// inspect-mode override off (MACRO_INSPECT_MODE = 0) and fsMain's fine
// quality.  The textures are this library's arrays, sampled as WebGPU's
// linear clamp-to-edge sampler interpolates (in FP32): the light volume
// (k_light.cu, binary16, velocity grid), the four-channel dye (dye grid),
// the dilated 4x4x4 brick occupancy, the 512x512 wave field and a caller's
// 256x64 spectral transmittance table.  The submerged ray ends where it
// crosses the wave surface (intersectWaterSurface, render.ts:1004-1128).
//
// Compiled without multiply-add contraction (DOB_UNFUSED, -fmad=false) and
// with the library's own exp / pow / sqrt (dob_math.h), so the host oracle
// reproduces every pixel's bits.
//
// GB300 layout: one thread per pixel in 16x16 tiles, so a warp's rays are
// neighbours and march through neighbouring texels; rays in clear water
// leave through the brick skip after a few brick reads.  Capped at 128
// registers (two 256-thread blocks per SM): 2.44 -> 2.24 ms for a dense
// 960x540 frame against 168 registers in 16x8 tiles (same bits).
#define DOB_UNFUSED 1
#include "dob_kernels.cuh"

namespace dob {
namespace {

constexpr int kLutW = 256, kLutH = 64;  // common.ts:22-23
constexpr int kRenderBX = 16, kRenderBY = 16;

struct PlumeOut {
  dob_v3 radiance, transmittance, bentDir;
  float tauIntact, tauTotal;
};

template <class V4>
struct RenderTex {
  Grid g, gc, gb;  // light volume (velocity grid), dye grid, bricks
  const half4* light;
  const V4* conc;
  const float* bricks;
  const float4* wave;
  const float4* lut;
};

__device__ __forceinline__ float4 f4add(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ __forceinline__ float4 f4scale(float4 a, float s) { return make_float4(a.x * s, a.y * s, a.z * s, a.w * s); }
__device__ __forceinline__ float4 f4mix(float4 a, float4 b, float t) {
  return make_float4(dob_mix(a.x, b.x, t), dob_mix(a.y, b.y, t), dob_mix(a.z, b.z, t), dob_mix(a.w, b.w, t));
}
__device__ __forceinline__ dob_v3 v3max(dob_v3 a, float s) {
  return v3(dob_maxf(a.x, s), dob_maxf(a.y, s), dob_maxf(a.z, s));
}

template <class V4>
__device__ __forceinline__ float4 light_at(const RenderTex<V4>& T, dob_v3 uvw) {
  return lerp8x4(make_taps(T.g, uvw.x, uvw.y, uvw.z), T.light);
}
template <class V4>
__device__ __forceinline__ float4 conc_at(const RenderTex<V4>& T, float u, float v, float w) {
  return lerp8x4(make_taps(T.gc, u, v, w), T.conc);
}

// sampleConcTricubic (render.ts:1544-1584): the 8-tap trilinear form of the
// cubic B-spline on the dye grid
template <class V4>
__device__ float4 conc_tricubic(const RenderTex<V4>& T, dob_v3 uvwIn) {
  const dob_v3 uvw = clamp3(uvwIn, 0.002f, 0.998f);
  const dob_v3 dims = v3((float)T.gc.nx, (float)T.gc.ny, (float)T.gc.nz);
  const dob_v3 invDims = v3(1.0f / dims.x, 1.0f / dims.y, 1.0f / dims.z);
  const dob_v3 coord = uvw * dims - v3(0.5f, 0.5f, 0.5f);
  const dob_v3 idx = v3(floorf(coord.x), floorf(coord.y), floorf(coord.z));
  const dob_v3 f = coord - idx;
  const dob_v3 f2 = f * f;
  const dob_v3 f3 = f2 * f;
  const dob_v3 omf = v3(1.0f, 1.0f, 1.0f) - f;
  const float c6 = 1.0f / 6.0f;
  const dob_v3 w0 = c6 * omf * omf * omf;
  const dob_v3 w1 = c6 * (3.0f * f3 - 6.0f * f2 + v3(4.0f, 4.0f, 4.0f));
  const dob_v3 w2 = c6 * (-3.0f * f3 + 3.0f * f2 + 3.0f * f + v3(1.0f, 1.0f, 1.0f));
  const dob_v3 w3 = c6 * f3;
  const dob_v3 g0 = w0 + w1;
  const dob_v3 g1 = w2 + w3;
  const dob_v3 h0 = clamp3((idx - v3(1.0f, 1.0f, 1.0f) + w1 / v3max(g0, 1e-5f) + v3(0.5f, 0.5f, 0.5f)) * invDims, 0.001f, 0.999f);
  const dob_v3 h1 = clamp3((idx + v3(1.0f, 1.0f, 1.0f) + w3 / v3max(g1, 1e-5f) + v3(0.5f, 0.5f, 0.5f)) * invDims, 0.001f, 0.999f);
  const float4 c000 = conc_at(T, h0.x, h0.y, h0.z), c100 = conc_at(T, h1.x, h0.y, h0.z);
  const float4 c00 = f4mix(c100, c000, g0.x);
  const float4 c010 = conc_at(T, h0.x, h1.y, h0.z), c110 = conc_at(T, h1.x, h1.y, h0.z);
  const float4 c10 = f4mix(c110, c010, g0.x);
  const float4 c0 = f4mix(c10, c00, g0.y);
  const float4 c001 = conc_at(T, h0.x, h0.y, h1.z), c101 = conc_at(T, h1.x, h0.y, h1.z);
  const float4 c01 = f4mix(c101, c001, g0.x);
  const float4 c011 = conc_at(T, h0.x, h1.y, h1.z), c111 = conc_at(T, h1.x, h1.y, h1.z);
  const float4 c11 = f4mix(c111, c011, g0.x);
  const float4 c1 = f4mix(c11, c01, g0.y);
  return f4mix(c1, c0, g0.z);
}

// the wave field's height (.r) at wave uv, bilinear, clamp-to-edge
__device__ __forceinline__ float wave_r(const float4* wave, float su, float sv) {
  const float cx = su * (float)kWaveN - 0.5f, cy = sv * (float)kWaveN - 0.5f;
  const float bx = floorf(cx), by = floorf(cy);
  const float fx = cx - bx, fy = cy - by;
  const int x0 = dob_clampi((int)bx, 0, kWaveN - 1), x1 = dob_clampi((int)bx + 1, 0, kWaveN - 1);
  const int y0 = dob_clampi((int)by, 0, kWaveN - 1), y1 = dob_clampi((int)by + 1, 0, kWaveN - 1);
  const float a00 = __ldg(&wave[y0 * kWaveN + x0].x), a10 = __ldg(&wave[y0 * kWaveN + x1].x);
  const float a01 = __ldg(&wave[y1 * kWaveN + x0].x), a11 = __ldg(&wave[y1 * kWaveN + x1].x);
  return dob_mix(dob_mix(a00, a10, fx), dob_mix(a01, a11, fx), fy);
}
// the open meniscus's fade-out window (cuvetteSignedDistXZ, render.ts:48-51)
__device__ __forceinline__ float wave_window(float x, float z) {
  return 1.0f - dob_smoothstep(-0.14f, 0.06f, length2f(x, z) - 1.38f);
}
// evalSurfaceHeightOnly (render.ts:53-66, 105-107)
__device__ float surface_height(const StepParams& P, const float4* wave, float x, float z) {
  const float window = wave_window(x, z);
  float h = 0.0f;
  if (!(window <= 0.0001f)) {
    const float su = dob_clampf((x + 1.60f) / 3.20f, 0.002f, 0.998f);
    const float sv = dob_clampf((z + 1.60f) / 3.20f, 0.002f, 0.998f);
    h = wave_r(wave, su, sv) * window;
  }
  return P.U[40] + h;
}
// evalSurfaceHeightSmooth (render.ts:68-103, 109-111): the 4-tap bilinear
// form of the cubic B-spline on the wave grid
__device__ float surface_height_smooth(const StepParams& P, const float4* wave, float x, float z) {
  const float window = wave_window(x, z);
  float h = 0.0f;
  if (!(window <= 0.0001f)) {
    const float su = dob_clampf((x + 1.60f) / 3.20f, 0.002f, 0.998f);
    const float sv = dob_clampf((z + 1.60f) / 3.20f, 0.002f, 0.998f);
    const float dims = (float)kWaveN, invDims = 1.0f / (float)kWaveN;
    const float cx = su * dims - 0.5f, cy = sv * dims - 0.5f;
    const float ix = floorf(cx), iy = floorf(cy);
    const float fx = cx - ix, fy = cy - iy;
    const float fx2 = fx * fx, fy2 = fy * fy, fx3 = fx2 * fx, fy3 = fy2 * fy;
    const float ox = 1.0f - fx, oy = 1.0f - fy;
    const float c6 = 1.0f / 6.0f;
    const float w0x = c6 * ox * ox * ox, w0y = c6 * oy * oy * oy;
    const float w1x = c6 * (3.0f * fx3 - 6.0f * fx2 + 4.0f), w1y = c6 * (3.0f * fy3 - 6.0f * fy2 + 4.0f);
    const float w2x = c6 * (-3.0f * fx3 + 3.0f * fx2 + 3.0f * fx + 1.0f);
    const float w2y = c6 * (-3.0f * fy3 + 3.0f * fy2 + 3.0f * fy + 1.0f);
    const float w3x = c6 * fx3, w3y = c6 * fy3;
    const float g0x = w0x + w1x, g0y = w0y + w1y, g1x = w2x + w3x, g1y = w2y + w3y;
    const float h0x = dob_clampf((ix - 1.0f + w1x / dob_maxf(g0x, 1e-5f) + 0.5f) * invDims, 0.002f, 0.998f);
    const float h0y = dob_clampf((iy - 1.0f + w1y / dob_maxf(g0y, 1e-5f) + 0.5f) * invDims, 0.002f, 0.998f);
    const float h1x = dob_clampf((ix + 1.0f + w3x / dob_maxf(g1x, 1e-5f) + 0.5f) * invDims, 0.002f, 0.998f);
    const float h1y = dob_clampf((iy + 1.0f + w3y / dob_maxf(g1y, 1e-5f) + 0.5f) * invDims, 0.002f, 0.998f);
    const float s0 = dob_mix(wave_r(wave, h1x, h0y), wave_r(wave, h0x, h0y), g0x);
    const float s1 = dob_mix(wave_r(wave, h1x, h1y), wave_r(wave, h0x, h1y), g0x);
    h = dob_mix(s1, s0, g0y) * window;
  }
  return P.U[40] + h;
}

// marchSurfaceSegment (render.ts:1004-1067): the first crossing of the wave
// surface on [segLo, segHi] in `steps` uniform steps, bisected 4 times
// (on the cubic B-spline height where it brackets the crossing too), then
// the secant point
__device__ float march_surface_segment(const StepParams& P, const float4* wave, dob_v3 ro, dob_v3 rd, float segLo,
                                       float segHi, int steps, bool fromAir) {
  if (segHi <= segLo + 1e-5f) return -1.0f;
  const float dt = (segHi - segLo) / (float)steps;
  float prevT = segLo;
  const dob_v3 p0 = ro + rd * prevT;
  float prevF = p0.y - surface_height(P, wave, p0.x, p0.z);
  for (int i = 1; i <= steps; ++i) {
    const float currT = segLo + (float)i * dt;
    const dob_v3 pC = ro + rd * currT;
    const float currF = pC.y - surface_height(P, wave, pC.x, pC.z);
    const bool crossed = fromAir ? (prevF >= 0.0f && currF <= 0.0f) : (prevF <= 0.0f && currF >= 0.0f);
    if (crossed) {
      float a = prevT, b = currT;
      const dob_v3 pa0 = ro + rd * a, pb0 = ro + rd * b;
      const float faSmooth = pa0.y - surface_height_smooth(P, wave, pa0.x, pa0.z);
      const float fbSmooth = pb0.y - surface_height_smooth(P, wave, pb0.x, pb0.z);
      const bool useSmooth = fromAir ? (faSmooth >= 0.0f && fbSmooth <= 0.0f) : (faSmooth <= 0.0f && fbSmooth >= 0.0f);
      float fa = useSmooth ? faSmooth : prevF;
      float fb = useSmooth ? fbSmooth : currF;
      for (int j = 0; j < 4; ++j) {
        const float mid = 0.5f * (a + b);
        const dob_v3 pM = ro + rd * mid;
        const float hM = useSmooth ? surface_height_smooth(P, wave, pM.x, pM.z) : surface_height(P, wave, pM.x, pM.z);
        const float fm = pM.y - hM;
        const bool midCross = fromAir ? (fa >= 0.0f && fm <= 0.0f) : (fa <= 0.0f && fm >= 0.0f);
        if (midCross) {
          b = mid;
          fb = fm;
        } else {
          a = mid;
          fa = fm;
        }
      }
      const float denom = fb - fa;
      const float frac = fabsf(denom) > 1e-6f ? dob_clampf(-fa / denom, 0.0f, 1.0f) : 0.5f;
      return a + (b - a) * frac;
    }
    prevT = currT;
    prevF = currF;
  }
  return -1.0f;
}
// intersectWaterSurface (render.ts:1069-1128)
__device__ float intersect_water_surface(const StepParams& P, const float4* wave, dob_v3 ro, dob_v3 rd, float tMin,
                                         float tMax, bool fromAir) {
  const float baseY = P.U[40];
  const float minH = baseY - 0.145f, maxH = baseY + 0.145f;
  float tLo = tMin, tHi = tMax;
  if (fabsf(rd.y) < 1e-4f) {
    if (ro.y < minH || ro.y > maxH) return -1.0f;
    tHi = dob_minf(tMax, tMin + 2.8f);
  } else {
    const float tA = (minH - ro.y) / rd.y, tB = (maxH - ro.y) / rd.y;
    tLo = dob_maxf(tMin, dob_minf(tA, tB));
    tHi = dob_minf(tMax, dob_maxf(tA, tB));
    if (tHi < tLo) return -1.0f;
  }
  const float rdXZ2 = rd.x * rd.x + rd.z * rd.z;
  float wLo = tLo, wHi = dob_minf(tHi, tLo + 2.8f);
  bool checkWaves = true;
  if (rdXZ2 > 1e-6f) {
    const float bXZ = (ro.x * rd.x + ro.z * rd.z) / rdXZ2;
    const float cXZ = ((ro.x * ro.x + ro.z * ro.z) - 2.2080f * 2.2080f) / rdXZ2;
    const float discXZ = bXZ * bXZ - cXZ;
    if (discXZ <= 0.0f) {
      checkWaves = false;
    } else {
      const float sXZ = dob_sqrt(discXZ);
      wLo = dob_maxf(tLo, -bXZ - sXZ);
      wHi = dob_minf(tHi, -bXZ + sXZ);
      if (wHi <= wLo) checkWaves = false;
    }
  }
  if (checkWaves) {
    const float horizSpan = dob_sqrt(dob_maxf(rdXZ2, 0.0f)) * (wHi - wLo);
    const int adaptiveSteps = dob_clampi((int)ceilf(horizSpan / 0.0052f), 14, 56);
    const float hHit = march_surface_segment(P, wave, ro, rd, wLo, wHi, adaptiveSteps, fromAir);
    if (hHit > 0.0f) return hHit;
  }
  const bool validFlatDir = fromAir ? (ro.y >= baseY && rd.y < -1e-4f) : (ro.y <= baseY && rd.y > 1e-4f);
  if (validFlatDir) {
    const float tFlat = (baseY - ro.y) / rd.y;
    if (tFlat >= tMin && tFlat <= tMax) return tFlat;
  }
  return -1.0f;
}

// henyeyGreenstein (render.ts:208-212)
__device__ __forceinline__ float hg_phase(float cosTheta, float g) {
  const float g2 = g * g;
  const float denom = dob_pow(dob_maxf(1.0f + g2 - 2.0f * g * cosTheta, 1e-4f), 1.5f);
  return (1.0f - g2) / (4.0f * 3.14159265f * denom);
}

// sampleSpectralLut (render.ts:40-46), bilinear, clamp-to-edge
__device__ dob_v3 spectral_lut(const float4* lut, float tau, float lysisFrac) {
  const float safeTau = dob_maxf(0.0f, tau);
  const float uNorm = safeTau / (0.012f + 0.996f * safeTau);
  const float uTex = (0.5f + dob_clampf(uNorm, 0.0f, 1.0f) * (float)(kLutW - 1)) / (float)kLutW;
  const float vTex = (0.5f + dob_clampf(lysisFrac, 0.0f, 1.0f) * (float)(kLutH - 1)) / (float)kLutH;
  const float cx = uTex * (float)kLutW - 0.5f, cy = vTex * (float)kLutH - 0.5f;
  const float bx = floorf(cx), by = floorf(cy);
  const float fx = cx - bx, fy = cy - by;
  const int x0 = dob_clampi((int)bx, 0, kLutW - 1), x1 = dob_clampi((int)bx + 1, 0, kLutW - 1);
  const int y0 = dob_clampi((int)by, 0, kLutH - 1), y1 = dob_clampi((int)by + 1, 0, kLutH - 1);
  const float4 a00 = __ldg(lut + y0 * kLutW + x0), a10 = __ldg(lut + y0 * kLutW + x1);
  const float4 a01 = __ldg(lut + y1 * kLutW + x0), a11 = __ldg(lut + y1 * kLutW + x1);
  return v3(dob_mix(dob_mix(a00.x, a10.x, fx), dob_mix(a01.x, a11.x, fx), fy),
            dob_mix(dob_mix(a00.y, a10.y, fx), dob_mix(a01.y, a11.y, fx), fy),
            dob_mix(dob_mix(a00.z, a10.z, fx), dob_mix(a01.z, a11.z, fx), fy));
}

// intersectBox (render.ts:1528-1540)
__device__ __forceinline__ float safe_rcp(float d) {
  const float s = fabsf(d) < 1e-6f ? (d >= 0.0f ? 1e-6f : -1e-6f) : d;
  return 1.0f / s;
}
__device__ void intersect_box(dob_v3 ro, dob_v3 rd, dob_v3 bMin, dob_v3 bMax, float& tNear, float& tFar) {
  const dob_v3 invRd = v3(safe_rcp(rd.x), safe_rcp(rd.y), safe_rcp(rd.z));
  const dob_v3 t0 = (bMin - ro) * invRd;
  const dob_v3 t1 = (bMax - ro) * invRd;
  const dob_v3 ts = v3(dob_minf(t0.x, t1.x), dob_minf(t0.y, t1.y), dob_minf(t0.z, t1.z));
  const dob_v3 tb = v3(dob_maxf(t0.x, t1.x), dob_maxf(t0.y, t1.y), dob_maxf(t0.z, t1.z));
  tNear = dob_maxf(dob_maxf(ts.x, ts.y), ts.z);
  tFar = dob_minf(dob_minf(tb.x, tb.y), tb.z);
}

// invViewProj * (x, y, z, 1) / w (the block's matrix is column-major)
__device__ __forceinline__ dob_v3 unproject(const float* M, float x, float y, float z) {
  const float px = M[0] * x + M[4] * y + M[8] * z + M[12];
  const float py = M[1] * x + M[5] * y + M[9] * z + M[13];
  const float pz = M[2] * x + M[6] * y + M[10] * z + M[14];
  const float pw = M[3] * x + M[7] * y + M[11] * z + M[15];
  return v3(px / pw, py / pw, pz / pw);
}

// the lens cone's five-tap average of the light volume (render.ts:1756-1766)
template <class V4>
__device__ float4 cone_light(const RenderTex<V4>& T, float4 lit, dob_v3 uvw, dob_v3 rayDir, dob_v3 domSize,
                             dob_v3 diskAxis1, dob_v3 diskAxis2, float rCoC, float cocBlur, float tir) {
  const float rWorldCone = dob_maxf(dob_clampf(rCoC * 1.55f, 0.0009f, 0.022f), tir * 0.012f);
  const dob_v3 rayStepUVW = (rayDir / domSize) * dob_minf(rWorldCone * 0.50f, 0.0038f);
  const float4 l1 = light_at(T, clamp3(uvw + diskAxis1 * rWorldCone + rayStepUVW, 0.0f, 1.0f));
  const float4 l2 = light_at(T, clamp3(uvw + diskAxis2 * rWorldCone - rayStepUVW, 0.0f, 1.0f));
  const float4 l3 = light_at(T, clamp3(uvw - diskAxis1 * rWorldCone - rayStepUVW, 0.0f, 1.0f));
  const float4 l4 = light_at(T, clamp3(uvw - diskAxis2 * rWorldCone + rayStepUVW, 0.0f, 1.0f));
  const float4 litAvg = f4scale(f4add(f4add(f4add(f4add(lit, l1), l2), l3), l4), 0.20f);
  return f4mix(lit, litAvg, dob_maxf(dob_smoothstep(0.14f, 0.68f, cocBlur), tir * 0.92f));
}

// marchPlume (render.ts:1593-2109) with MACRO_INSPECT_MODE = 0 and fine quality
template <class V4>
__device__ PlumeOut march_plume(const RenderTex<V4>& T, const StepParams& P, dob_v3 ro, dob_v3 rdIn, float tMinClamp,
                                float tMaxClamp, float tFocus, float apRadius, float jitter) {
  const float* U = P.U;
  PlumeOut out;
  out.radiance = v3(0.0f, 0.0f, 0.0f);
  out.transmittance = v3(1.0f, 1.0f, 1.0f);
  out.bentDir = rdIn;
  out.tauIntact = 0.0f;
  out.tauTotal = 0.0f;
  const float surfY = U[40];
  const float spongeHalfXZ = dob_minf(U[52], 0.435f);
  const dob_v3 bMin = v3(-spongeHalfXZ, U[53], -spongeHalfXZ);
  const dob_v3 bMax = v3(spongeHalfXZ, U[54] + 0.002f, spongeHalfXZ);
  float bxNear, bxFar;
  intersect_box(ro, rdIn, bMin, bMax, bxNear, bxFar);
  const float tStart = dob_maxf(bxNear + 1.5e-4f, tMinClamp);
  const float tEnd = dob_minf(bxFar - 1.5e-4f, tMaxClamp);
  if (tEnd <= tStart) return out;

  const float focalRef = dob_maxf(U[56], 0.18f);
  const float fineBase = 0.0026f;  // fine quality, no macro zoom
  const float coarseSkip = 0.015f;
  const int maxSteps = 160;
  const float effJitter = 0.5f + 0.08f * (jitter - 0.5f);
  float t = tStart + effJitter * fineBase * 0.40f;
  dob_v3 rayPos = ro + rdIn * t;
  dob_v3 rayDir = rdIn;
  float prevLitA = 0.0f, prevCoarseStep = 0.0f, prevConeD = 0.0f, prevHaloStep = 0.0f;

  const bool darkMode = U[51] > 0.5f;
  const dob_v3 camPos = v3(U[32], U[33], U[34]);
  const bool topsideCam = camPos.y > surfY;
  const dob_v3 camFwd3 = normalize3(unproject(U, 0.0f, 0.0f, 1.0f) - camPos);
  const float aimXZLen = length2f(camFwd3.x, camFwd3.z);
  const float uax = aimXZLen > 1e-4f ? camFwd3.x / aimXZLen : 0.0f;
  const float uaz = aimXZLen > 1e-4f ? camFwd3.z / aimXZLen : -1.0f;
  const float hax = uax * 1.24f, haz = uaz * 1.24f;
  const float crx = -uaz, crz = uax;
  const dob_v3 keyDir = darkMode ? normalize3(v3(0.64f, 0.70f, 0.32f)) : normalize3(v3(0.22f, 0.95f, 0.20f));
  const dob_v3 studioBackDir = normalize3(v3(hax, 0.22f, haz));
  const dob_v3 chiaroRimDir = normalize3(v3(-0.78f * crx + 0.38f * hax, 0.24f, -0.78f * crz + 0.38f * haz));
  const dob_v3 backDir = darkMode ? chiaroRimDir : studioBackDir;
  const float cosKey = dot3(rdIn, keyDir), cosBack = dot3(rdIn, backDir);
  const float phaseKey = 0.82f * dob_minf(hg_phase(cosKey, 0.94f), 5.8f) + 0.18f * hg_phase(cosKey, -0.22f);
  const float phaseBack = 0.88f * dob_minf(hg_phase(cosBack, 0.94f), 6.4f) + 0.12f * hg_phase(cosBack, -0.20f);

  const float albedoScale = U[49];
  const float tauScale = 1.68f * U[48];
  const float schlierenStr = U[60];
  const dob_v3 domSize = dsize_of(P);
  const bool hasActiveDrops = U[42] > 0.5f;
  const dob_v3 brickDimsF = v3((float)T.gb.nx, (float)T.gb.ny, (float)T.gb.nz);

  const dob_v3 refUp = fabsf(rdIn.y) > 0.92f ? v3(1.0f, 0.0f, 0.0f) : v3(0.0f, 1.0f, 0.0f);
  const dob_v3 uPerpWorld = normalize3(cross3(rdIn, refUp));
  const dob_v3 vPerpWorld = cross3(rdIn, uPerpWorld);
  const dob_v3 uLens = uPerpWorld / domSize, vLens = vPerpWorld / domSize;
  const dob_v3 diskAxis1 = 0.894427f * uLens + 0.447214f * vLens;
  const dob_v3 diskAxis2 = -0.447214f * uLens + 0.894427f * vLens;

  const dob_v3 lightDims = v3((float)T.g.nx, (float)T.g.ny, (float)T.g.nz);
  const dob_v3 hTet = v3(1.62f / lightDims.x, 1.62f / lightDims.y, 1.62f / lightDims.z);
  const dob_v3 tetK0 = v3(1.0f, -1.0f, -1.0f), tetK1 = v3(-1.0f, -1.0f, 1.0f);
  const dob_v3 tetK2 = v3(-1.0f, 1.0f, -1.0f), tetK3 = v3(1.0f, 1.0f, 1.0f);
  const dob_v3 tden = 4.0f * hTet * domSize;
  const dob_v3 invTetDenom = v3(1.0f / tden.x, 1.0f / tden.y, 1.0f / tden.z);
  const float transStopThresh = 0.010f;

  float tauTotal = 0.0f, tauLysed = 0.0f, tauIntact = 0.0f, tauOx = 0.0f;
  for (int i = 0; i < maxSteps; ++i) {
    if (t >= tEnd) break;
    const dob_v3 uvwRaw = to_uvw(P, rayPos);
    if (uvwRaw.x < -0.002f || uvwRaw.x > 1.002f || uvwRaw.z < -0.002f || uvwRaw.z > 1.002f || uvwRaw.y < -0.002f ||
        uvwRaw.y > 1.002f)
      break;
    dob_v3 uvw = clamp3(uvwRaw, 0.0005f, 0.9995f);
    // hierarchical empty-space skip on the dilated brick occupancy
    const int bx = dob_clampi((int)floorf(uvw.x * brickDimsF.x), 0, T.gb.nx - 1);
    const int by = dob_clampi((int)floorf(uvw.y * brickDimsF.y), 0, T.gb.ny - 1);
    const int bz = dob_clampi((int)floorf(uvw.z * brickDimsF.z), 0, T.gb.nz - 1);
    const float occ = __ldg(T.bricks + T.gb.at(bx, by, bz));
    if (occ < 1.5f) {
      const float brickSkip = occ < 0.5f ? 0.072f : 0.034f;
      prevLitA = 0.0f; prevCoarseStep = 0.0f; prevConeD = 0.0f; prevHaloStep = 0.0f;
      t = t + brickSkip;
      rayPos = rayPos + rayDir * brickSkip;
      continue;
    }
    float rCoC = apRadius * fabsf(t - tFocus) / focalRef;
    float cocBlur = dob_smoothstep(0.00032f, 0.0036f, rCoC);
    float4 lit = light_at(T, uvw);
    if (lit.w < 0.000005f) {
      prevLitA = lit.w; prevCoarseStep = coarseSkip; prevConeD = 0.0f; prevHaloStep = 0.0f;
      t = t + coarseSkip;
      rayPos = rayPos + rayDir * coarseSkip;
      continue;
    }
    if (prevCoarseStep > 0.0f) {
      const float crossFrac = dob_clampf((0.000005f - prevLitA) / dob_maxf(lit.w - prevLitA, 1e-8f), 0.0f, 1.0f);
      const float tCross = dob_maxf(tStart, (t - prevCoarseStep) + crossFrac * prevCoarseStep + (effJitter - 0.5f) * fineBase * 0.30f);
      rayPos = rayPos + rayDir * (tCross - t);
      t = tCross;
      prevCoarseStep = 0.0f;
      uvw = clamp3(to_uvw(P, rayPos), 0.0005f, 0.9995f);
      rCoC = apRadius * fabsf(t - tFocus) / focalRef;
      cocBlur = dob_smoothstep(0.00032f, 0.0036f, rCoC);
      lit = light_at(T, uvw);
    }
    const float tir = 0.0f;  // grazing top-slice filter: coarse quality only
    float coneDensity = lit.w;
    if ((cocBlur > 0.14f || tir > 0.04f) && lit.w > 0.000008f) {
      lit = cone_light(T, lit, uvw, rayDir, domSize, diskAxis1, diskAxis2, rCoC, cocBlur, tir);
      coneDensity = lit.w;
    }
    if (coneDensity < 0.000034f) {
      const float skipHalo = fineBase * 2.15f;
      prevConeD = coneDensity;
      prevHaloStep = skipHalo;
      t = t + skipHalo;
      rayPos = rayPos + rayDir * skipHalo;
      continue;
    }
    if (prevHaloStep > 0.0f) {
      const float haloFrac = dob_clampf((0.000034f - prevConeD) / dob_maxf(coneDensity - prevConeD, 1e-8f), 0.0f, 1.0f);
      const float tHaloCross = dob_maxf(tStart, (t - prevHaloStep) + haloFrac * prevHaloStep + (effJitter - 0.5f) * fineBase * 0.25f);
      rayPos = rayPos + rayDir * (tHaloCross - t);
      t = tHaloCross;
      prevHaloStep = 0.0f;
      uvw = clamp3(to_uvw(P, rayPos), 0.0005f, 0.9995f);
      rCoC = apRadius * fabsf(t - tFocus) / focalRef;
      cocBlur = dob_smoothstep(0.00032f, 0.0036f, rCoC);
      lit = light_at(T, uvw);
      coneDensity = lit.w;
      if ((cocBlur > 0.14f || tir > 0.04f) && lit.w > 0.000008f) {
        lit = cone_light(T, lit, uvw, rayDir, domSize, diskAxis1, diskAxis2, rCoC, cocBlur, tir);
        coneDensity = lit.w;
      }
    }
    // cubic B-spline dye near focus and at the meniscus collar
    const float wideConeMix = dob_smoothstep(0.14f, 0.72f, cocBlur);
    float4 conc;
    const float nearMeniscusCollar = dob_smoothstep(surfY - 0.072f, surfY - 0.020f, rayPos.y);
    const float tauSplineLo = 0.12f, tauSplineHi = 0.22f, cocSplineEdge = 0.36f;
    if ((cocBlur < cocSplineEdge || nearMeniscusCollar > 0.02f) && tauTotal < tauSplineHi) {
      const float cocSplineW = dob_maxf(1.0f - dob_smoothstep(cocSplineEdge - 0.16f, cocSplineEdge, cocBlur), nearMeniscusCollar);
      const float splineW = cocSplineW * (1.0f - dob_smoothstep(tauSplineLo, tauSplineHi, tauTotal));
      const float4 cB = conc_tricubic(T, uvw);
      if (splineW >= 0.995f) {
        conc = cB;
      } else {
        const float4 cT = conc_at(T, uvw.x, uvw.y, uvw.z);
        conc = f4mix(cT, cB, splineW);
      }
    } else {
      conc = conc_at(T, uvw.x, uvw.y, uvw.z);
    }
    const float cLocalRaw = dob_maxf(0.0f, conc.x) + dob_maxf(0.0f, conc.y);
    const float fLocalLysis = cLocalRaw > 0.00008f ? dob_clampf(conc.y / dob_maxf(cLocalRaw, 1e-5f), 0.0f, 1.0f) : 0.22f;
    const float vOxShear = dob_clampf(conc.z, 0.0f, 1.0f);
    if (wideConeMix > 0.001f) {
      const float collarConeGate = dob_mix(1.0f, dob_smoothstep(0.00018f, 0.0028f, cLocalRaw), nearMeniscusCollar);
      const float cPreserve = dob_maxf(cLocalRaw * dob_mix(0.72f, 0.32f, cocBlur), coneDensity * collarConeGate);
      const float cSoft = dob_mix(cLocalRaw, cPreserve, wideConeMix);
      conc.x = cSoft * (1.0f - fLocalLysis);
      conc.y = cSoft * fLocalLysis;
    }
    // step size
    const float haloCoarsen = 1.05f * (1.0f - dob_smoothstep(0.00006f, 0.00038f, dob_maxf(conc.x, coneDensity * 0.65f)));
    const float depthCoarsen = 1.35f * dob_smoothstep(0.025f, 0.22f, tauTotal);
    const float cocCoarsen = dob_clampf((rCoC / fineBase) * 0.72f, 0.0f, 2.35f) * cocBlur;
    const float ds = dob_minf(fineBase * (1.0f + haloCoarsen + depthCoarsen + cocCoarsen), tEnd - t);
    // meniscus clip, sub-collar containment and the draining orifice
    float meniscusMask = 1.0f, subCollarContain = 1.0f, collarSmoothMix = 0.0f, orificeCoreBoost = 1.0f;
    float orificeWeight = 0.0f;
    if (rayPos.y > surfY - 0.145f) {
      const bool useSmoothWaveH = rayPos.y > surfY - 0.065f;
      const float hWaveLocal = useSmoothWaveH ? surface_height_smooth(P, T.wave, rayPos.x, rayPos.z)
                                              : surface_height(P, T.wave, rayPos.x, rayPos.z);
      const float depthBelowCrater = hWaveLocal - rayPos.y;
      float bridgeWeight = 0.0f;
      if (hasActiveDrops) {
        bool deepASampled = false;
        float deepACache = 0.0f;
        for (int d = 0; d < kMaxDrops; ++d) {
          const float* sl = U + 64 + 8 * d;
          if (sl[7] > 0.0f && (sl[3] > 0.001f || sl[6] > 0.001f)) {
            const float rCol = dob_maxf(sl[3] * 0.84f, 0.018f);
            const float rD = length2f(rayPos.x - sl[0], rayPos.z - sl[2]);
            bridgeWeight = dob_maxf(bridgeWeight, 1.0f - dob_smoothstep(rCol * 0.48f, rCol, rD));
            if (sl[3] > 0.015f && sl[6] > 0.012f && depthBelowCrater > -0.008f && depthBelowCrater < 0.044f) {
              if (!deepASampled) {
                deepACache = light_at(T, v3(uvw.x, dob_maxf(0.002f, uvw.y - 0.033f), uvw.z)).w;
                deepASampled = true;
              }
              const float emerg = (sl[1] - surfY) / dob_maxf(sl[3], 0.010f);
              const float domeStillEmerging = dob_smoothstep(-0.85f, 0.05f, emerg);
              const float stemBelowGate = 1.0f - dob_smoothstep(0.00025f, 0.0018f, deepACache);
              const float nascentTouch = dob_smoothstep(-0.28f, 0.24f, emerg) * stemBelowGate;
              const float depthFade = (1.0f - dob_smoothstep(0.015f, 0.036f, depthBelowCrater)) * stemBelowGate * domeStillEmerging;
              const float rSubFoot = sl[3] * 0.78f + dob_maxf(0.0f, depthBelowCrater) * 0.44f;
              const float rFeather = dob_mix(0.0016f, 0.0044f, dob_maxf(nascentTouch, topsideCam ? 0.0f : 1.0f));
              const float radialClip = 1.0f - dob_smoothstep(rSubFoot * 0.84f, rSubFoot + rFeather, rD);
              subCollarContain = dob_minf(subCollarContain, dob_mix(1.0f, radialClip, depthFade));
              const float innerSmooth = dob_smoothstep(rSubFoot * 0.18f, rSubFoot * 0.68f, rD) *
                                        (1.0f - dob_smoothstep(rSubFoot * 0.72f, rSubFoot * 0.96f, rD));
              collarSmoothMix = dob_maxf(collarSmoothMix, depthFade * innerSmooth);
              const float rOrifice = rSubFoot * 0.98f;
              const float orificeRadial = 1.0f - dob_smoothstep(rOrifice * 0.78f, rOrifice + 0.0015f, rD);
              const float orificeVertical = 1.0f - dob_smoothstep(0.014f, 0.038f, dob_maxf(0.0f, depthBelowCrater));
              const float drainActive = dob_smoothstep(0.012f, 0.085f, sl[6]);
              const float slotOrifice = orificeRadial * orificeVertical * drainActive * domeStillEmerging;
              orificeWeight = dob_maxf(orificeWeight, slotOrifice);
              orificeCoreBoost = dob_maxf(orificeCoreBoost, 1.0f + (topsideCam ? 0.65f : 0.40f) * slotOrifice);
            }
          }
        }
      }
      const float surfLocal =
          topsideCam ? dob_mix(hWaveLocal, dob_maxf(hWaveLocal, surfY + 0.003f), bridgeWeight) : hWaveLocal;
      const float meniscusBokeh = dob_smoothstep(0.00028f, 0.0018f, rCoC);
      const float grazingTopside = topsideCam ? 1.0f - dob_smoothstep(0.06f, 0.24f, fabsf(rayDir.y)) : 0.0f;
      const float cocMeniscusFade = 0.008f + meniscusBokeh * (0.022f + 0.024f * grazingTopside);
      const float topsideMask = dob_mix(dob_smoothstep(0.0f, cocMeniscusFade, surfLocal - rayPos.y),
                                        dob_smoothstep(-0.003f, 0.008f, surfLocal - rayPos.y), bridgeWeight);
      meniscusMask = (topsideCam ? topsideMask : dob_smoothstep(0.0005f, 0.0085f, hWaveLocal - rayPos.y)) * subCollarContain;
    }
    if (collarSmoothMix > 0.001f) {
      conc.x = dob_mix(conc.x, dob_maxf(conc.x * 0.80f, coneDensity * (1.0f - fLocalLysis)), collarSmoothMix * 0.35f);
      conc.y = dob_mix(conc.y, dob_maxf(conc.y * 0.80f, coneDensity * fLocalLysis), collarSmoothMix * 0.35f);
    }
    const float intactMask = dob_smoothstep(0.00006f, 0.00085f, conc.x) * meniscusMask;
    const float lysedMask = dob_smoothstep(0.00028f, 0.0016f, conc.y) * meniscusMask;
    const float cIntact = dob_maxf(0.0f, conc.x) * intactMask * orificeCoreBoost;
    const float cLysed = dob_maxf(0.0f, conc.y) * lysedMask * (1.0f - 0.55f * orificeWeight);
    const float cTotal = cIntact + cLysed;
    if (cTotal > 0.00004f) {
      const float fLysis = dob_clampf(cLysed / dob_maxf(cTotal, 1e-5f), 0.0f, 1.0f);
      const float intactFrac = 1.0f - fLysis;
      const float topDownTauRelief =
          dob_mix(1.0f, 0.56f, dob_smoothstep(0.62f, 0.94f, -rayDir.y) * dob_smoothstep(0.028f, 0.18f, tauTotal));
      const float dTauIntact = cIntact * ds * (1.22f * tauScale * topDownTauRelief);
      const float dTauLysed = cLysed * ds * (2.65f * tauScale * topDownTauRelief);
      const float dTau = dTauIntact + dTauLysed;
      tauTotal = tauTotal + dTau;
      tauLysed = tauLysed + dTauLysed;
      tauIntact = tauIntact + dTauIntact;
      const float coherentOxWeight = dob_smoothstep(0.0014f, 0.0068f, conc.x) * (1.0f - 0.85f * dob_smoothstep(0.28f, 0.72f, cocBlur));
      tauOx = tauOx + dTau * (vOxShear * coherentOxWeight);
      const float meanOxShear = dob_clampf(tauOx / dob_maxf(tauTotal, 1e-6f), 0.0f, 1.0f);
      // Duysens sieve + Prahl spectral table
      const float tauCell = dob_mix(0.0042f, 0.0065f, dob_smoothstep(0.10f, 0.55f, cocBlur));
      const float tauSieveRef = dob_maxf(tauTotal, tauCell);
      const float sieveAlpha = dob_clampf(tauTotal / tauCell, 0.0f, 1.0f);
      const dob_v3 tCell = spectral_lut(T.lut, tauSieveRef, meanOxShear * dob_mix(1.0f, 0.35f, cocBlur));
      const float rAnchor = tCell.x + (0.96f - tCell.x) * (1.0f - sieveAlpha);
      const dob_v3 lutSieveRaw = v3(1.0f - sieveAlpha * (1.0f - rAnchor), 1.0f - sieveAlpha * (1.0f - tCell.y),
                                    1.0f - sieveAlpha * (1.0f - tCell.z));
      const float intactDichroGate = intactFrac * dob_smoothstep(0.010f, 0.042f, tauTotal);
      const float gRoseGuard =
          dob_minf(lutSieveRaw.y, dob_mix(lutSieveRaw.z * 0.94f + 0.04f * lutSieveRaw.x, lutSieveRaw.y, intactDichroGate));
      const dob_v3 lutSieve = v3(lutSieveRaw.x, gRoseGuard, lutSieveRaw.z);
      const dob_v3 lutTrans = v3(dob_minf(out.transmittance.x, lutSieve.x), dob_minf(out.transmittance.y, lutSieve.y),
                                 dob_minf(out.transmittance.z, lutSieve.z));
      const float keyIllum = lit.x, backIllum = lit.y, multiScat = lit.z;
      const float orificeScatterDamp = 1.0f - (topsideCam ? 0.16f : 0.08f) * orificeWeight;
      const float thinNeighborhood = 1.0f - dob_smoothstep(0.016f, 0.042f, coneDensity);
      const float subPlugZone = 1.0f - 0.96f * dob_smoothstep(surfY - 0.115f, surfY - 0.042f, rayPos.y);
      const float dfSubPlugZone = 1.0f - dob_smoothstep(surfY - 0.135f, surfY - 0.058f, rayPos.y);
      const float thinSheetFactor = dob_smoothstep(0.16f, 0.52f, vOxShear) * (1.0f - dob_smoothstep(0.006f, 0.030f, tauTotal)) *
                                    (1.0f - dob_smoothstep(0.018f, 0.056f, cLocalRaw)) * thinNeighborhood * subPlugZone;
      const float dfDichroFactor = dob_smoothstep(0.09f, 0.32f, vOxShear) *
                                   dob_smoothstep(0.14f, 0.52f, dob_maxf(backIllum, keyIllum * 0.78f)) *
                                   (1.0f - dob_smoothstep(0.009f, 0.032f, tauTotal)) *
                                   (1.0f - dob_smoothstep(0.022f, 0.060f, cLocalRaw)) * thinNeighborhood * dfSubPlugZone *
                                   intactFrac;
      dob_v3 stepRad = v3(0.0f, 0.0f, 0.0f), dfCoherentRim = v3(0.0f, 0.0f, 0.0f);
      const float topDownCoreWarm = dob_smoothstep(0.55f, 0.92f, -rayDir.y) * dob_smoothstep(0.04f, 0.26f, tauTotal);
      if (!darkMode) {
        const dob_v3 fwdTint = mix3(v3(0.064f, 0.0020f, 0.0016f), v3(0.094f, 0.0140f, 0.0014f), thinSheetFactor);
        const dob_v3 keyTint = mix3(v3(0.068f, 0.0011f, 0.0010f), v3(0.105f, 0.0034f, 0.0011f), vOxShear);
        const dob_v3 coreTint = mix3(v3(0.032f, 0.00055f, 0.00068f), v3(0.026f, 0.00062f, 0.00072f), vOxShear);
        const dob_v3 rubyForward = fwdTint * (backIllum * (0.22f + 0.58f * phaseBack)) * orificeScatterDamp;
        const dob_v3 carmineKey = keyTint * (keyIllum * (0.38f + 0.54f * phaseKey + 0.42f * topDownCoreWarm));
        const dob_v3 venousMulti = coreTint * (0.34f + 1.35f * multiScat + 0.48f * topDownCoreWarm);
        stepRad = (rubyForward + carmineKey + venousMulti) * albedoScale;
      } else {
        const dob_v3 rimTint = mix3(v3(1.08f, 0.032f, 0.020f), v3(2.85f, 0.465f, 0.018f), dfDichroFactor);
        const dob_v3 baseKeyTint =
            mix3(v3(0.58f, 0.014f, 0.013f), v3(0.88f, 0.028f, 0.015f), dob_smoothstep(0.24f, 0.78f, vOxShear));
        const dob_v3 keyTint = mix3(baseKeyTint, v3(2.05f, 0.330f, 0.018f), dfDichroFactor * 0.65f);
        const float plugSelfShadow = 1.0f - 0.76f * dob_smoothstep(0.028f, 0.088f, coneDensity);
        const dob_v3 darkRimFwd = rimTint * (backIllum * (0.22f + 1.08f * phaseBack)) * dob_mix(0.32f, 1.0f, plugSelfShadow);
        const dob_v3 darkKey = keyTint * (keyIllum * (0.24f + 0.72f * phaseKey)) * plugSelfShadow;
        const dob_v3 oxbloodCore = v3(0.052f, 0.0010f, 0.0011f) * (0.040f + 1.22f * multiScat);
        stepRad = (darkRimFwd + darkKey + oxbloodCore) * albedoScale;
      }
      // tetrahedral density gradient: cellular sheet glow and Schlieren bending
      const float sheetGate = dob_smoothstep(0.0032f, 0.0110f, coneDensity) * (1.0f - dob_smoothstep(0.18f, 0.34f, tauTotal)) *
                              dob_smoothstep(0.032f, 0.11f, out.transmittance.x) * (1.0f - dob_smoothstep(0.44f, 0.88f, cocBlur));
      if (sheetGate > 0.002f) {
        const float d0 = light_at(T, clamp3(uvw + tetK0 * hTet, 0.0f, 1.0f)).w;
        const float d1 = light_at(T, clamp3(uvw + tetK1 * hTet, 0.0f, 1.0f)).w;
        const float d2 = light_at(T, clamp3(uvw + tetK2 * hTet, 0.0f, 1.0f)).w;
        const float d3 = light_at(T, clamp3(uvw + tetK3 * hTet, 0.0f, 1.0f)).w;
        const dob_v3 gradWorld = (tetK0 * d0 + tetK1 * d1 + tetK2 * d2 + tetK3 * d3) * invTetDenom;
        const float gradLen = length3(gradWorld);
        if (gradLen > 0.12f) {
          const dob_v3 nSheet = -gradWorld / gradLen;
          const float grazing = dob_pow(1.0f - dob_clampf(fabsf(dot3(nSheet, -rayDir)), 0.0f, 1.0f), 1.90f);
          const float sheetCrisp = dob_smoothstep(0.15f, 2.0f, gradLen) * intactFrac * sheetGate;
          if (!darkMode) {
            const dob_v3 nMacro = normalize3(v3(-gradWorld.x, -gradWorld.y * 0.65f, -gradWorld.z) + v3(1e-6f, 0.0f, 0.0f));
            const float keyFace = dob_smoothstep(-0.18f, 0.82f, dot3(nMacro, keyDir)) * keyIllum;
            const dob_v3 keyShoulderTint = mix3(v3(0.095f, 0.0018f, 0.0014f), v3(0.145f, 0.0052f, 0.0016f), vOxShear);
            const dob_v3 sheetTint = mix3(v3(0.125f, 0.0038f, 0.0028f), v3(0.185f, 0.028f, 0.0026f), thinSheetFactor);
            stepRad = stepRad + (sheetTint * (grazing * backIllum) + keyShoulderTint * (0.68f * keyFace)) *
                                    (sheetCrisp * orificeScatterDamp);
          } else {
            const dob_v3 nChiaro = normalize3(v3(-gradWorld.x, -gradWorld.y * 0.40f, -gradWorld.z) + v3(1e-6f, 0.0f, 0.0f));
            const float sideKeyFace = dob_smoothstep(-0.14f, 0.76f, dot3(nChiaro, keyDir)) * keyIllum;
            const float rimEdgeFace = dob_smoothstep(-0.14f, 0.76f, dot3(nChiaro, backDir)) * backIllum;
            const float chiaroSheet =
                sheetCrisp * (1.48f * sideKeyFace + 1.82f * rimEdgeFace + 2.35f * grazing * (0.04f + 0.96f * dob_maxf(keyIllum, backIllum)));
            const dob_v3 chiaroTint = mix3(v3(0.82f, 0.025f, 0.016f), v3(3.15f, 0.510f, 0.018f), dfDichroFactor);
            stepRad = stepRad + chiaroTint * chiaroSheet;
            const float thinRimDrive =
                sheetCrisp * dfDichroFactor * (0.28f + 0.90f * grazing + 0.38f * dob_maxf(sideKeyFace, rimEdgeFace));
            const float dfRimProb = 1.0f - dob_exp(-thinRimDrive * ds * 11.5f);
            dfCoherentRim = v3(1.36f, 0.220f, 0.008f) * dfRimProb * albedoScale;
          }
          const dob_v3 gradN = (schlierenStr * sheetGate) * gradWorld;
          const dob_v3 gradPerp = gradN - dot3(gradN, rayDir) * rayDir;
          rayDir = normalize3(rayDir + clamp3(gradPerp / 1.333f, -1.2f, 1.2f) * ds);
        }
      }
      const float scatterProb = 1.0f - dob_exp(-cIntact * ds * 24.0f);
      dob_v3 inScatter = scatterProb * stepRad + dfCoherentRim;
      if (darkMode && cLysed > 0.00015f) {
        const float beamHalo = 0.26f * (keyIllum + backIllum) + 1.65f * multiScat;
        const float haloTransillum = (1.0f - dob_exp(-cLysed * ds * 18.0f)) * dob_clampf(beamHalo, 0.0f, 0.55f);
        inScatter = inScatter + v3(0.32f, 0.016f, 0.012f) * haloTransillum;
      }
      out.radiance = out.radiance + out.transmittance * inScatter;
      out.transmittance = lutTrans;
      const float maxTrans = dob_maxf(out.transmittance.x, dob_maxf(out.transmittance.y, out.transmittance.z));
      if (maxTrans < transStopThresh) {
        out.transmittance = v3(0.0f, 0.0f, 0.0f);
        break;
      }
    }
    t = t + ds;
    rayPos = rayPos + rayDir * ds;
  }
  out.bentDir = rayDir;
  out.tauIntact = tauIntact;
  out.tauTotal = tauTotal;
  return out;
}

// One pixel: fsMain's camera ray and lens (render.ts:2659-2684), then the
// submerged branch's primary march (render.ts:2420-2434), ending at the
// ray's crossing of the wave surface (the flat plane for rays within 0.052
// of horizontal, as the reference takes it).  Output per pixel, 8 halves: radiance rgb,
// tauTotal, transmittance rgb, tauIntact.
template <class V4>
__global__ void __launch_bounds__(kRenderBX * kRenderBY, 2)
    k_render_plume(RenderTex<V4> T, const StepParams* __restrict__ Pp, int W, int H, __half* __restrict__ out) {
  const int px = blockIdx.x * kRenderBX + threadIdx.x;
  const int py = blockIdx.y * kRenderBY + threadIdx.y;
  if (px >= W || py >= H) return;
  const StepParams& P = *Pp;
  const float* U = P.U;
  const float fragX = (float)px + 0.5f, fragY = (float)py + 0.5f;
  const float ndcX = fragX / (float)W * 2.0f - 1.0f;
  const float ndcY = 1.0f - fragY / (float)H * 2.0f;
  const dob_v3 ro = v3(U[32], U[33], U[34]);
  const dob_v3 rd = normalize3(unproject(U, ndcX, ndcY, 1.0f) - ro);
  const dob_v3 camFwd = normalize3(unproject(U, 0.0f, 0.0f, 0.5f) - ro);
  const float fx = fragX + U[39] * 5.588238f, fy = fragY + U[39] * 3.14159f;
  const float jitter = dob_fract(52.9829189f * dob_fract(0.06711056f * fx + 0.00583715f * fy));
  const float camRelY = ro.y - surface_height(P, T.wave, ro.x, ro.z);
  const float focalDist = dob_maxf(0.18f, U[56]);
  const float cosAxis = dob_maxf(dot3(rd, camFwd), 0.35f);
  const float tFocus = focalDist / cosAxis;
  const float apRadius = dob_maxf(0.0f, U[57]);
  float tUnderSurf = -1.0f;
  if (camRelY < -0.0005f && rd.y > 0.001f) {
    const float tFlatApprox = (U[40] - ro.y) / rd.y;
    if (rd.y > 0.052f && tFlatApprox < 4.5f)
      tUnderSurf = intersect_water_surface(P, T.wave, ro, rd, 0.004f, dob_minf(12.0f, tFlatApprox + 0.8f), false);
    else
      tUnderSurf = dob_minf(12.0f, tFlatApprox);
  }
  const float tPlumeEnd = tUnderSurf > 0.0f ? tUnderSurf + 0.004f : 5.5f;
  const PlumeOut o = march_plume(T, P, ro, rd, 0.02f, tPlumeEnd, tFocus, apRadius, jitter);
  __half* q = out + 8 * ((size_t)py * W + px);
  q[0] = __float2half_rn(o.radiance.x);
  q[1] = __float2half_rn(o.radiance.y);
  q[2] = __float2half_rn(o.radiance.z);
  q[3] = __float2half_rn(o.tauTotal);
  q[4] = __float2half_rn(o.transmittance.x);
  q[5] = __float2half_rn(o.transmittance.y);
  q[6] = __float2half_rn(o.transmittance.z);
  q[7] = __float2half_rn(o.tauIntact);
}

}  // namespace

void launch_render_plume(const DevState& s, const float4* lut, int W, int H, __half* out, cudaStream_t st) {
  const dim3 block(kRenderBX, kRenderBY);
  const dim3 grid((W + kRenderBX - 1) / kRenderBX, (H + kRenderBY - 1) / kRenderBY);
  const Grid gb{s.g.nx / 4, s.g.ny / 4, s.g.nz / 4};
  DOB_VEL_DISPATCH(s.prec, {
    using V4 = typename Vec4Of<DS>::type;
    RenderTex<V4> T{s.g, s.gc, gb, s.light, (const V4*)s.conc, s.bricks, s.wave, lut};
    k_render_plume<V4><<<grid, block, 0, st>>>(T, s.params, W, H, out);
  });
}

}  // namespace dob
