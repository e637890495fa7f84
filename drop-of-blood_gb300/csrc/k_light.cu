// k_light.cu — the volumetric light cache and the empty-space brick map that
// the reference renderer reads after each frame's physics
// (src/shaders/lighting.ts:19-240, dispatched by BloodDropEngine's
// encodeLightingPasses): per velocity-grid voxel, the overhead key light's
// transmittance through the dye with the wave surface's caustics and the
// falling drops' ball-lens shadows, the camera-coupled back light's
// transmittance, the multiply scattered red light of intact cells, and a
// filtered total haemoglobin; then a 4x4x4 occupancy reduction of that total
// and its two-shell Chebyshev dilation.
//
// Compiled without multiply-add contraction (DOB_UNFUSED, -fmad=false) and
// with the library's own exp (dob_math.h), so the host oracle reproduces
// every stored half.
//
// GB300 layout: one thread per voxel in 16x4x4 blocks, so every block owns
// four whole 4x4x4 bricks and forms their occupancy from the halves it has
// just stored (shared-memory OR, no extra pass over the 9.4 MB light
// volume).  The two marches sample the 4-channel dye (16 B per voxel FP32)
// along the same direction for every voxel, so neighbouring threads gather
// neighbouring texels.
#define DOB_UNFUSED 1
#include "dob_kernels.cuh"

namespace dob {
namespace {

constexpr float kOccupied = 0.000028f;  // lighting.ts:68 (flush) and :190 (occupancy)
constexpr int kLightBX = 16, kLightBY = 4, kLightBZ = 4;

// evalOpticalDensity (lighting.ts:26-30)
__device__ __forceinline__ float optical_density(float4 c) { return 1.16f * c.x + 0.78f * c.y; }

__device__ __forceinline__ bool in_unit(dob_v3 p) {
  return !(p.x < 0.0f || p.y < 0.0f || p.z < 0.0f || p.x > 1.0f || p.y > 1.0f || p.z > 1.0f);
}

// Optical depth along one march: 9 samples stepping `d` in uvw from uvw + d/2,
// stopping early when the transmittance is below exp(-4.8) or the march
// leaves the box (lighting.ts:107-121, 139-150).
template <class V4>
__device__ __forceinline__ float march(const Grid& gc, const V4* conc, dob_v3 uvw, dob_v3 d, float step,
                                       float scale) {
  float tau = 0.0f;
  dob_v3 pos = uvw + d * 0.5f;
  for (int i = 0; i < 9; ++i) {
    if (!in_unit(pos) || tau * scale > 4.8f) break;
    const float4 cs = lerp8x4(make_taps(gc, pos.x, pos.y, pos.z), conc);
    tau = tau + optical_density(cs) * step;
    pos = pos + d;
  }
  return tau;
}

template <class DS>
__global__ void __launch_bounds__(kLightBX * kLightBY * kLightBZ)
    k_light_volume(Grid g, Grid gc, const StepParams* __restrict__ Pp,
                   const typename Vec4Of<DS>::type* __restrict__ conc, const float4* __restrict__ wave,
                   half4* __restrict__ light, float* __restrict__ brick_raw) {
  const int x = blockIdx.x * kLightBX + threadIdx.x;
  const int y = blockIdx.y * kLightBY + threadIdx.y;
  const int z = blockIdx.z * kLightBZ + threadIdx.z;
  const StepParams& P = *Pp;
  const float* U = P.U;
  float4 out = make_float4(1.0f, 1.0f, 0.0f, 0.0f);
  const bool inside = x < g.nx;
  if (inside) {
    const Recip3 dims = grid_recip(g);
    const dob_v3 uvw = (v3((float)x, (float)y, (float)z) + v3(0.5f, 0.5f, 0.5f)) / dims;
    const dob_v3 p = to_world(P, uvw);
    const dob_v3 dom = dsize_of(P);
    if (!(dob_maxf(fabsf(p.x), fabsf(p.z)) > 0.462f)) {
      // centre tap plus a tetrahedron of taps 1.02 voxels out (lighting.ts:47-58)
      const dob_v3 e = v3(1.02f, 1.02f, 1.02f) / dims;
      const float4 cC = lerp8x4(make_taps(gc, uvw.x, uvw.y, uvw.z), conc);
      const dob_v3 q0 = clamp3(uvw + v3(e.x, -e.y, -e.z), 0.0f, 1.0f);
      const dob_v3 q1 = clamp3(uvw + v3(-e.x, -e.y, e.z), 0.0f, 1.0f);
      const dob_v3 q2 = clamp3(uvw + v3(-e.x, e.y, -e.z), 0.0f, 1.0f);
      const dob_v3 q3 = clamp3(uvw + v3(e.x, e.y, e.z), 0.0f, 1.0f);
      const float4 c0 = lerp8x4(make_taps(gc, q0.x, q0.y, q0.z), conc);
      const float4 c1 = lerp8x4(make_taps(gc, q1.x, q1.y, q1.z), conc);
      const float4 c2 = lerp8x4(make_taps(gc, q2.x, q2.y, q2.z), conc);
      const float4 c3 = lerp8x4(make_taps(gc, q3.x, q3.y, q3.z), conc);
      const float totC = cC.x + cC.y;
      const float tet = 0.25f * ((c0.x + c0.y) + (c1.x + c1.y) + (c2.x + c2.y) + (c3.x + c3.y));
      const float filtered = dob_maxf(0.50f * totC + 0.50f * tet, tet);
      const float occ = dob_maxf(totC, filtered);
      const float smoothIntact = 0.28f * cC.x + 0.18f * (c0.x + c1.x + c2.x + c3.x);
      if (!(occ < kOccupied)) {
        const bool dark = U[51] > 0.5f;
        const float surfaceY = U[40];
        // 1. key light, surface caustics, drop ball lenses (lighting.ts:75-122)
        const dob_v3 keyDir = dark ? normalize3(v3(0.64f, 0.70f, 0.32f)) : normalize3(v3(0.22f, 0.95f, 0.20f));
        const float distToSurf = dob_maxf(0.0f, (surfaceY - p.y) / keyDir.y);
        const float hx = p.x + keyDir.x * distToSurf, hz = p.z + keyDir.z * distToSurf;
        const float wu = (hx + 1.60f) / 3.20f, wv = (hz + 1.60f) / 3.20f;
        float caustic = 1.0f;
        if (wu >= 0.01f && wv >= 0.01f && wu <= 0.99f && wv <= 0.99f) {
          const float4 ws = sample_wave(wave, hx, hz, 0.0f, 1.0f);
          const float depthFactor = dob_smoothstep(0.0f, 0.30f, surfaceY - p.y);
          caustic = dob_clampf(1.0f - ws.z * 28.0f * depthFactor * U[50], 0.72f, 1.38f);
        }
        for (int d = 0; d < kMaxDrops; ++d) {
          const float* sl = U + 64 + 8 * d;
          const float rDrop = sl[3];
          if (rDrop > 0.002f && sl[1] > p.y && sl[1] > surfaceY - 0.55f * rDrop) {
            const float tDrop = (sl[1] - p.y) / keyDir.y;
            const float rx = p.x + keyDir.x * tDrop, rz = p.z + keyDir.z * tDrop;
            const float rNorm = length2f(rx - sl[0], rz - sl[2]) / rDrop;
            if (rNorm < 1.25f) {
              const float shadowRing = 1.0f - 0.55f * (1.0f - dob_smoothstep(0.55f, 1.15f, rNorm));
              const float focusCore = 1.0f + 0.32f * (1.0f - dob_smoothstep(0.0f, 0.42f, rNorm));
              caustic = caustic * shadowRing * focusCore;
            }
          }
        }
        const float keyScale = (dark ? 38.0f : 22.0f) * U[48];
        const float tauKey = march(gc, conc, uvw, (keyDir * 0.042f) / dom, 0.042f, keyScale);
        const float keyLight = caustic * dob_exp(-tauKey * keyScale);
        // 2. back light aimed from the camera's horizontal heading (lighting.ts:124-151);
        // invViewProj * (0, 0, 1, 1) is the sum of the matrix's last two columns
        const float aw = U[11] + U[15];
        const dob_v3 aim = v3(U[8] + U[12], U[9] + U[13], U[10] + U[14]) / aw;
        const dob_v3 fwd = normalize3(aim - v3(U[32], U[33], U[34]));
        const float aimLen = length2f(fwd.x, fwd.z);
        const float ux = aimLen > 1e-4f ? fwd.x / aimLen : 0.0f;
        const float uz = aimLen > 1e-4f ? fwd.z / aimLen : -1.0f;
        const float hax = ux * 1.24f, haz = uz * 1.24f;
        const float rgx = -uz, rgz = ux;
        const dob_v3 backDir = dark ? normalize3(v3(-0.78f * rgx + 0.38f * hax, 0.24f, -0.78f * rgz + 0.38f * haz))
                                    : normalize3(v3(hax, 0.22f, haz));
        const float backScale = (dark ? 42.0f : 23.0f) * U[48];
        const float tauBack = march(gc, conc, uvw, (backDir * 0.040f) / dom, 0.040f, backScale);
        const float backLight = dob_exp(-tauBack * backScale);
        // 3. multiply scattered red light in intact cells (lighting.ts:153-158)
        const float midScatter = dob_exp(-tauKey * (dark ? 26.0f : 15.0f)) * 0.44f +
                                 dob_exp(-tauBack * (dark ? 28.0f : 14.0f)) * 0.36f;
        const float deepRed = dob_exp(-tauKey * (dark ? 10.5f : 5.8f)) * 0.30f +
                              dob_exp(-tauBack * (dark ? 10.0f : 5.2f)) * 0.28f + (dark ? 0.07f : 0.14f);
        out = make_float4(keyLight, backLight, smoothIntact * (midScatter + 0.62f * deepRed), filtered);
      }
    }
    st4(light + g.at(x, y, z), out);
  }
  // occupancy of the block's four bricks from the stored (rounded) totals
  // (PLUME_OCCUPANCY_RAW, lighting.ts:172-203)
  __shared__ int occupied[kLightBX / 4];
  const int tid = threadIdx.x + kLightBX * (threadIdx.y + kLightBY * threadIdx.z);
  if (tid < kLightBX / 4) occupied[tid] = 0;
  __syncthreads();
  if (inside && __half2float(__float2half_rn(out.w)) >= kOccupied) occupied[threadIdx.x >> 2] = 1;
  __syncthreads();
  if (tid < kLightBX / 4) {
    const int bx = blockIdx.x * (kLightBX / 4) + tid;
    const Grid b{g.nx / 4, g.ny / 4, g.nz / 4};
    if (bx < b.nx) brick_raw[b.at(bx, blockIdx.y, blockIdx.z)] = occupied[tid] ? 1.0f : 0.0f;
  }
}

// PLUME_OCCUPANCY_DILATE (lighting.ts:205-240): 2 within one brick (Chebyshev)
// of an occupied brick, 1 within two, else 0; neighbours clamped to the grid.
__global__ void __launch_bounds__(256) k_brick_dilate(Grid b, const float* __restrict__ raw, float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int)b.n()) return;
  const int x = i % b.nx, y = (i / b.nx) % b.ny, z = i / (b.nx * b.ny);
  bool near1 = false, near2 = false;
  for (int dz = -2; dz <= 2; ++dz)
    for (int dy = -2; dy <= 2; ++dy)
      for (int dx = -2; dx <= 2; ++dx) {
        const int nx = dob_clampi(x + dx, 0, b.nx - 1), ny = dob_clampi(y + dy, 0, b.ny - 1);
        const int nz = dob_clampi(z + dz, 0, b.nz - 1);
        if (__ldg(raw + b.at(nx, ny, nz)) > 0.5f) {
          near2 = true;
          if (max(abs(dx), max(abs(dy), abs(dz))) <= 1) near1 = true;
        }
      }
  out[i] = near1 ? 2.0f : (near2 ? 1.0f : 0.0f);
}

}  // namespace

bool light_dims_ok(const Grid& g) { return g.nx % 4 == 0 && g.ny % 4 == 0 && g.nz % 4 == 0; }

void launch_light_volume(const DevState& s, cudaStream_t st) {
  const dim3 block(kLightBX, kLightBY, kLightBZ);
  const dim3 grid((s.g.nx + kLightBX - 1) / kLightBX, s.g.ny / kLightBY, s.g.nz / kLightBZ);
  DOB_VEL_DISPATCH(s.prec, k_light_volume<DS><<<grid, block, 0, st>>>(
                               s.g, s.gc, s.params, static_cast<const typename Vec4Of<DS>::type*>(s.conc), s.wave,
                               s.light, s.brick_raw));
  const Grid b{s.g.nx / 4, s.g.ny / 4, s.g.nz / 4};
  k_brick_dilate<<<(unsigned)((b.n() + 255) / 256), 256, 0, st>>>(b, s.brick_raw, s.bricks);
}

}  // namespace dob
