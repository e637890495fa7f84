// k_wave.cu — the 512x512 gravity-capillary wave solver (wave.ts:55-388)
// that writes the wave texture the step samples (top pressure, Marangoni
// layer, emission).  The reference runs it as seven passes at the start of
// every substep (BloodDropEngine.ts:1886-1912): spatial force, row FFT,
// column FFT, spectral propagation, inverse column FFT, inverse row FFT,
// finalize.  Here they are four kernels:
//
//   k_wave_force_rows   force on one row of texels, its forward 512-point
//                       FFT in shared memory                    (passes 1-2)
//   k_wave_columns      a column and its Hermitian mirror column: forward
//                       FFT of both, the propagation (which pairs (kx, kz)
//                       with (-kx, -kz)), inverse FFT of both   (passes 3-5)
//   k_wave_rows_inverse inverse FFT of one row, in place         (pass 6)
//   k_wave_finalize     Laplacian, border fade, half rounding    (pass 7)
//
// The spectra never leave shared memory between the column passes, so the
// solver moves the 2 MB complex field through memory three times instead of
// five.  Every butterfly is the reference's radix-2 decimation in time
// (bit-reversed load, stage s pairs i0 and i0 + 2^s) and the twiddle of
// (k, span) is taken from a 256-entry table of sign * (2 pi m) / 512 at
// m = k * 512 / span, which is the same float: both products and the
// division only differ by powers of two.  The unit is compiled without
// multiply-add contraction and with the host's transcendental functions
// (dob_math.h), so every texel equals the CPU restatement's bit for bit.
#define DOB_UNFUSED 1
#include "dob_kernels.cuh"

namespace dob {
namespace {

constexpr int kN = kWaveN, kHalf = kWaveN / 2, kStages = 9;
constexpr float kUnitary = 0.04419417382f;  // 1/sqrt(512) as the reference writes it

__device__ __forceinline__ uint32_t rev9(uint32_t i) { return __brev(i) >> (32 - kStages); }
__device__ __forceinline__ float wave_world(int i) {
  const float uv = ((float)i + 0.5f) / 512.0f;
  return uv * 3.20f - 1.60f;
}
// twiddle table: tw[m] = (cos, sin) of sign * (2 pi m) / 512, m < 256
__device__ __forceinline__ void make_twiddles(float2* tw, float sign, int t, int nthreads) {
  for (int m = t; m < kHalf; m += nthreads) {
    const float angle = sign * (6.28318530718f * (float)m) / 512.0f;
    float s, c;
    dob_sincos(angle, &s, &c);
    tw[m] = make_float2(c, s);
  }
}
// nine butterfly stages over one 512-point line in shared memory, thread t
// of 256 taking butterfly t of every stage
__device__ __forceinline__ void butterflies(float2* a, const float2* tw, int t, int sync_threads) {
  (void)sync_threads;
#pragma unroll 1
  for (int stage = 0; stage < kStages; ++stage) {
    const int halfSpan = 1 << stage;
    const int k = t & (halfSpan - 1);
    const int i0 = ((t >> stage) << (stage + 1)) + k, i1 = i0 + halfSpan;
    const float2 x = a[i0], b = a[i1];
    const float2 w = tw[k << (kStages - 1 - stage)];
    const float bx = b.x * w.x - b.y * w.y, by = b.x * w.y + b.y * w.x;
    __syncthreads();
    a[i0] = make_float2(x.x + bx, x.y + by);
    a[i1] = make_float2(x.x - bx, x.y - by);
    __syncthreads();
  }
}

// Passes 1-2 (wave.ts:55-172, 174-245): block = one row iy, 256 threads,
// texels ix = t and t + 256.  Writes the film to `film` and the row's
// unitary forward FFT of (eta, deta/dt) to `spec`.
template <class VS>
__global__ void __launch_bounds__(256) k_wave_force_rows(Grid g, const StepParams* __restrict__ Pp,
                                                         const float4* __restrict__ wave, const VS* __restrict__ v,
                                                         float* __restrict__ film_out, float2* __restrict__ spec) {
  __shared__ float2 line[kN];
  __shared__ float2 tw[kHalf];
  const int t = threadIdx.x, iy = blockIdx.x;
  const float* U = Pp->U;
  make_twiddles(tw, -1.0f, t, 256);
  const float dt = dob_clampf(U[38], 0.0f, 0.025f);
  const float timeScale = dt / 0.0166667f;
  const float marangoniStr = U[41], halfXZ = U[52];
  auto film_at = [&](int x, int y) {
    x = dob_clampi(x, 0, kN - 1);
    y = dob_clampi(y, 0, kN - 1);
    return __ldg(&wave[y * kN + x].w);
  };
#pragma unroll 1
  for (int h = 0; h < 2; ++h) {
    const int ix = t + h * 256;
    const float4 c = __ldg(&wave[iy * kN + ix]);
    float eta = c.x, vel = c.y, film = c.w;
    const float s1 = ((film_at(ix, iy + 1) + film_at(ix, iy - 1)) + film_at(ix + 1, iy)) + film_at(ix - 1, iy);
    const float s2 = ((film_at(ix + 1, iy + 1) + film_at(ix - 1, iy + 1)) + film_at(ix + 1, iy - 1)) +
                     film_at(ix - 1, iy - 1);
    const float rawLapFilm = (0.20f * s1 + 0.05f * s2) - film;
    const float lapFilm = rawLapFilm * 4.0f;
    const float wx = wave_world(ix), wz = wave_world(iy);
    float forceDrops = 0.0f, activeExcav = 0.0f, maxDrain = 0.0f;
#pragma unroll 1
    for (int d = 0; d < 8; ++d) {
      const float* S = U + 64 + 8 * d;
      const float signedSeed = S[7], drainRate = S[6];
      if (!(signedSeed > 0.0f && drainRate > 0.0005f)) continue;
      maxDrain = dob_maxf(maxDrain, drainRate);
      const float rDrop = dob_maxf(S[3], 0.018f);
      const float speedY = dob_clampf(-S[4], 0.06f, 0.65f);
      const float r = length2f(wx - S[0], wz - S[2]);
      const float rNorm = r / dob_clampf(rDrop * 1.05f, 0.024f, 0.082f);
      const float emergNorm = (S[1] - U[40]) / dob_maxf(rDrop, 0.018f);
      const float excavGate = dob_smoothstep(-0.78f, -0.04f, emergNorm);
      const float impactBell = dob_sin(dob_clampf((1.05f - emergNorm) / 1.83f, 0.0f, 1.0f) * 3.14159265f) * excavGate;
      const float impactShape = dob_exp(-rNorm * rNorm) * (1.0f - rNorm * rNorm);
      const float dynImpulse = (6.8f * impactBell * (rDrop / 0.056f)) * (0.72f + 2.65f * speedY);
      const float rNormCap = r / dob_clampf(rDrop * 0.44f, 0.013f, 0.030f);
      const float capWindow =
          dob_smoothstep(-0.35f, 0.28f, emergNorm) * (1.0f - dob_smoothstep(0.68f, 1.06f, emergNorm));
      const float capShape = dob_exp(-rNormCap * rNormCap) * (1.0f - rNormCap * rNormCap);
      const float capImpulse = (4.6f * capWindow * (0.60f + 0.40f * (rDrop / 0.056f))) * (0.65f + 2.20f * speedY);
      forceDrops = forceDrops - dynImpulse * impactShape - capImpulse * capShape;
      activeExcav = dob_maxf(activeExcav, excavGate * dob_exp(-0.5f * rNorm * rNorm));
      const float rStain = dob_maxf(0.018f, rDrop * 0.60f);
      const float stain = dob_exp(-(r * r) / (rStain * rStain)) * dob_clampf(drainRate * 0.42f, 0.0f, 1.0f);
      film = dob_maxf(film, stain * 0.65f);
    }
    const float effLapFilm = dob_mix(dob_maxf(lapFilm, -0.0015f), lapFilm, activeExcav);
    const float forceMarangoni = marangoniStr * 0.28f * effLapFilm;
    film = dob_clampf(film + marangoniStr * 0.065f * rawLapFilm * timeScale, 0.0f, 1.0f);
    film = film * dob_pow(0.88f, timeScale);
    float forceSubsurface = 0.0f;
    const float subsurfGate = dob_clampf(activeExcav * 1.4f + dob_smoothstep(0.0f, 0.06f, maxDrain), 0.0f, 1.0f);
    const float rw = length2f(wx, wz);
    if (subsurfGate > 0.001f && rw < halfXZ * 0.94f) {
      const float tu = (wx + halfXZ) / (2.0f * halfXZ), tv = (wz + halfXZ) / (2.0f * halfXZ);
      const float vSubY = lerp8(make_taps(g, tu, 0.988f, tv), v);
      const float wallTaper = 1.0f - dob_smoothstep(halfXZ * 0.62f, halfXZ * 0.92f, rw);
      forceSubsurface = dob_clampf(dob_maxf(vSubY, 0.0f), 0.0f, 0.48f) * 0.42f * wallTaper * subsurfGate;
    }
    vel = vel + (forceDrops + forceMarangoni + forceSubsurface) * dt;
    const float absorbZone = dob_smoothstep(0.90f, 1.54f, rw);
    const float rayleighDamp = dob_exp(-dt * (24.0f * absorbZone * absorbZone));
    const float borderZero = 1.0f - dob_smoothstep(1.22f, 1.56f, rw);
    eta = dob_clampf(eta * rayleighDamp * borderZero, -0.14f, 0.14f);
    vel = dob_clampf(vel * rayleighDamp * borderZero, -1.8f, 1.8f);
    film_out[iy * kN + ix] = film * borderZero;
    line[rev9((uint32_t)ix)] = make_float2(eta, vel);
  }
  __syncthreads();
  butterflies(line, tw, t, 1);
  for (int h = 0; h < 2; ++h) {
    const int i = t + h * 256;
    const float2 z = line[i];
    spec[iy * kN + i] = make_float2(z.x * kUnitary + 0.0f, z.y * kUnitary + 0.0f);
  }
}

// Passes 3-5 (wave.ts:174-245, 252-322): block b holds column b and its
// mirror column (512 - b) mod 512 (block 0: columns 0 and 256, each its own
// mirror), 512 threads, threads 0-255 on the first column and 256-511 on the
// second.  Forward FFT along y, the propagation of every (kx, kz) from
// Z(kx, kz) and Z(-kx, -kz) (both in this block), inverse FFT, stored back.
__global__ void __launch_bounds__(512) k_wave_columns(const StepParams* __restrict__ Pp, float2* __restrict__ spec) {
  __shared__ float2 col[2][kN];
  __shared__ float2 twf[kHalf], twi[kHalf];
  const int t = threadIdx.x, side = t >> 8, tl = t & 255;
  const int cA = blockIdx.x, cB = blockIdx.x == 0 ? kHalf : kN - blockIdx.x;
  const int cx = side ? cB : cA;
  // mirror of this thread's column: the other side, except in block 0
  const int mside = blockIdx.x == 0 ? side : 1 - side;
  make_twiddles(twf, -1.0f, t, 512);
  make_twiddles(twi, 1.0f, t, 512);
  for (int h = 0; h < 2; ++h) {
    const int i = tl + h * 256;
    col[side][rev9((uint32_t)i)] = spec[i * kN + cx];
  }
  __syncthreads();
  butterflies(col[side], twf, tl, 2);  // the two halves run the same stage sequence
  for (int h = 0; h < 2; ++h) {
    const int i = tl + h * 256;
    const float2 z = col[side][i];
    col[side][i] = make_float2(z.x * kUnitary + 0.0f, z.y * kUnitary + 0.0f);
  }
  __syncthreads();
  // propagation of (ux = cx, uy) for uy = tl and tl + 256
  const float* U = Pp->U;
  const float dt = dob_clampf(U[38], 0.0f, 0.025f);
  const float depthH = U[54] - U[53];
  const float twoPiOverL = (float)(6.28318530718 / 3.2);
  float2 outv[2];
  for (int h = 0; h < 2; ++h) {
    const int uy = tl + h * 256;
    if ((cx == 0 && uy == 0) || cx == kHalf || uy == kHalf) { outv[h] = make_float2(0.0f, 0.0f); continue; }
    const int ny = (kN - uy) & (kN - 1);
    const float2 fp = col[side][uy], fn = col[mside][ny];
    const float ehx = 0.5f * (fp.x + fn.x), ehy = 0.5f * (fp.y - fn.y);
    const float vhx = 0.5f * (fp.y + fn.y), vhy = 0.5f * (-fp.x + fn.x);
    const float mx = (float)(cx > kHalf ? cx - kN : cx), mz = (float)(uy > kHalf ? uy - kN : uy);
    const float kx = mx * twoPiOverL, kz = mz * twoPiOverL;
    const float k2 = kx * kx + kz * kz;
    const float k = dob_sqrt(k2);
    const float tanhKH = dob_tanh(dob_minf(k * depthH, 12.0f));
    const float omega = dob_sqrt(dob_maxf((0.84f * k + 0.0024f * k * k2) * tanhKH, 1e-8f));
    const float viscRate = 0.36f + 0.00018f * k2;
    const float nyquistRoll = 1.0f - dob_smoothstep(335.0f, 465.0f, k);
    const float damp = dob_exp(-viscRate * dt) * nyquistRoll;
    const float phase = omega * dt;
    float sinP, cosP;
    dob_sincos(phase, &sinP, &cosP);
    const float so = sinP / omega, os = omega * sinP;
    const float enx = damp * (ehx * cosP + vhx * so), eny = damp * (ehy * cosP + vhy * so);
    const float vnx = damp * (-ehx * os + vhx * cosP), vny = damp * (-ehy * os + vhy * cosP);
    outv[h] = make_float2(enx - vny, eny + vnx);
  }
  __syncthreads();  // every mirror value is read before any is overwritten
  for (int h = 0; h < 2; ++h) col[side][rev9((uint32_t)(tl + h * 256))] = outv[h];
  __syncthreads();
  butterflies(col[side], twi, tl, 2);
  for (int h = 0; h < 2; ++h) {
    const int i = tl + h * 256;
    const float2 z = col[side][i];
    spec[i * kN + cx] = make_float2(z.x * kUnitary + 0.0f, z.y * kUnitary + 0.0f);
  }
}

// Pass 6 (wave.ts:174-245, inverse, rows): one row per block, in place.
__global__ void __launch_bounds__(256) k_wave_rows_inverse(float2* __restrict__ spec) {
  __shared__ float2 line[kN];
  __shared__ float2 tw[kHalf];
  const int t = threadIdx.x, iy = blockIdx.x;
  make_twiddles(tw, 1.0f, t, 256);
  for (int h = 0; h < 2; ++h) {
    const int i = t + h * 256;
    line[rev9((uint32_t)i)] = spec[iy * kN + i];
  }
  __syncthreads();
  butterflies(line, tw, t, 1);
  for (int h = 0; h < 2; ++h) {
    const int i = t + h * 256;
    const float2 z = line[i];
    spec[iy * kN + i] = make_float2(z.x * kUnitary + 0.0f, z.y * kUnitary + 0.0f);
  }
}

// Pass 7 (wave.ts:330-388): (eta, deta/dt, 9-point Laplacian of eta, film),
// faded at the border and rounded to half (the rgba16float wave texture).
__global__ void __launch_bounds__(256) k_wave_finalize(const float2* __restrict__ spec,
                                                       const float* __restrict__ film, float4* __restrict__ wave) {
  const int ix = blockIdx.x * 32 + (threadIdx.x & 31), iy = blockIdx.y * 8 + (threadIdx.x >> 5);
  auto eta = [&](int x, int y) {
    x = dob_clampi(x, 0, kN - 1);
    y = dob_clampi(y, 0, kN - 1);
    return __ldg(&spec[y * kN + x].x);
  };
  const float2 p = __ldg(&spec[iy * kN + ix]);
  const float s1 = ((eta(ix, iy + 1) + eta(ix, iy - 1)) + eta(ix + 1, iy)) + eta(ix - 1, iy);
  const float s2 = ((eta(ix + 1, iy + 1) + eta(ix - 1, iy + 1)) + eta(ix + 1, iy - 1)) + eta(ix - 1, iy - 1);
  const float lap = ((0.20f * s1 + 0.05f * s2) - p.x) * 4.0f;
  const float borderZero = 1.0f - dob_smoothstep(1.22f, 1.56f, length2f(wave_world(ix), wave_world(iy)));
  wave[iy * kN + ix] = make_float4(dob_round_f16(dob_clampf(p.x * borderZero, -0.14f, 0.14f)),
                                   dob_round_f16(dob_clampf(p.y * borderZero, -1.8f, 1.8f)),
                                   dob_round_f16(lap * borderZero),
                                   dob_round_f16(__ldg(&film[iy * kN + ix]) * borderZero));
}

}  // namespace

void launch_wave_step(const DevState& s, cudaStream_t st) {
  DOB_VEL_DISPATCH(s.prec, k_wave_force_rows<VS><<<kN, 256, 0, st>>>(s.g, s.params, s.wave, (const VS*)s.v,
                                                                     s.wfilm, s.wspec));
  k_wave_columns<<<kHalf, 512, 0, st>>>(s.params, s.wspec);
  k_wave_rows_inverse<<<kN, 256, 0, st>>>(s.wspec);
  k_wave_finalize<<<dim3(kN / 32, kN / 8), 256, 0, st>>>(s.wspec, s.wfilm, s.wave);
}

}  // namespace dob
