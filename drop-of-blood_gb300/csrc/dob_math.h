// dob_math.h — the library's own single-precision elementary functions and
// the WGSL built-ins the reference kernels use, written once for host and
// device so that a host build and a device build of the same expression give
// the same bits (when both are compiled without FMA contraction).
//
// Methods (all from the mathematics, no vendor code or constants):
//   sin/cos : Cody–Waite reduction by pi/2 split into three 12-bit parts,
//             Taylor series to r^11 / r^12 on [-pi/4, pi/4];
//   exp     : k = rint(x/ln2), two-part ln2 reduction, Taylor to r^8,
//             scaling by 2^k built from the exponent field;
//   log     : m in [sqrt(1/2), sqrt(2)), log m = 2 atanh((m-1)/(m+1)) series;
//   atan2   : octant folding, table of tan(i*pi/16), Taylor series of atan
//             on |t| <= tan(pi/32);
//   tanh    : expm1(2|x|) / (expm1(2|x|) + 2) with a Taylor expm1 near 0;
//   pow     : exp(y * log x) for x > 0 (the reference only takes pow of
//             non-negative values, particles.ts:150, 326; fluid.ts:236).
// WGSL built-ins follow the WGSL specification's definitions:
//   mix(a,b,t) = a*(1-t) + b*t; smoothstep = t*t*(3-2t), t = clamp((x-e0)/(e1-e0));
//   clamp(e,lo,hi) = min(max(e,lo),hi); fract(x) = x - floor(x);
//   round = half-to-even (rintf).
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define DOB_HD __host__ __device__ __forceinline__
#else
#define DOB_HD static inline
#endif

// ---- bit casts ------------------------------------------------------------
DOB_HD uint32_t dob_f2u(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  uint32_t u;
  memcpy(&u, &x, 4);
  return u;
#endif
}
DOB_HD float dob_u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float x;
  memcpy(&x, &u, 4);
  return x;
#endif
}

// ---- WGSL scalar built-ins ---------------------------------------------------
DOB_HD float dob_minf(float a, float b) { return a < b ? a : b; }
DOB_HD float dob_maxf(float a, float b) { return a > b ? a : b; }
DOB_HD float dob_clampf(float e, float lo, float hi) { return dob_minf(dob_maxf(e, lo), hi); }
DOB_HD int dob_clampi(int e, int lo, int hi) { return e < lo ? lo : (e > hi ? hi : e); }
// On the device one fixed rounding sequence (the rounded a (1 - t), then one
// FMA with b t), so every kernel that interpolates the same taps gets the
// same bits whatever the compiler would contract.  A translation unit that
// must match the host's unfused arithmetic (compiled with -fmad=false)
// defines DOB_UNFUSED before including this header.
DOB_HD float dob_mix(float a, float b, float t) {
#if defined(__CUDA_ARCH__) && !defined(DOB_UNFUSED)
  return __fmaf_rn(b, t, __fmul_rn(a, 1.0f - t));
#else
  return a * (1.0f - t) + b * t;
#endif
}
DOB_HD float dob_smoothstep(float e0, float e1, float x) {
  float t = dob_clampf((x - e0) / (e1 - e0), 0.0f, 1.0f);
  return t * t * (3.0f - 2.0f * t);
}
DOB_HD float dob_fract(float x) { return x - floorf(x); }
DOB_HD float dob_round(float x) { return rintf(x); }
DOB_HD float dob_sqrt(float x) {
#if defined(__CUDA_ARCH__)
  return __fsqrt_rn(x);
#else
  return sqrtf(x);
#endif
}
DOB_HD float dob_div(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fdiv_rn(a, b);
#else
  return a / b;
#endif
}

// 2^n as a float for n in [-126, 127].
DOB_HD float dob_pow2i(int n) { return dob_u2f((uint32_t)(n + 127) << 23); }

// ---- sin / cos ----------------------------------------------------------------
DOB_HD void dob_sincos(float x, float* s, float* c) {
  const float k = rintf(x * 0.636619747f);  // 2/pi
  // pi/2 = 1.5703125 + 4.837512969970703e-4 + 7.549790126404332e-8 (12-bit parts)
  float r = x - k * 1.5703125f;
  r = r - k * 4.837512969970703e-4f;
  r = r - k * 7.549790126404332e-8f;
  const int q = ((int)k) & 3;
  const float r2 = r * r;
  float ps = -2.5052108385441718e-8f;          // -1/11!
  ps = 2.7557319223985893e-6f + r2 * ps;       //  1/9!
  ps = -1.984126984126984e-4f + r2 * ps;       // -1/7!
  ps = 8.333333333333333e-3f + r2 * ps;        //  1/5!
  ps = -0.16666666666666666f + r2 * ps;        // -1/3!
  const float sp = r + (r * r2) * ps;
  float pc = 2.08767569878681e-9f;             //  1/12!
  pc = -2.755731922398589e-7f + r2 * pc;       // -1/10!
  pc = 2.48015873015873e-5f + r2 * pc;         //  1/8!
  pc = -1.388888888888889e-3f + r2 * pc;       // -1/6!
  pc = 4.1666666666666664e-2f + r2 * pc;       //  1/4!
  pc = -0.5f + r2 * pc;                        // -1/2!
  const float cp = 1.0f + r2 * pc;
  if (q == 0) { *s = sp; *c = cp; }
  else if (q == 1) { *s = cp; *c = -sp; }
  else if (q == 2) { *s = -sp; *c = -cp; }
  else { *s = -cp; *c = sp; }
}
DOB_HD float dob_sin(float x) { float s, c; dob_sincos(x, &s, &c); return s; }
DOB_HD float dob_cos(float x) { float s, c; dob_sincos(x, &s, &c); return c; }

// ---- exp / expm1 / log / pow ---------------------------------------------------
DOB_HD float dob_exp(float x) {
  if (x != x) return x;
  if (x > 88.7228394f) return dob_u2f(0x7f800000u);
  if (x < -103.972084f) return 0.0f;
  const float k = rintf(x * 1.44269502f);      // 1/ln2
  // ln2 = 0.693115234375 + 3.194618329871446e-05 (12-bit high part)
  float r = x - k * 0.693115234375f;
  r = r - k * 3.194618329871446e-05f;
  float p = 2.48015873015873e-5f;              // 1/8!
  p = 1.984126984126984e-4f + r * p;           // 1/7!
  p = 1.388888888888889e-3f + r * p;           // 1/6!
  p = 8.333333333333333e-3f + r * p;           // 1/5!
  p = 4.1666666666666664e-2f + r * p;          // 1/4!
  p = 0.16666666666666666f + r * p;            // 1/3!
  p = 0.5f + r * p;
  p = 1.0f + r * p;
  p = 1.0f + r * p;
  const int ki = (int)k;
  if (ki > 127) return p * dob_pow2i(127) * dob_pow2i(ki - 127);
  if (ki < -126) return p * dob_pow2i(-126) * dob_pow2i(ki + 126);
  return p * dob_pow2i(ki);
}

DOB_HD float dob_expm1(float z) {
  if (fabsf(z) < 0.35f) {
    float p = 2.7557319223985893e-6f;          // 1/9!
    p = 2.48015873015873e-5f + z * p;
    p = 1.984126984126984e-4f + z * p;
    p = 1.388888888888889e-3f + z * p;
    p = 8.333333333333333e-3f + z * p;
    p = 4.1666666666666664e-2f + z * p;
    p = 0.16666666666666666f + z * p;
    p = 0.5f + z * p;
    return z + (z * z) * p;
  }
  return dob_exp(z) - 1.0f;
}

DOB_HD float dob_log(float x) {
  if (x != x) return x;
  if (x < 0.0f) return dob_u2f(0x7fc00000u);
  if (x == 0.0f) return dob_u2f(0xff800000u);
  uint32_t u = dob_f2u(x);
  if (u >= 0x7f800000u) return x;
  int e = 0;
  if (u < 0x00800000u) {  // subnormal
    x = x * 8388608.0f;   // 2^23
    u = dob_f2u(x);
    e = -23;
  }
  e += (int)((u >> 23) & 0xffu) - 127;
  float m = dob_u2f((u & 0x007fffffu) | 0x3f800000u);
  if (m > 1.41421356f) { m = m * 0.5f; e += 1; }
  const float s = (m - 1.0f) / (m + 1.0f);
  const float s2 = s * s;
  float p = 0.07692307692307693f;              // 1/13
  p = 0.09090909090909091f + s2 * p;           // 1/11
  p = 0.1111111111111111f + s2 * p;            // 1/9
  p = 0.14285714285714285f + s2 * p;           // 1/7
  p = 0.2f + s2 * p;                           // 1/5
  p = 0.3333333333333333f + s2 * p;            // 1/3
  p = 1.0f + s2 * p;
  const float lm = (2.0f * s) * p;
  const float fe = (float)e;
  return fe * 0.693115234375f + (lm + fe * 3.194618329871446e-05f);
}

DOB_HD float dob_pow(float x, float y) {
  if (y == 0.0f) return 1.0f;
  if (x == 0.0f) return y > 0.0f ? 0.0f : dob_u2f(0x7f800000u);
  if (x < 0.0f) return dob_u2f(0x7fc00000u);
  return dob_exp(y * dob_log(x));
}

// ---- atan2 / tanh -------------------------------------------------------------
DOB_HD float dob_atan2(float y, float x) {
  const float ax = fabsf(x), ay = fabsf(y);
  if (ax == 0.0f && ay == 0.0f) return 0.0f;
  const bool swap = ay > ax;
  const float a = swap ? ax / ay : ay / ax;  // [0, 1]
  float c, th;
  if (a < 0.09849140048027039f) { c = 0.0f; th = 0.0f; }
  else if (a < 0.3033466935157776f) { c = 0.1989123672246933f; th = 0.19634954631328583f; }
  else if (a < 0.534511148929596f) { c = 0.4142135679721832f; th = 0.39269909262657166f; }
  else if (a < 0.8206787705421448f) { c = 0.6681786179542542f; th = 0.5890486240386963f; }
  else { c = 1.0f; th = 0.7853981852531433f; }
  const float t = (a - c) / (1.0f + a * c);
  const float t2 = t * t;
  float p = 0.07692307692307693f;              //  1/13
  p = -0.09090909090909091f + t2 * p;          // -1/11
  p = 0.1111111111111111f + t2 * p;            //  1/9
  p = -0.14285714285714285f + t2 * p;          // -1/7
  p = 0.2f + t2 * p;                           //  1/5
  p = -0.3333333333333333f + t2 * p;           // -1/3
  float r = th + (t + (t * t2) * p);
  if (swap) r = 1.5707963705062866f - r;
  if (x < 0.0f) r = 3.1415927410125732f - r;
  if (y < 0.0f) r = -r;
  return r;
}

DOB_HD float dob_tanh(float x) {
  const float ax = fabsf(x);
  if (ax > 9.0f) return x < 0.0f ? -1.0f : 1.0f;
  const float e = dob_expm1(2.0f * ax);
  const float t = e / (e + 2.0f);
  return x < 0.0f ? -t : t;
}

// ---- binary16 / bfloat16 storage rounding (host restatement of IEEE RNE) ------
DOB_HD uint16_t dob_f32_to_f16_bits(float x) {
  const uint32_t u = dob_f2u(x);
  const uint32_t sign = (u >> 16) & 0x8000u;
  const uint32_t a = u & 0x7fffffffu;
  if (a >= 0x7f800000u) return (uint16_t)(sign | (a > 0x7f800000u ? 0x7e00u : 0x7c00u));
  if (a >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);  // >= 65520 rounds to inf
  if (a >= 0x38800000u) {                                   // normal binary16
    const uint32_t mant = a & 0x7fffffu;
    const uint32_t e = (a >> 23) - 127u + 15u;
    uint32_t h = (e << 10) | (mant >> 13);
    const uint32_t rem = mant & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h++;
    return (uint16_t)(sign | h);
  }
  if (a <= 0x33000000u) return (uint16_t)sign;              // <= 2^-25 rounds to 0
  const uint32_t e = a >> 23;                               // biased, <= 112
  const uint32_t m = (a & 0x7fffffu) | 0x800000u;
  const uint32_t shift = 126u - e;                          // 14 .. 24
  uint32_t h = m >> shift;
  const uint32_t rem = m & ((1u << shift) - 1u);
  const uint32_t half = 1u << (shift - 1u);
  if (rem > half || (rem == half && (h & 1u))) h++;
  return (uint16_t)(sign | h);
}

DOB_HD float dob_f16_bits_to_f32(uint16_t h) {
  const uint32_t sign = ((uint32_t)h & 0x8000u) << 16;
  const uint32_t e = ((uint32_t)h >> 10) & 0x1fu;
  const uint32_t m = (uint32_t)h & 0x3ffu;
  if (e == 0x1fu) return dob_u2f(sign | 0x7f800000u | (m << 13));
  if (e == 0u) {
    if (m == 0u) return dob_u2f(sign);
    const float v = (float)m * 5.9604644775390625e-8f;     // m * 2^-24, exact
    return sign ? -v : v;
  }
  return dob_u2f(sign | ((e + 112u) << 23) | (m << 13));
}

DOB_HD float dob_round_f16(float x) { return dob_f16_bits_to_f32(dob_f32_to_f16_bits(x)); }

DOB_HD uint16_t dob_f32_to_bf16_bits(float x) {
  const uint32_t u = dob_f2u(x);
  if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x40u);
  const uint32_t r = u + 0x7fffu + ((u >> 16) & 1u);
  return (uint16_t)(r >> 16);
}
DOB_HD float dob_bf16_bits_to_f32(uint16_t b) { return dob_u2f((uint32_t)b << 16); }
DOB_HD float dob_round_bf16(float x) { return dob_bf16_bits_to_f32(dob_f32_to_bf16_bits(x)); }

// ---- seeded noise for sphere injection ------------------------------------------
// SplitMix64 (Steele, Lea & Flood, "Fast splittable pseudorandom number
// generators", OOPSLA 2014) and a Box-Muller normal deviate in float built
// from the functions above, so host and device draw the same numbers.
DOB_HD uint64_t dob_splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
// N(0,1) for MAC face `index`, velocity component `comp`.
DOB_HD float dob_sphere_noise(uint64_t seed, uint64_t index, int comp) {
  const uint64_t key = seed * 0x100000001B3ull + (index * 3ull + (uint64_t)comp) * 2ull;
  const uint32_t a = (uint32_t)(dob_splitmix64(key) >> 40);
  const uint32_t b = (uint32_t)(dob_splitmix64(key + 1ull) >> 40);
  const float u1 = ((float)a + 1.0f) * 5.9604644775390625e-8f;  // (0, 1]
  const float u2 = (float)b * 5.9604644775390625e-8f;          // [0, 1)
  const float rad = dob_sqrt(-2.0f * dob_log(u1));
  return rad * dob_cos(6.28318548f * u2);
}

// ---- small 3-vector for the WGSL vec3<f32> expressions ------------------------
struct dob_v3 {
  float x, y, z;
};
DOB_HD dob_v3 v3(float x, float y, float z) { dob_v3 r; r.x = x; r.y = y; r.z = z; return r; }
DOB_HD dob_v3 operator+(dob_v3 a, dob_v3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
DOB_HD dob_v3 operator-(dob_v3 a, dob_v3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
DOB_HD dob_v3 operator*(dob_v3 a, dob_v3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
DOB_HD dob_v3 operator/(dob_v3 a, dob_v3 b) { return v3(a.x / b.x, a.y / b.y, a.z / b.z); }
DOB_HD dob_v3 operator*(dob_v3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
DOB_HD dob_v3 operator*(float s, dob_v3 a) { return v3(s * a.x, s * a.y, s * a.z); }
DOB_HD dob_v3 operator/(dob_v3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
DOB_HD dob_v3 operator-(dob_v3 a) { return v3(-a.x, -a.y, -a.z); }
DOB_HD float dot3(dob_v3 a, dob_v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
DOB_HD float length3(dob_v3 a) { return dob_sqrt(dot3(a, a)); }
DOB_HD dob_v3 cross3(dob_v3 a, dob_v3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
DOB_HD dob_v3 clamp3(dob_v3 a, float lo, float hi) {
  return v3(dob_clampf(a.x, lo, hi), dob_clampf(a.y, lo, hi), dob_clampf(a.z, lo, hi));
}
DOB_HD dob_v3 normalize3(dob_v3 a) { return a / length3(a); }
DOB_HD dob_v3 mix3(dob_v3 a, dob_v3 b, float t) {
  return v3(dob_mix(a.x, b.x, t), dob_mix(a.y, b.y, t), dob_mix(a.z, b.z, t));
}
DOB_HD float length2f(float x, float y) { return dob_sqrt(x * x + y * y); }

// Soft-edged sphere of radius r and edge width h around c at point p: the
// weight is 1 for |p - c| <= r - h/2, 0 for |p - c| >= r + h/2 and the
// smoothstep t^2 (3 - 2t), t = (r + h/2 - |p - c|) / h, in between, so it is
// continuously differentiable in c; *g receives d weight / d c.  Compiled
// without FMA contraction on the device, so host and device agree bit for bit.
DOB_HD float dob_soft_sphere(dob_v3 p, dob_v3 c, float r, float h, dob_v3* g) {
  const dob_v3 dpc = p - c;
  const float d = length3(dpc);
  const float t = (r + 0.5f * h - d) / h;
  if (!(t > 0.0f) || t >= 1.0f) {
    *g = v3(0.0f, 0.0f, 0.0f);
    return t >= 1.0f ? 1.0f : 0.0f;
  }
  const float s = d > 0.0f ? 6.0f * t * (1.0f - t) / (h * d) : 0.0f;
  *g = dpc * s;
  return t * t * (3.0f - 2.0f * t);
}
