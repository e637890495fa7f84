// dob_oracle.cpp — TEST INFRASTRUCTURE (the oracle), not part of the product.
//
// CPU restatement of the drop-of-blood staggered-MAC fluid step, templated on
// the arithmetic type (float = the reference's f32 arithmetic; double = the
// FP64 oracle).  Every stage cites the reference file:line it follows.  The
// reference is TypeScript + WGSL run by a browser's WebGPU, which cannot run
// here, so this restatement is the checker; texture filtering is restated as
// WebGPU linear/clamp-to-edge sampling (texel = uvw*dims - 0.5) with FP32
// weights, and rgba16float stores as IEEE binary16 round-to-nearest-even.
//
// It includes the product's math header (own sin/cos/exp/log/atan2/tanh and
// the WGSL built-ins) on purpose: those play the role of libm for both sides,
// so the float build of the parcel stage reproduces the device bits.
#include "dob_oracle.h"

#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "../drop-of-blood_gb300/csrc/dob_math.h"

namespace {

constexpr int kMaxDrops = 8;
constexpr int kWaveN = 512;
constexpr float kSplatScale = 65536.0f;
constexpr float kParcelMass = 0.13400f;  // INITIAL_PARCEL_VOXEL_MASS.toFixed(5), particles.ts:14,177

// ---- precision-generic helpers -----------------------------------------------
inline float Sin(float x) { return dob_sin(x); }
inline double Sin(double x) { return sin(x); }
inline float Cos(float x) { return dob_cos(x); }
inline double Cos(double x) { return cos(x); }
inline float Exp(float x) { return dob_exp(x); }
inline double Exp(double x) { return exp(x); }
inline float Pow(float x, float y) { return dob_pow(x, y); }
inline double Pow(double x, double y) { return x == 0.0 ? (y > 0 ? 0.0 : 1.0) : pow(x, y); }
inline float Atan2(float y, float x) { return dob_atan2(y, x); }
inline double Atan2(double y, double x) { return (x == 0.0 && y == 0.0) ? 0.0 : atan2(y, x); }
inline float Tanh(float x) { return dob_tanh(x); }
inline double Tanh(double x) { return tanh(x); }
inline float Sqrt(float x) { return dob_sqrt(x); }
inline double Sqrt(double x) { return sqrt(x); }
inline float Floor(float x) { return floorf(x); }
inline double Floor(double x) { return floor(x); }
inline float Round(float x) { return rintf(x); }
inline double Round(double x) { return rint(x); }

template <class R> inline R Min(R a, R b) { return a < b ? a : b; }
template <class R> inline R Max(R a, R b) { return a > b ? a : b; }
template <class R> inline R Clamp(R e, R lo, R hi) { return Min(Max(e, lo), hi); }
template <class R> inline R Mix(R a, R b, R t) { return a * (R(1) - t) + b * t; }
template <class R> inline R Smooth(R e0, R e1, R x) {
  R t = Clamp((x - e0) / (e1 - e0), R(0), R(1));
  return t * t * (R(3) - R(2) * t);
}
template <class R> inline R Fract(R x) { return x - Floor(x); }
inline int ClampI(int e, int lo, int hi) { return e < lo ? lo : (e > hi ? hi : e); }

template <class R> struct V3 {
  R x, y, z;
};
template <class R> inline V3<R> mk(R x, R y, R z) { return V3<R>{x, y, z}; }
template <class R> inline V3<R> operator+(V3<R> a, V3<R> b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class R> inline V3<R> operator-(V3<R> a, V3<R> b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class R> inline V3<R> operator*(V3<R> a, V3<R> b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
template <class R> inline V3<R> operator/(V3<R> a, V3<R> b) { return mk(a.x / b.x, a.y / b.y, a.z / b.z); }
template <class R> inline V3<R> operator*(V3<R> a, R s) { return mk(a.x * s, a.y * s, a.z * s); }
template <class R> inline V3<R> operator*(R s, V3<R> a) { return mk(s * a.x, s * a.y, s * a.z); }
template <class R> inline V3<R> operator/(V3<R> a, R s) { return mk(a.x / s, a.y / s, a.z / s); }
template <class R> inline R Dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> inline R Len(V3<R> a) { return Sqrt(Dot(a, a)); }
template <class R> inline V3<R> Cross(V3<R> a, V3<R> b) {
  return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <class R> inline V3<R> ClampV(V3<R> a, R lo, R hi) {
  return mk(Clamp(a.x, lo, hi), Clamp(a.y, lo, hi), Clamp(a.z, lo, hi));
}
template <class R> inline V3<R> MixV(V3<R> a, V3<R> b, R t) {
  return mk(Mix(a.x, b.x, t), Mix(a.y, b.y, t), Mix(a.z, b.z, t));
}
template <class R> inline V3<R> Normalize(V3<R> a) { return a / Len(a); }
template <class R> inline R Len2(R x, R y) { return Sqrt(x * x + y * y); }
// dob_soft_sphere (dob_math.h) in R arithmetic: same operations, so the
// float instance has the device's bits
template <class R> inline R SoftSphere(V3<R> p, V3<R> c, R r, R h, V3<R>& g) {
  const V3<R> dpc = p - c;
  const R d = Len(dpc);
  const R t = (r + R(0.5) * h - d) / h;
  if (!(t > R(0)) || t >= R(1)) {
    g = mk(R(0), R(0), R(0));
    return t >= R(1) ? R(1) : R(0);
  }
  const R sc = d > R(0) ? R(6) * t * (R(1) - t) / (h * d) : R(0);
  g = dpc * sc;
  return t * t * (R(3) - R(2) * t);
}

struct Dims {
  int nx = 0, ny = 0, nz = 0;
  size_t n() const { return (size_t)nx * ny * nz; }
  size_t at(int x, int y, int z) const { return ((size_t)z * ny + y) * nx + x; }
};

// Trilinear sample with WebGPU linear/clamp-to-edge semantics.
struct Tap {
  size_t i[8];
  float fx, fy, fz;
};
template <class R> struct Taps {
  size_t i[8];
  R fx, fy, fz;
  size_t lx, ly, lz;  // element offset base -> base - 1 (0 at the lower edge)
  size_t hx, hy, hz;  // element offset base + 1 -> base + 2 (0 at the upper edge)
};
template <class R> inline Taps<R> taps(const Dims& d, R u, R v, R w) {
  Taps<R> t;
  const R cx = u * R(d.nx) - R(0.5), cy = v * R(d.ny) - R(0.5), cz = w * R(d.nz) - R(0.5);
  const R bx = Floor(cx), by = Floor(cy), bz = Floor(cz);
  t.fx = cx - bx; t.fy = cy - by; t.fz = cz - bz;
  const int ix = (int)bx, iy = (int)by, iz = (int)bz;
  const int x0 = ClampI(ix, 0, d.nx - 1), x1 = ClampI(ix + 1, 0, d.nx - 1);
  const int y0 = ClampI(iy, 0, d.ny - 1), y1 = ClampI(iy + 1, 0, d.ny - 1);
  const int z0 = ClampI(iz, 0, d.nz - 1), z1 = ClampI(iz + 1, 0, d.nz - 1);
  t.i[0] = d.at(x0, y0, z0); t.i[1] = d.at(x1, y0, z0);
  t.i[2] = d.at(x0, y1, z0); t.i[3] = d.at(x1, y1, z0);
  t.i[4] = d.at(x0, y0, z1); t.i[5] = d.at(x1, y0, z1);
  t.i[6] = d.at(x0, y1, z1); t.i[7] = d.at(x1, y1, z1);
  t.lx = x0 > 0 ? 1 : 0;
  t.ly = y0 > 0 ? (size_t)d.nx : 0;
  t.lz = z0 > 0 ? (size_t)d.nx * d.ny : 0;
  t.hx = x0 + 2 <= d.nx - 1 ? 1 : 0;
  t.hy = y0 + 2 <= d.ny - 1 ? (size_t)d.nx : 0;
  t.hz = z0 + 2 <= d.nz - 1 ? (size_t)d.nx * d.ny : 0;
  return t;
}
template <class R> inline R lerp8(const Taps<R>& t, const R* a) {
  const R x00 = Mix(a[t.i[0]], a[t.i[1]], t.fx);
  const R x10 = Mix(a[t.i[2]], a[t.i[3]], t.fx);
  const R x01 = Mix(a[t.i[4]], a[t.i[5]], t.fx);
  const R x11 = Mix(a[t.i[6]], a[t.i[7]], t.fx);
  const R y0 = Mix(x00, x10, t.fy);
  const R y1 = Mix(x01, x11, t.fy);
  return Mix(y0, y1, t.fz);
}

int g_threads = 0;

// Dense (pseudo-)inverse of the coarsest operator A = -L / h2 (L: 7-point
// graph Laplacian with the level's boundary terms; the reference mode counts
// the +y face of every cell, the Dirichlet ghost above the top), natural cell
// order, in double.  Gauss-Jordan on A + J/n (closed box: J/n restores the
// null space, removed again afterwards), symmetrised: O(n^3), used to check
// the separable form below on small grids.
inline std::vector<double> cinv_direct(const Dims& c, double hh, int ref) {
  const int n = (int)c.n();
  std::vector<double> a((size_t)n * n, 0.0), inv((size_t)n * n, 0.0);
  for (int z = 0; z < c.nz; ++z)
    for (int y = 0; y < c.ny; ++y)
      for (int x = 0; x < c.nx; ++x) {
        const int i = (int)c.at(x, y, z);
        double diag = ref ? 1.0 : 0.0;
        auto nb = [&](int xx, int yy, int zz, bool count) {
          a[(size_t)i * n + c.at(xx, yy, zz)] += 1.0 / hh;
          if (count) diag += 1.0;
        };
        if (x > 0) nb(x - 1, y, z, true);
        if (x < c.nx - 1) nb(x + 1, y, z, true);
        if (y > 0) nb(x, y - 1, z, true);
        if (y < c.ny - 1) nb(x, y + 1, z, !ref);
        if (z > 0) nb(x, y, z - 1, true);
        if (z < c.nz - 1) nb(x, y, z + 1, true);
        a[(size_t)i * n + i] -= diag / hh;
      }
  if (!ref)
    for (auto& v : a) v += 1.0 / n;
  for (int i = 0; i < n; ++i) inv[(size_t)i * n + i] = 1.0;
  for (int col = 0; col < n; ++col) {
    int piv = col;
    for (int r = col + 1; r < n; ++r)
      if (std::fabs(a[(size_t)r * n + col]) > std::fabs(a[(size_t)piv * n + col])) piv = r;
    if (piv != col)
      for (int k = 0; k < n; ++k) {
        std::swap(a[(size_t)piv * n + k], a[(size_t)col * n + k]);
        std::swap(inv[(size_t)piv * n + k], inv[(size_t)col * n + k]);
      }
    const double d = a[(size_t)col * n + col];
    for (int k = 0; k < n; ++k) { a[(size_t)col * n + k] /= d; inv[(size_t)col * n + k] /= d; }
    for (int r = 0; r < n; ++r) {
      if (r == col) continue;
      const double f = a[(size_t)r * n + col];
      if (f == 0.0) continue;
      for (int k = 0; k < n; ++k) {
        a[(size_t)r * n + k] -= f * a[(size_t)col * n + k];
        inv[(size_t)r * n + k] -= f * inv[(size_t)col * n + k];
      }
    }
  }
  std::vector<double> out((size_t)n * n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      out[(size_t)i * n + j] = 0.5 * (inv[(size_t)i * n + j] + inv[(size_t)j * n + i]) - (ref ? 0.0 : 1.0 / n);
  return out;
}
// The same inverse from the eigenpairs of the three axis operators (L is
// their Kronecker sum): closed box and reference x/z, Neumann at both ends:
// vectors cos(pi k (i + 1/2) / m), values 2 - 2 cos(pi k / m); reference y,
// Neumann below and the Dirichlet ghost above: cos(t (i + 1/2)),
// t = pi (k + 1/2) / (m + 1/2), 2 - 2 cos t.  M = -h2 sum over the modes with
// a nonzero value of phi phi^T / value (the closed box's constant mode is
// left out: the minimum-norm inverse).  Column b: its mode coefficients
// phi(b) / value, taken back to cells one axis at a time,
// O(n (nx + ny + nz)) per column.
inline std::vector<double> cinv_separable(const Dims& c, double hh, int ref) {
  const double pi = 3.14159265358979323846;
  auto eig = [&](int m, bool dir, std::vector<double>& V, std::vector<double>& mu) {
    V.assign((size_t)m * m, 0.0);
    mu.assign(m, 0.0);
    for (int k = 0; k < m; ++k) {
      const double t = dir ? pi * (k + 0.5) / (m + 0.5) : pi * k / m;
      mu[k] = (!dir && k == 0) ? 0.0 : 2.0 - 2.0 * std::cos(t);
      double s2 = 0.0;
      for (int i = 0; i < m; ++i) s2 += std::cos(t * (i + 0.5)) * std::cos(t * (i + 0.5));
      for (int i = 0; i < m; ++i) V[(size_t)k * m + i] = std::cos(t * (i + 0.5)) / std::sqrt(s2);
    }
  };
  std::vector<double> X, Y, Z, mx, my, mz;
  const int nx = c.nx, ny = c.ny, nz = c.nz;
  eig(nx, false, X, mx);
  eig(ny, ref != 0, Y, my);
  eig(nz, false, Z, mz);
  const size_t n = c.n();
  std::vector<double> out(n * n, 0.0);
#pragma omp parallel for schedule(dynamic)
  for (long b = 0; b < (long)n; ++b) {
    const int bx = (int)(b % nx), by = (int)((b / nx) % ny), bz = (int)(b / ((size_t)nx * ny));
    std::vector<double> w(n), t(n);
    for (int k = 0; k < nz; ++k)  // mode coefficients, indexed (k, j, i)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          const double m = mx[i] + my[j] + mz[k];
          w[c.at(i, j, k)] = m > 0.0 ? X[(size_t)i * nx + bx] * Y[(size_t)j * ny + by] * Z[(size_t)k * nz + bz] / m : 0.0;
        }
    for (int k = 0; k < nz; ++k)  // modes i -> cells x
      for (int j = 0; j < ny; ++j)
        for (int x = 0; x < nx; ++x) {
          double acc = 0.0;
          for (int i = 0; i < nx; ++i) acc += X[(size_t)i * nx + x] * w[c.at(i, j, k)];
          t[c.at(x, j, k)] = acc;
        }
    for (int k = 0; k < nz; ++k)  // modes j -> cells y
      for (int y = 0; y < ny; ++y)
        for (int x = 0; x < nx; ++x) {
          double acc = 0.0;
          for (int j = 0; j < ny; ++j) acc += Y[(size_t)j * ny + y] * t[c.at(x, j, k)];
          w[c.at(x, y, k)] = acc;
        }
    for (int z = 0; z < nz; ++z)  // modes k -> cells z
      for (int y = 0; y < ny; ++y)
        for (int x = 0; x < nx; ++x) {
          double acc = 0.0;
          for (int k = 0; k < nz; ++k) acc += Z[(size_t)k * nz + z] * w[c.at(x, y, k)];
          out[c.at(x, y, z) * n + (size_t)b] = -hh * acc;
        }
  }
  return out;
}

template <class R> class Sim {
 public:
  dob_config cfg;
  bool fp64;
  bool ref;  // bc_mode == DOB_BC_REFERENCE
  Dims dv;   // velocity / pressure grid
  Dims dc;   // dye / conc grid
  float U[128];
  std::vector<R> u, v, w, u2, v2, w2;
  std::vector<R> cen[4], curl[4];
  std::vector<R> p, rhs;
  std::vector<double> p64;  // mixed mode: the pressure the defect loop carries (the device's p + plo)
  struct Level {
    Dims d;
    std::vector<R> e, b, r;
  };
  std::vector<Level> lv;
  int nconc = 1;
  std::vector<R> conc[4], concN[4];
  std::vector<R> pred;
  std::vector<uint32_t> splatI, splatL;
  std::vector<R> parcels;
  uint32_t cap = 0, highWater = 0;
  std::vector<float> wave;  // 4 * 512 * 512, interleaved
  double last_stats[5] = {0, 0, 0, 0, 0};

  explicit Sim(const dob_config& c, bool f64) : cfg(c), fp64(f64) {
    ref = cfg.bc_mode == DOB_BC_REFERENCE;
    dv.nx = cfg.nx; dv.ny = cfg.ny; dv.nz = cfg.nz;
    dc.nx = cfg.nx * cfg.dye_refine; dc.ny = cfg.ny * cfg.dye_refine; dc.nz = cfg.nz * cfg.dye_refine;
    const size_t N = dv.n();
    for (auto* a : {&u, &v, &w, &u2, &v2, &w2, &p, &rhs}) a->assign(N, R(0));
    for (int c = 0; c < 4; ++c) { cen[c].assign(N, R(0)); curl[c].assign(N, R(0)); }
    nconc = ref ? 4 : 1;
    for (int c = 0; c < nconc; ++c) { conc[c].assign(dc.n(), R(0)); concN[c].assign(dc.n(), R(0)); }
    pred.assign(dc.n(), R(0));
    splatI.assign(dc.n(), 0u);
    splatL.assign(dc.n(), 0u);
    cap = cfg.parcel_capacity;
    parcels.assign((size_t)cap * 8, R(0));
    wave.assign((size_t)4 * kWaveN * kWaveN, 0.0f);
    lv.resize(cfg.mg_levels);
    for (int l = 0; l < cfg.mg_levels; ++l) {
      lv[l].d.nx = dv.nx >> l; lv[l].d.ny = dv.ny >> l; lv[l].d.nz = dv.nz >> l;
      if (l > 0) {
        lv[l].e.assign(lv[l].d.n(), R(0));
        lv[l].b.assign(lv[l].d.n(), R(0));
      }
      lv[l].r.assign(lv[l].d.n(), R(0));
    }
    default_uniforms();
  }

  // The reference engine's default uniform block (uniformLayout.ts:31-46,
  // 92-159) with dt = FIXED_SIM_DT, no drops and globalSeed = 1.
  void default_uniforms() {
    memset(U, 0, sizeof(U));
    U[35] = 0.0f; U[36] = 1.0f; U[37] = 1.0f; U[38] = 1.0f / 60.0f;
    U[40] = 0.30f; U[41] = 1.0f; U[43] = 1.0f;
    U[44] = 1.02f; U[45] = 0.48f; U[46] = 0.9993f; U[47] = 0.995f;
    U[48] = 1.0f; U[49] = 1.0f; U[50] = 1.0f;
    U[52] = 0.48f; U[53] = -0.98f; U[54] = 0.30f; U[55] = 1.10f;
    U[57] = 0.0032f; U[58] = 1.0f; U[59] = 0.088f;
    U[60] = 0.032f; U[63] = 0.028f;
  }

  // ---- storage rounding (float oracle only) --------------------------------
  R st_vel(R x) const {  // rgba16float textures in the reference-faithful mode
    if (fp64 || cfg.precision_mode != DOB_PREC_REFERENCE_FP16) return x;
    return (R)dob_round_f16((float)x);
  }
  R st_dye(R x) const {
    if (fp64) return x;
    if (cfg.precision_mode == DOB_PREC_REFERENCE_FP16 || cfg.precision_mode == DOB_PREC_MIXED)
      return (R)dob_round_f16((float)x);
    return x;
  }

  // ---- uniform accessors (common.ts:31-63) -----------------------------------
  R dt() const {
    if (!ref) return (R)cfg.dt;
    return Clamp((R)U[38], R(0), R(0.025));
  }
  V3<R> dmin() const {
    if (!ref) return mk((R)cfg.domain_min[0], (R)cfg.domain_min[1], (R)cfg.domain_min[2]);
    return mk((R)-U[52], (R)U[53], (R)-U[52]);
  }
  V3<R> dmax() const {
    if (!ref) return mk((R)cfg.domain_max[0], (R)cfg.domain_max[1], (R)cfg.domain_max[2]);
    return mk((R)U[52], (R)U[54], (R)U[52]);
  }
  V3<R> dsize() const { return dmax() - dmin(); }
  V3<R> to_world(V3<R> uvw) const { return dmin() + uvw * dsize(); }
  V3<R> to_uvw(V3<R> pw) const { return (pw - dmin()) / dsize(); }
  V3<R> vdims() const { return mk((R)dv.nx, (R)dv.ny, (R)dv.nz); }
  V3<R> cdims() const { return mk((R)dc.nx, (R)dc.ny, (R)dc.nz); }
  R drop(int d, int k) const { return (R)U[64 + 8 * d + k]; }
  bool flag(int f) const { return ref && (cfg.physics_flags & f); }

  // ---- samplers ------------------------------------------------------------------
  V3<R> sample_center(V3<R> uvw) const {
    const Taps<R> t = taps(dv, uvw.x, uvw.y, uvw.z);
    return mk(lerp8(t, cen[0].data()), lerp8(t, cen[1].data()), lerp8(t, cen[2].data()));
  }
  R sample_scalar(const Dims& d, const std::vector<R>& a, V3<R> uvw) const {
    const Taps<R> t = taps(d, uvw.x, uvw.y, uvw.z);
    return lerp8(t, a.data());
  }
  // 2D bilinear sample of the 512x512 wave texture (clamp-to-edge).
  void sample_wave(R su, R sv, R out[4]) const {
    const R cx = su * R(kWaveN) - R(0.5), cy = sv * R(kWaveN) - R(0.5);
    const R bx = Floor(cx), by = Floor(cy);
    const R fx = cx - bx, fy = cy - by;
    const int x0 = ClampI((int)bx, 0, kWaveN - 1), x1 = ClampI((int)bx + 1, 0, kWaveN - 1);
    const int y0 = ClampI((int)by, 0, kWaveN - 1), y1 = ClampI((int)by + 1, 0, kWaveN - 1);
    for (int c = 0; c < 4; ++c) {
      const R a00 = (R)wave[((size_t)y0 * kWaveN + x0) * 4 + c];
      const R a10 = (R)wave[((size_t)y0 * kWaveN + x1) * 4 + c];
      const R a01 = (R)wave[((size_t)y1 * kWaveN + x0) * 4 + c];
      const R a11 = (R)wave[((size_t)y1 * kWaveN + x1) * 4 + c];
      out[c] = Mix(Mix(a00, a10, fx), Mix(a01, a11, fx), fy);
    }
  }
  // worldXZToWaveUV (common.ts:65-67), clamped like every caller.
  void wave_at(R x, R z, R lo, R hi, R out[4]) const {
    const R su = Clamp((x + R(1.60)) / R(3.20), lo, hi);
    const R sv = Clamp((z + R(1.60)) / R(3.20), lo, hi);
    sample_wave(su, sv, out);
  }

  // ---- evalTopDirichletPressure (fluid.ts:16-77) ---------------------------------
  R top_pressure(int ix, int iz) const {
    const R halfXZ = (R)U[52];
    const R fx = ((R)ix + R(0.5)) / (R)dv.nx;
    const R fz = ((R)iz + R(0.5)) / (R)dv.nz;
    const R wx = Mix(-halfXZ, halfXZ, fx), wz = Mix(-halfXZ, halfXZ, fz);
    const R dtv = dt();
    const R cellH = (R(2) * halfXZ) / (R)dv.nx;
    const R dtOverH = dtv / cellH;
    R ws[4];
    wave_at(wx, wz, R(0.002), R(0.998), ws);
    const R eta = ws[0], lap = ws[2];
    const R gEff = R(0.155);
    const R capTerm = R(-18.4) * lap;
    R pK = R(2.45) * (gEff * eta + R(0.00095) * capTerm);
    for (int d = 0; d < kMaxDrops; ++d) {
      const R signedSeed = drop(d, 7), drain = drop(d, 6);
      if (signedSeed > R(0) && drain > R(0.0005)) {
        const R rx = wx - drop(d, 0), rz = wz - drop(d, 2);
        const R r = Len2(rx, rz);
        const R theta = Atan2(rz, rx);
        const R seed = signedSeed;
        const R azim = R(1) + R(0.022) * Cos(R(4) * theta + seed * R(1.73)) +
                       R(0.016) * Cos(R(6) * theta - seed * R(2.31)) +
                       R(0.010) * Sin(R(8) * theta + seed * R(0.89));
        const R slugPhase = Smooth(R(0.32), R(0.92), drain);
        const R rOrifice =
            Clamp(drop(d, 3) * R(1.12) + Mix(R(0.018), R(0.032), slugPhase), R(0.030), R(0.090)) * azim;
        const R rNorm = r / Max(rOrifice, R(1e-4));
        const R speedY = Clamp(-drop(d, 4), R(0.08), R(0.65));
        const R neck = (R(0.28) + R(1.05) * rNorm * rNorm) * Exp(R(-0.92) * rNorm * rNorm) *
                       (R(1) - R(0.38) * rNorm * rNorm);
        pK = pK + drain * (R(0.014) + R(0.048) * speedY) * neck;
      }
    }
    const R wallTaper = R(1) - Smooth(halfXZ * R(0.72), halfXZ * R(0.96), Max(std::fabs(wx), std::fabs(wz)));
    return pK * dtOverH * wallTaper;
  }

  // ---- FLUID_INIT_VEL (fluid.ts:80-121) ------------------------------------------
  void init_vel() {
    const V3<R> dims = vdims();
    const R seed = (R)U[43], surfY = (R)U[40], halfXZ = (R)U[52];
#pragma omp parallel for schedule(static)
    for (int z = 0; z < dv.nz; ++z)
      for (int y = 0; y < dv.ny; ++y)
        for (int x = 0; x < dv.nx; ++x) {
          const V3<R> pX = to_world(mk((R)x + R(1), (R)y + R(0.5), (R)z + R(0.5)) / dims);
          const V3<R> pY = to_world(mk((R)x + R(0.5), (R)y + R(1), (R)z + R(0.5)) / dims);
          const V3<R> pZ = to_world(mk((R)x + R(0.5), (R)y + R(0.5), (R)z + R(1)) / dims);
          auto fade = [&](V3<R> q) {
            return (R(1) - Smooth(halfXZ * R(0.55), halfXZ * R(0.96), Max(std::fabs(q.x), std::fabs(q.z)))) *
                   (R(1) - Smooth(surfY - R(0.12), surfY, q.y)) * Smooth(R(0.06), R(0.24), Len2(q.x, q.z));
          };
          R vx = R(0.00045) * Sin(pX.x * R(6.5)) * Cos(pX.z * R(6.5)) * Sin(pX.y * R(5.2) + seed * R(1.3)) * fade(pX);
          R vy = R(0.00030) * Cos(pY.x * R(6.5)) * Sin(pY.z * R(6.5)) * Cos(pY.y * R(5.2) + seed * R(0.7)) * fade(pY);
          R vz = R(-0.00045) * Cos(pZ.x * R(6.5)) * Sin(pZ.z * R(6.5)) * Sin(pZ.y * R(5.2) + seed * R(1.3)) * fade(pZ);
          if (x >= dv.nx - 1) vx = R(0);
          if (z >= dv.nz - 1) vz = R(0);
          const size_t i = dv.at(x, y, z);
          // BloodDropEngine.ts:1734-1738 writes this shader into velA, velB,
          // velCenter and curl alike.
          u[i] = st_vel(vx); v[i] = st_vel(vy); w[i] = st_vel(vz);
          cen[0][i] = st_vel(vx); cen[1][i] = st_vel(vy); cen[2][i] = st_vel(vz); cen[3][i] = R(0);
          curl[0][i] = st_vel(vx); curl[1][i] = st_vel(vy); curl[2][i] = st_vel(vz); curl[3][i] = R(0);
        }
  }

  void reset() {
    inject_pending = 0;
    std::fill(u.begin(), u.end(), R(0)); std::fill(v.begin(), v.end(), R(0)); std::fill(w.begin(), w.end(), R(0));
    for (int c = 0; c < 4; ++c) { std::fill(cen[c].begin(), cen[c].end(), R(0)); std::fill(curl[c].begin(), curl[c].end(), R(0)); }
    if (ref) init_vel();
    std::fill(p.begin(), p.end(), R(0));
    if (mixed()) p64.assign(p.size(), 0.0);
    std::fill(rhs.begin(), rhs.end(), R(0));
    for (auto& L : lv) { std::fill(L.e.begin(), L.e.end(), R(0)); std::fill(L.b.begin(), L.b.end(), R(0)); std::fill(L.r.begin(), L.r.end(), R(0)); }
    for (int c = 0; c < nconc; ++c) { std::fill(conc[c].begin(), conc[c].end(), R(0)); std::fill(concN[c].begin(), concN[c].end(), R(0)); }
    std::fill(pred.begin(), pred.end(), R(0));
    std::fill(splatI.begin(), splatI.end(), 0u);
    std::fill(splatL.begin(), splatL.end(), 0u);
    // PARTICLE_RESET (particles.ts:27-45)
    for (uint32_t k = 0; k < cap; ++k) {
      R* q = &parcels[(size_t)k * 8];
      q[0] = q[1] = q[2] = q[3] = R(0);
      q[4] = R(0); q[5] = R(-0.003); q[6] = R(0); q[7] = R(0);
    }
    highWater = 0;
    // the reset's lighting passes (BloodDropEngine.ts:1760)
    if (ref && nconc == 4 && dv.nx % 4 == 0 && dv.ny % 4 == 0 && dv.nz % 4 == 0) light_volume();
  }

  // ---- FLUID_ADVECT_MAC (fluid.ts:144-329) ----------------------------------------
  R sample_mac(const std::vector<R>& a, V3<R> uvw, int comp) const {
    V3<R> sh = uvw;
    if (comp == 0) sh.x = sh.x - R(0.5) / (R)dv.nx;
    if (comp == 1) sh.y = sh.y - R(0.5) / (R)dv.ny;
    if (comp == 2) sh.z = sh.z - R(0.5) / (R)dv.nz;
    sh = ClampV(sh, R(0.001), R(0.999));
    return sample_scalar(dv, a, sh);
  }
  V3<R> trace_back(V3<R> uvwF, R dtv, V3<R> dom) const {
    const V3<R> v0 = sample_center(ClampV(uvwF, R(0.002), R(0.998)));
    const V3<R> uvwMid = ClampV(uvwF - (R(0.5) * (v0 * dtv)) / dom, R(0.002), R(0.998));
    const V3<R> vMid = sample_center(uvwMid);
    return ClampV(uvwF - (vMid * dtv) / dom, R(0.002), R(0.998));
  }
  R azim_neck(R theta, R seed) const {
    return R(1) + R(0.036) * Cos(R(4) * theta + seed * R(1.73)) + R(0.026) * Cos(R(6) * theta - seed * R(2.31)) +
           R(0.018) * Sin(R(8) * theta + seed * R(0.89));
  }
  void advect_mac() {
    const V3<R> dims = vdims();
    const R dtv = dt();
    const V3<R> dom = dsize();
    const R damp = ref ? (R)U[46] : (R)cfg.vel_damping;
    const R surfY = (R)U[40];
#pragma omp parallel for schedule(static)
    for (int z = 0; z < dv.nz; ++z)
      for (int y = 0; y < dv.ny; ++y)
        for (int x = 0; x < dv.nx; ++x) {
          const V3<R> uvwX = mk((R)x + R(1), (R)y + R(0.5), (R)z + R(0.5)) / dims;
          const V3<R> uvwY = mk((R)x + R(0.5), (R)y + R(1), (R)z + R(0.5)) / dims;
          const V3<R> uvwZ = mk((R)x + R(0.5), (R)y + R(0.5), (R)z + R(1)) / dims;
          R vx = sample_mac(u, trace_back(uvwX, dtv, dom), 0) * damp;
          R vy = sample_mac(v, trace_back(uvwY, dtv, dom), 1) * damp;
          R vz = sample_mac(w, trace_back(uvwZ, dtv, dom), 2) * damp;
          if (ref) {
            const V3<R> pCell = to_world((mk((R)x, (R)y, (R)z) + mk(R(0.5), R(0.5), R(0.5))) / dims);
            const V3<R> pFaceY = to_world(uvwY);
            R activeNeckMask = R(0);
            if (flag(DOB_PHYS_NECK)) {
              for (int d = 0; d < kMaxDrops; ++d) {
                const R signedSeed = drop(d, 7), drain = drop(d, 6);
                if (!(signedSeed > R(0) && drain > R(0.0005))) continue;
                const R dX = drop(d, 0), dZ = drop(d, 2);
                const R relx = pFaceY.x - dX, relz = pFaceY.z - dZ;
                const R r = Len2(relx, relz);
                const R theta = Atan2(relz, relx);
                const R seed = signedSeed;
                const R azim = azim_neck(theta, seed);
                const R sp = Smooth(R(0.14), R(0.76), drain);
                const R rNeckBase = Clamp(drop(d, 3) * Mix(R(0.80), R(1.08), sp) + Mix(R(0.012), R(0.030), sp), R(0.018), R(0.088));
                const R rNeck = rNeckBase * azim;
                const R rRatio = r / Max(rNeck, R(1e-4));
                const R slugRadial = (R(0.14) + R(1.00) * Min(rRatio * rRatio, R(1.20))) * (R(1) - Smooth(R(0.78), R(1.15), rRatio));
                const R stemRadial = (R(0.68) + R(0.32) * Min(rRatio * rRatio, R(1.0))) * (R(1) - Smooth(R(0.74), R(1.10), rRatio));
                const R radialProfile = Mix(stemRadial, slugRadial, sp);
                const R vertMask = Smooth(surfY - R(0.058), surfY - R(0.014), pFaceY.y);
                const R meniscusShear = Mix(R(1.0), R(0.36), Smooth(surfY - R(0.024), surfY - R(0.002), pFaceY.y));
                const R mask = radialProfile * vertMask;
                activeNeckMask = Max(activeNeckMask, radialProfile);
                if (mask > R(0.001)) {
                  const R lobeMod = R(1) + R(0.036) * Cos(R(4) * theta + seed * R(1.73)) + R(0.026) * Cos(R(6) * theta - seed * R(2.31));
                  const R impactSpeed = Clamp(-drop(d, 4), R(0.10), R(0.65));
                  const R slugDrive = Clamp(Pow(Max(drain, R(0)), R(0.66)) * R(0.84), R(0), R(1.24));
                  const R stemDrive = Clamp(R(0.045) + drain * R(0.22), R(0), R(0.20)) * Smooth(R(0), R(0.05), drain);
                  const R fluxDrive = Mix(stemDrive, slugDrive, sp);
                  const R targetVy = -Clamp(R(0.14) + R(0.64) * impactSpeed, R(0.15), R(0.39)) * fluxDrive * lobeMod * meniscusShear;
                  const R blend = Clamp(dtv * Mix(R(14), R(22), sp) * mask, R(0), R(1));
                  vy = Mix(vy, targetVy, blend);
                }
                const R vertMaskXZ = Smooth(surfY - R(0.058), surfY - R(0.014), pCell.y);
                if (vertMaskXZ > R(0.001)) {
                  const R flare = Mix(R(0.104) * (R(0.35) + R(0.65) * sp), R(-0.020), Smooth(surfY - R(0.066), surfY - R(0.012), pCell.y)) *
                                  Clamp(drain, R(0), R(1.3));
                  for (int comp = 0; comp < 2; ++comp) {
                    const V3<R> fw = to_world(comp == 0 ? uvwX : uvwZ);
                    const R ax = fw.x - dX, az = fw.z - dZ;
                    const R rF = Len2(ax, az);
                    if (rF > R(1e-4) && rF < rNeckBase * R(1.34)) {
                      const R thF = Atan2(az, ax);
                      const R azF = azim_neck(thF, seed);
                      const R rR = rF / Max(rNeckBase * azF, R(1e-4));
                      if (rR < R(1.22)) {
                        const R slugR = (R(0.14) + R(1.00) * Min(rR * rR, R(1.20))) * (R(1) - Smooth(R(0.78), R(1.15), rR));
                        const R stemR = (R(0.68) + R(0.32) * Min(rR * rR, R(1.0))) * (R(1) - Smooth(R(0.74), R(1.10), rR));
                        const R maskF = Mix(stemR, slugR, sp) * vertMaskXZ;
                        const R blendF = Clamp(dtv * Mix(R(14), R(22), sp) * maskF, R(0), R(1));
                        if (comp == 0) vx = Mix(vx, (ax / rF) * flare, blendF * R(0.65));
                        else vz = Mix(vz, (az / rF) * flare, blendF * R(0.65));
                      }
                    }
                  }
                }
              }
            }
            if (flag(DOB_PHYS_SURFACE) && y >= dv.ny - 3) {
              const R topFade = (R)(y - (dv.ny - 3) + 1) / R(3);
              const R epsW = R(0.015);
              R wc[4], t4[4];
              wave_at(pCell.x, pCell.z, R(0.002), R(0.998), wc);
              const R wC = wc[3];
              wave_at(pCell.x + epsW, pCell.z, R(0.002), R(0.998), t4); const R wXp = t4[3];
              wave_at(pCell.x - epsW, pCell.z, R(0.002), R(0.998), t4); const R wXn = t4[3];
              wave_at(pCell.x, pCell.z + epsW, R(0.002), R(0.998), t4); const R wZp = t4[3];
              wave_at(pCell.x, pCell.z - epsW, R(0.002), R(0.998), t4); const R wZn = t4[3];
              const R cmcWindow = R(1) - Smooth(R(0.45), R(0.88), wC);
              const R gx = (wXp - wXn) / (R(2) * epsW), gz = (wZp - wZn) / (R(2) * epsW);
              const R sc = -(R)U[41] * R(0.026) * cmcWindow;
              const R mpx = sc * gx * topFade, mpz = sc * gz * topFade;
              vx = vx + mpx * dtv;
              vz = vz + mpz * dtv;
              if (y >= dv.ny - 2 && activeNeckMask < R(0.02)) {
                const R calmGate = R(1) - Smooth(R(0.020), R(0.14), (R)std::fabs(wc[1]));
                const R layerWeight = (y == dv.ny - 1) ? R(0.72) : R(0.26);
                vy = Mix(vy, Clamp(wc[1] * R(0.35), R(-0.045), R(0.045)), calmGate * layerWeight);
              }
            }
            if (flag(DOB_PHYS_SPONGE)) {
              const R halfXZ = (R)U[52], yMin = (R)U[53];
              const R rCellXZ = Len2(pCell.x, pCell.z);
              const R wallFade = (R(1) - Smooth(halfXZ * R(0.68), halfXZ * R(0.94), rCellXZ)) *
                                 Smooth(yMin + R(0.004), yMin + R(0.052), pCell.y);
              const R spongeMul = Mix(R(0.84), R(1.0), wallFade);
              vx = vx * spongeMul; vy = vy * spongeMul; vz = vz * spongeMul;
            }
          }
          if (x >= dv.nx - 1) vx = R(0);
          if (z >= dv.nz - 1) vz = R(0);
          if (!ref && y >= dv.ny - 1) vy = R(0);
          const size_t i = dv.at(x, y, z);
          u2[i] = st_vel(vx); v2[i] = st_vel(vy); w2[i] = st_vel(vz);
        }
    u.swap(u2); v.swap(v2); w.swap(w2);
  }

  // ---- FLUID_MAC_TO_CENTER (fluid.ts:917-962) -------------------------------------
  void mac_to_center() {
    const V3<R> dims = vdims();
#pragma omp parallel for schedule(static)
    for (int z = 0; z < dv.nz; ++z)
      for (int y = 0; y < dv.ny; ++y)
        for (int x = 0; x < dv.nx; ++x) {
          const size_t i = dv.at(x, y, z);
          const R uR = x >= dv.nx - 1 ? R(0) : u[i];
          const R uL = x == 0 ? R(0) : u[dv.at(x - 1, y, z)];
          const R vU = (!ref && y >= dv.ny - 1) ? R(0) : v[i];
          const R vD = y == 0 ? R(0) : v[dv.at(x, y - 1, z)];
          const R wF = z >= dv.nz - 1 ? R(0) : w[i];
          const R wB = z == 0 ? R(0) : w[dv.at(x, y, z - 1)];
          R cx = R(0.5) * (uL + uR), cy = R(0.5) * (vD + vU), cz = R(0.5) * (wB + wF);
          if (flag(DOB_PHYS_SURFACE) && y >= dv.ny - 2 && cy < R(0)) {
            const V3<R> pCell = to_world((mk((R)x, (R)y, (R)z) + mk(R(0.5), R(0.5), R(0.5))) / dims);
            R activeNeck = R(0);
            for (int d = 0; d < kMaxDrops; ++d) {
              if (drop(d, 7) > R(0) && drop(d, 6) > R(0.008)) {
                const R rActive = Clamp(drop(d, 3) * R(1.15) + R(0.032), R(0.046), R(0.092));
                const R rDist = Len2(pCell.x - drop(d, 0), pCell.z - drop(d, 2));
                const R drainGate = Smooth(R(0.008), R(0.065), drop(d, 6));
                activeNeck = Max(activeNeck, (R(1) - Smooth(rActive * R(0.78), rActive * R(1.20), rDist)) * drainGate);
              }
            }
            const R stagGate = Mix(R(0.45), R(1.0), Smooth(R(0.002), R(0.018), Max(R(0), (R)U[40] - pCell.y)));
            cy = cy * Mix(stagGate, R(1.0), activeNeck);
          }
          cen[0][i] = st_vel(cx); cen[1][i] = st_vel(cy); cen[2][i] = st_vel(cz); cen[3][i] = R(0);
        }
  }

  // ---- FLUID_CURL (fluid.ts:331-369) --------------------------------------------------
  V3<R> loadC(int x, int y, int z) const {
    const size_t i = dv.at(ClampI(x, 0, dv.nx - 1), ClampI(y, 0, dv.ny - 1), ClampI(z, 0, dv.nz - 1));
    return mk(cen[0][i], cen[1][i], cen[2][i]);
  }
  void curl_stage() {
#pragma omp parallel for schedule(static)
    for (int z = 0; z < dv.nz; ++z)
      for (int y = 0; y < dv.ny; ++y)
        for (int x = 0; x < dv.nx; ++x) {
          const V3<R> vR = loadC(x + 1, y, z), vL = loadC(x - 1, y, z), vU = loadC(x, y + 1, z);
          const V3<R> vD = loadC(x, y - 1, z), vF = loadC(x, y, z + 1), vB = loadC(x, y, z - 1);
          const V3<R> om = R(0.5) * mk((vU.z - vD.z) - (vF.y - vB.y), (vF.x - vB.x) - (vR.z - vL.z), (vR.y - vL.y) - (vU.x - vD.x));
          const R mag = Len(om);
          const size_t i = dv.at(x, y, z);
          curl[0][i] = st_vel(om.x); curl[1][i] = st_vel(om.y); curl[2][i] = st_vel(om.z); curl[3][i] = st_vel(mag);
        }
  }

  // ---- FLUID_CASSON_FORCES (fluid.ts:377-511) -----------------------------------------
  V3<R> loadM(int x, int y, int z) const {
    const size_t i = dv.at(ClampI(x, 0, dv.nx - 1), ClampI(y, 0, dv.ny - 1), ClampI(z, 0, dv.nz - 1));
    return mk(u[i], v[i], w[i]);
  }
  R curlw(int x, int y, int z) const {
    return curl[3][dv.at(ClampI(x, 0, dv.nx - 1), ClampI(y, 0, dv.ny - 1), ClampI(z, 0, dv.nz - 1))];
  }
  V3<R> vort_conf(int ix, int iy, int iz, R vc) const {
    if (ix <= 1 || ix >= dv.nx - 2 || iy <= 1 || iy >= dv.ny - 3 || iz <= 1 || iz >= dv.nz - 2) return mk(R(0), R(0), R(0));
    const size_t i = dv.at(ix, iy, iz);
    const V3<R> omega = mk(curl[0][i], curl[1][i], curl[2][i]);
    const R omegaMag = curl[3][i];
    if (omegaMag <= R(0.18)) return mk(R(0), R(0), R(0));
    const R ringGate = Smooth(R(0.18), R(0.95), omegaMag) / (R(1) + R(0.28) * omegaMag);
    const V3<R> eta = R(0.5) * mk(curlw(ix + 1, iy, iz) - curlw(ix - 1, iy, iz), curlw(ix, iy + 1, iz) - curlw(ix, iy - 1, iz),
                                   curlw(ix, iy, iz + 1) - curlw(ix, iy, iz - 1));
    const R etaLen = Len(eta);
    if (etaLen <= R(1e-5)) return mk(R(0), R(0), R(0));
    return (vc * ringGate) * Cross(eta / etaLen, omega);
  }
  V3<R> sample_conc_rg(V3<R> uvw) const {  // .r and .g of the conc texture
    const Taps<R> t = taps(dc, uvw.x, uvw.y, uvw.z);
    return mk(lerp8(t, conc[0].data()), nconc > 1 ? lerp8(t, conc[1].data()) : R(0), R(0));
  }
  void casson_forces() {
    const V3<R> dims = vdims();
    const R dtv = dt();
#pragma omp parallel for schedule(static)
    for (int z = 0; z < dv.nz; ++z)
      for (int y = 0; y < dv.ny; ++y)
        for (int x = 0; x < dv.nx; ++x) {
          V3<R> mac = loadM(x, y, z);
          const V3<R> mXp = loadM(x + 1, y, z), mXn = loadM(x - 1, y, z);
          const V3<R> mYp = loadM(x, y + 1, z), mYn = loadM(x, y - 1, z);
          const V3<R> mZp = loadM(x, y, z + 1), mZn = loadM(x, y, z - 1);
          const V3<R> uvwCell = (mk((R)x, (R)y, (R)z) + mk(R(0.5), R(0.5), R(0.5))) / dims;
          const V3<R> du = mXp - mXn, dvv = mYp - mYn, dw = mZp - mZn;
          const V3<R> lapMac = (mXp + mXn + mYp + mYn + mZp + mZn) - R(6) * mac;
          if (ref) {
            const V3<R> concCell = sample_conc_rg(uvwCell);
            const R cRbc = Clamp(concCell.x, R(0), R(1.5));
            const R shearRate = R(50) * Sqrt(Dot(du, du) + Dot(dvv, dvv) + Dot(dw, dw) + R(1e-6));
            const R cassonScale = (R)U[58];
            const R sqrtMuInf = Sqrt(R(0.00010) * (R(1) + R(1.35) * cRbc));
            const R tauYield = R(0.0036) * cassonScale * cRbc * cRbc;
            const R sqrtYieldTerm = Sqrt(tauYield / Max(shearRate + R(0.40), R(0.40)));
            const R alpha = Clamp((sqrtMuInf + sqrtYieldTerm) * (sqrtMuInf + sqrtYieldTerm), R(0.00010), R(0.0044));
            mac = mac + alpha * lapMac;
            if (flag(DOB_PHYS_VORT_CONF)) {
              const R vcs = (R)U[44];
              const V3<R> vc0 = vort_conf(x, y, z, vcs);
              const R vcX = R(0.5) * (vc0.x + vort_conf(std::min(x + 1, dv.nx - 1), y, z, vcs).x);
              const R vcY = R(0.5) * (vc0.y + vort_conf(x, std::min(y + 1, dv.ny - 1), z, vcs).y);
              const R vcZ = R(0.5) * (vc0.z + vort_conf(x, y, std::min(z + 1, dv.nz - 1), vcs).z);
              mac = mac + mk(vcX, vcY, vcZ) * dtv;
            }
            if (flag(DOB_PHYS_BUOYANCY)) {
              const V3<R> uvwFaceY = mk((R)x + R(0.5), (R)y + R(1), (R)z + R(0.5)) / dims;
              const V3<R> cf = sample_conc_rg(ClampV(uvwFaceY, R(0.001), R(0.999)));
              const R buoyDensity = R(1.24) * cf.x + R(0.26) * cf.y;
              if (buoyDensity > R(0.0008)) {
                const V3<R> pFaceY = to_world(uvwFaceY);
                const R surfBuoyGate = Smooth(R(0.002), R(0.024), Max(R(0), (R)U[40] - pFaceY.y));
                const R effBuoyConc = R(1.24) * Tanh(buoyDensity / R(1.24));
                const R buoyAccel = -(R)U[45] * R(0.345) * effBuoyConc * surfBuoyGate;
                mac.y = mac.y + buoyAccel * dtv;
              }
            }
            if (flag(DOB_PHYS_SOLENOIDAL)) {
              const V3<R> pc = to_world(uvwCell);
              const R depthBelow = (R)U[40] - pc.y;
              const R unfurlGate = Smooth(R(0.11), R(0.36), depthBelow) * Smooth(R(0.0008), R(0.015), cRbc + R(0.45) * concCell.y);
              if (unfurlGate > R(0.001)) {
                const R tSwirl = (R)U[35] * R(0.36) + (R)U[60] * R(1.7);
                const R q1 = R(6.4) * pc.x + R(4.0) * pc.y + R(5.2) * pc.z + tSwirl;
                const R q2 = R(-5.6) * pc.x + R(4.8) * pc.y + R(7.2) * pc.z - tSwirl * R(0.77);
                const R q3 = R(9.0) * pc.x - R(6.0) * pc.y - R(6.4) * pc.z + tSwirl * R(1.13);
                const R c1 = Cos(q1), c2 = Cos(q2), s3 = R(0.42) * Sin(q3);
                const V3<R> sf = mk(R(-6.25), R(2.85), R(5.50)) * c1 + mk(R(-6.30), R(-1.26), R(-4.06)) * c2 + mk(R(6.40), R(-0.96), R(9.90)) * s3;
                const R vertMod = Smooth(R(0.16), R(0.42), depthBelow);
                mac = mac + mk(sf.x, sf.y * vertMod, sf.z) * (R(0.0028) * unfurlGate * dtv);
              }
            }
            mac = ClampV(mac, R(-1.8), R(1.8));
          } else {
            // Closed box: parametric Casson fluid, nu = (sqrt(mu_p) + sqrt(tau_y c^2 / (gdot + 0.4)))^2,
            // explicit step u += (nu dt / dx^2) lap u, capped at 1/8 for stability.
            const R c = Clamp(cfg.dye_refine == 1 ? conc[0][dc.at(x, y, z)] : sample_scalar(dc, conc[0], uvwCell), R(0), R(1.5));
            const R dxv = (R)cfg.dx;
            const R gdot = Sqrt(Dot(du, du) + Dot(dvv, dvv) + Dot(dw, dw)) / (R(2) * dxv);
            const R sqrtMu = Sqrt((R)cfg.casson_mu_p);
            const R sqrtYield = Sqrt((R)cfg.casson_tau_y * c * c / (gdot + R(0.4)));
            const R nu = (sqrtMu + sqrtYield) * (sqrtMu + sqrtYield);
            const R alpha = Min(nu * dtv / (dxv * dxv), R(0.125));
            mac = mac + alpha * lapMac;
          }
          if (x >= dv.nx - 1) mac.x = R(0);
          if (z >= dv.nz - 1) mac.z = R(0);
          if (!ref && y >= dv.ny - 1) mac.y = R(0);
          const size_t i = dv.at(x, y, z);
          u2[i] = st_vel(mac.x); v2[i] = st_vel(mac.y); w2[i] = st_vel(mac.z);
        }
    u.swap(u2); v.swap(v2); w.swap(w2);
  }

  // ---- FLUID_MAC_RHS (fluid.ts:517-555) --------------------------------------------------
  R divergence(int x, int y, int z) const {
    const size_t i = dv.at(x, y, z);
    const R uRight = x >= dv.nx - 1 ? R(0) : u[i];
    const R uLeft = x == 0 ? R(0) : u[dv.at(x - 1, y, z)];
    const R vTop = (!ref && y >= dv.ny - 1) ? R(0) : v[i];
    const R vBot = y == 0 ? R(0) : v[dv.at(x, y - 1, z)];
    const R wFront = z >= dv.nz - 1 ? R(0) : w[i];
    const R wBack = z == 0 ? R(0) : w[dv.at(x, y, z - 1)];
    return (uRight - uLeft) + (vTop - vBot) + (wFront - wBack);
  }
  void mac_rhs() {
#pragma omp parallel for schedule(static)
    for (int z = 0; z < dv.nz; ++z)
      for (int y = 0; y < dv.ny; ++y)
        for (int x = 0; x < dv.nx; ++x) {
          R r = divergence(x, y, z);
          if (ref && y == dv.ny - 1) r = r - top_pressure(x, z);
          rhs[dv.at(x, y, z)] = r;
        }
    if (!ref) {  // compatibility: FP64 zero-mean right-hand side
      const R mean = (R)(sum64(rhs) / (double)rhs.size());
      for (auto& r : rhs) r = r - mean;
    }
  }
  static double sum64(const std::vector<R>& a) {
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (long long i = 0; i < (long long)a.size(); ++i) s += (double)a[i];
    return s;
  }

  // ---- multigrid (fluid.ts:561-855; schedule BloodDropEngine.ts:1942-2059) ---------------
  // Mixed mode (float oracle only): defect correction of a higher-precision
  // pressure p64 whose correction V-cycles store levels >= 2 as BF16.
  bool mixed() const { return !fp64 && cfg.precision_mode == DOB_PREC_MIXED; }
  bool bf16_level(int l, bool inner) const { return inner && mixed() && l >= 2; }
  R h2(const Dims& d) const {
    const R s = (R)dv.nx / (R)d.nx;
    return s * s;
  }
  // evalMgStencil: neighbour sum and diagonal count (x-, x+, y-, y+, z-, z+).
  inline void stencil(const R* a, const Dims& d, int x, int y, int z, R& sumN, R& diag) const {
    sumN = R(0);
    diag = ref ? R(1) : R(0);
    if (x > 0) { sumN = sumN + a[d.at(x - 1, y, z)]; diag = diag + R(1); }
    if (x < d.nx - 1) { sumN = sumN + a[d.at(x + 1, y, z)]; diag = diag + R(1); }
    if (y > 0) { sumN = sumN + a[d.at(x, y - 1, z)]; diag = diag + R(1); }
    if (y < d.ny - 1) { sumN = sumN + a[d.at(x, y + 1, z)]; if (!ref) diag = diag + R(1); }
    if (z > 0) { sumN = sumN + a[d.at(x, y, z - 1)]; diag = diag + R(1); }
    if (z < d.nz - 1) { sumN = sumN + a[d.at(x, y, z + 1)]; diag = diag + R(1); }
  }
  // One colour of RBGS, in place (createMgRbgsShader, fluid.ts:605-681).
  void rbgs_color(R* a, const R* b, const Dims& d, int color, bool bf16) {
    const R hh = h2(d);
#pragma omp parallel for schedule(static)
    for (int z = 0; z < d.nz; ++z)
      for (int y = 0; y < d.ny; ++y)
        for (int x = ((y + z + color) & 1); x < d.nx; x += 2) {
          R sumN, diag;
          stencil(a, d, x, y, z, sumN, diag);
          if (diag == R(0)) continue;
          const R val = (sumN - hh * b[d.at(x, y, z)]) / diag;
          a[d.at(x, y, z)] = bf16 ? (R)dob_round_bf16((float)val) : val;
        }
  }
  void smooth(R* a, const R* b, const Dims& d, int sweeps, bool bf16) {
    for (int s = 0; s < sweeps; ++s) {
      rbgs_color(a, b, d, 0, bf16);
      rbgs_color(a, b, d, 1, bf16);
    }
  }
  // MG_RESIDUAL + MG_RESTRICT (fluid.ts:744-800)
  void residual(const R* a, const R* b, const Dims& d, R* r) {
    const R hh = h2(d);
#pragma omp parallel for schedule(static)
    for (int z = 0; z < d.nz; ++z)
      for (int y = 0; y < d.ny; ++y)
        for (int x = 0; x < d.nx; ++x) {
          R sumN, diag;
          stencil(a, d, x, y, z, sumN, diag);
          const R pC = a[d.at(x, y, z)];
          const R lapScaled = (sumN - diag * pC) / hh;
          r[d.at(x, y, z)] = b[d.at(x, y, z)] - lapScaled;
        }
  }
  void restrict_to(const R* r, const Dims& f, R* bc, const Dims& c, bool bf16) {
#pragma omp parallel for schedule(static)
    for (int z = 0; z < c.nz; ++z)
      for (int y = 0; y < c.ny; ++y)
        for (int x = 0; x < c.nx; ++x) {
          R sum = R(0);
          for (int dz = 0; dz < 2; ++dz)
            for (int dy = 0; dy < 2; ++dy)
              for (int dx = 0; dx < 2; ++dx) sum = sum + r[f.at(2 * x + dx, 2 * y + dy, 2 * z + dz)];
          const R avg = sum * R(0.125);
          bc[c.at(x, y, z)] = bf16 ? (R)dob_round_bf16((float)avg) : avg;
        }
  }
  // MG_PROLONG_ADD (fluid.ts:806-855)
  R coarse_err(const R* e, const Dims& c, int x, int y, int z) const {
    if (ref && y >= c.ny) return R(0);
    return e[c.at(ClampI(x, 0, c.nx - 1), ClampI(y, 0, c.ny - 1), ClampI(z, 0, c.nz - 1))];
  }
  void prolong_add(R* a, const Dims& f, const R* e, const Dims& c, bool bf16) {
#pragma omp parallel for schedule(static)
    for (int z = 0; z < f.nz; ++z)
      for (int y = 0; y < f.ny; ++y)
        for (int x = 0; x < f.nx; ++x) {
          const R cx = (((R)x + R(0.5)) / (R)f.nx) * (R)c.nx - R(0.5);
          const R cy = (((R)y + R(0.5)) / (R)f.ny) * (R)c.ny - R(0.5);
          const R cz = (((R)z + R(0.5)) / (R)f.nz) * (R)c.nz - R(0.5);
          const R bx = Floor(cx), by = Floor(cy), bz = Floor(cz);
          const int ix = (int)bx, iy = (int)by, iz = (int)bz;
          const R fx = cx - bx, fy = cy - by, fz = cz - bz;
          const R c000 = coarse_err(e, c, ix, iy, iz), c100 = coarse_err(e, c, ix + 1, iy, iz);
          const R c010 = coarse_err(e, c, ix, iy + 1, iz), c110 = coarse_err(e, c, ix + 1, iy + 1, iz);
          const R c001 = coarse_err(e, c, ix, iy, iz + 1), c101 = coarse_err(e, c, ix + 1, iy, iz + 1);
          const R c011 = coarse_err(e, c, ix, iy + 1, iz + 1), c111 = coarse_err(e, c, ix + 1, iy + 1, iz + 1);
          const R x00 = Mix(c000, c100, fx), x10 = Mix(c010, c110, fx);
          const R x01 = Mix(c001, c101, fx), x11 = Mix(c011, c111, fx);
          const R y0 = Mix(x00, x10, fy), y1 = Mix(x01, x11, fy);
          const R corr = Mix(y0, y1, fz);
          const size_t i = f.at(x, y, z);
          const R val = a[i] + corr;
          a[i] = bf16 ? (R)dob_round_bf16((float)val) : val;
        }
  }
  // Exact coarsest solve (mg_coarse_sweeps = -1): e = M b with M the
  // symmetric (pseudo-)inverse of the coarsest operator, built once by
  // Gauss-Jordan in double on A + J/n (pure Neumann; J/n removed afterwards)
  // or on A (Dirichlet top).  The float oracle applies M rounded to float.
  std::vector<double> cinv;
  void build_cinv(const Dims& c) { cinv = cinv_separable(c, (double)h2(c), ref); }
  R cinv_at(size_t k) const { return fp64 ? (R)cinv[k] : (R)(float)cinv[k]; }
  void coarse_exact(R* e, const R* b, const Dims& c, bool bf16) {
    const size_t n = c.n();
    if (cinv.size() != n * n) build_cinv(c);
    // every output is its own sum (in i order): threads over j give the same bits
#pragma omp parallel for schedule(static) if (n >= 512)
    for (size_t j = 0; j < n; ++j) {
      R acc = R(0);
      for (size_t i = 0; i < n; ++i) acc = acc + cinv_at(i * n + j) * b[i];
      e[j] = bf16 ? (R)dob_round_bf16((float)acc) : acc;
    }
  }
  int sweeps_pre(int l) const { return (l == 0 && cfg.reference_schedule) ? 1 : cfg.mg_pre; }
  int sweeps_post(int l) const { return (l == 0 && cfg.reference_schedule) ? 1 : cfg.mg_post; }

  // One V-cycle on (x0, b0) at level 0.  inner = correction solve of the
  // mixed-precision defect loop (level-0 arrays stored BF16).
  void vcycle(R* x0, const R* b0, bool inner) {
    const int L = cfg.mg_levels;
    if (L == 1) {
      smooth(x0, b0, lv[0].d, cfg.mg_pre + cfg.mg_post, inner);
      return;
    }
    smooth(x0, b0, lv[0].d, sweeps_pre(0), inner);
    residual(x0, b0, lv[0].d, lv[0].r.data());
    restrict_to(lv[0].r.data(), lv[0].d, lv[1].b.data(), lv[1].d, bf16_level(1, inner));
    for (int l = 1; l < L - 1; ++l) {
      std::fill(lv[l].e.begin(), lv[l].e.end(), R(0));
      smooth(lv[l].e.data(), lv[l].b.data(), lv[l].d, cfg.mg_pre, bf16_level(l, inner));
      residual(lv[l].e.data(), lv[l].b.data(), lv[l].d, lv[l].r.data());
      restrict_to(lv[l].r.data(), lv[l].d, lv[l + 1].b.data(), lv[l + 1].d, bf16_level(l + 1, inner));
    }
    Level& C = lv[L - 1];
    std::fill(C.e.begin(), C.e.end(), R(0));
    if (cfg.mg_coarse_sweeps < 0) coarse_exact(C.e.data(), C.b.data(), C.d, bf16_level(L - 1, inner));
    else smooth(C.e.data(), C.b.data(), C.d, cfg.mg_coarse_sweeps, bf16_level(L - 1, inner));
    for (int l = L - 2; l >= 1; --l) {
      prolong_add(lv[l].e.data(), lv[l].d, lv[l + 1].e.data(), lv[l + 1].d, bf16_level(l, inner));
      smooth(lv[l].e.data(), lv[l].b.data(), lv[l].d, cfg.mg_post, bf16_level(l, inner));
    }
    prolong_add(x0, lv[0].d, lv[1].e.data(), lv[1].d, inner);
    smooth(x0, b0, lv[0].d, sweeps_post(0), inner);
  }

  // ||b - A p||_2 accumulated in double.
  double residual_l2(const std::vector<R>& a, const std::vector<R>& b, std::vector<double>* out) {
    const Dims& d = lv[0].d;
    const double hh = (double)h2(d);
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (int z = 0; z < d.nz; ++z)
      for (int y = 0; y < d.ny; ++y)
        for (int x = 0; x < d.nx; ++x) {
          double sumN = 0.0, diag = ref ? 1.0 : 0.0;
          if (x > 0) { sumN += (double)a[d.at(x - 1, y, z)]; diag += 1.0; }
          if (x < d.nx - 1) { sumN += (double)a[d.at(x + 1, y, z)]; diag += 1.0; }
          if (y > 0) { sumN += (double)a[d.at(x, y - 1, z)]; diag += 1.0; }
          if (y < d.ny - 1) { sumN += (double)a[d.at(x, y + 1, z)]; if (!ref) diag += 1.0; }
          if (z > 0) { sumN += (double)a[d.at(x, y, z - 1)]; diag += 1.0; }
          if (z < d.nz - 1) { sumN += (double)a[d.at(x, y, z + 1)]; diag += 1.0; }
          const double r = (double)b[d.at(x, y, z)] - (sumN - diag * (double)a[d.at(x, y, z)]) / hh;
          if (out) (*out)[d.at(x, y, z)] = r;
          s += r * r;
        }
    return sqrt(s);
  }

  // ||b - A p64|| and max |b - A p64| in double (the mixed loop's residual)
  double residual64(std::vector<double>* out, double* rmax) {
    const Dims& d = lv[0].d;
    double s = 0.0, m = 0.0;
#pragma omp parallel for reduction(+ : s) reduction(max : m) schedule(static)
    for (int z = 0; z < d.nz; ++z)
      for (int y = 0; y < d.ny; ++y)
        for (int x = 0; x < d.nx; ++x) {
          double sumN = 0.0, diag = ref ? 1.0 : 0.0;
          if (x > 0) { sumN += p64[d.at(x - 1, y, z)]; diag += 1.0; }
          if (x < d.nx - 1) { sumN += p64[d.at(x + 1, y, z)]; diag += 1.0; }
          if (y > 0) { sumN += p64[d.at(x, y - 1, z)]; diag += 1.0; }
          if (y < d.ny - 1) { sumN += p64[d.at(x, y + 1, z)]; if (!ref) diag += 1.0; }
          if (z > 0) { sumN += p64[d.at(x, y, z - 1)]; diag += 1.0; }
          if (z < d.nz - 1) { sumN += p64[d.at(x, y, z + 1)]; diag += 1.0; }
          const double r = (double)rhs[d.at(x, y, z)] - (sumN - diag * p64[d.at(x, y, z)]);
          if (out) (*out)[d.at(x, y, z)] = r;
          s += r * r;
          m = std::max(m, std::fabs(r));
        }
    if (rmax) *rmax = m;
    return sqrt(s);
  }

  void pressure_solve() {
    int cycles = 0, outer = 0;
    if (mixed()) {
      // Defect correction: residual of the high-precision pressure, stop at
      // max |r| (the projected divergence) and/or ||r|| / ||b||, else an
      // FP32 correction V-cycle (BF16 storage from level 2) added to p64.
      const double bnorm = sqrt(dot64(rhs, rhs));
      const double div_r = ref ? cfg.mg_div_tol : cfg.mg_div_tol * (double)cfg.dx / (double)cfg.dt;
      std::vector<double> r64(p.size());
      std::vector<R> rin(p.size()), e(p.size());
      const int max_outer = std::max(1, cfg.mg_max_outer);
      for (outer = 0; outer < max_outer; ++outer) {
        double rmax = 0.0;
        const double rn = residual64(&r64, &rmax);
        const bool div_ok = cfg.mg_div_tol <= 0.0 || rmax <= (double)(float)div_r;
        const bool rel_ok = cfg.mg_rel_tol <= 0.0 || bnorm == 0.0 || rn <= cfg.mg_rel_tol * bnorm;
        if (div_ok && rel_ok) break;
        for (size_t i = 0; i < p.size(); ++i) rin[i] = (R)r64[i];
        std::fill(e.begin(), e.end(), R(0));
        for (int c = 0; c < cfg.mg_cycles; ++c) { vcycle(e.data(), rin.data(), true); ++cycles; }
        for (size_t i = 0; i < p.size(); ++i) p64[i] += (double)e[i];
      }
      if (!ref) {
        double s = 0.0;
        for (double q : p64) s += q;
        const double mean = s / (double)p64.size();
        for (auto& q : p64) q -= mean;
      }
      for (size_t i = 0; i < p.size(); ++i) p[i] = (R)p64[i];
    } else {
      const int ncyc = cycles_override > 0 ? cycles_override : cfg.mg_cycles;
      for (int c = 0; c < ncyc; ++c) { vcycle(p.data(), rhs.data(), false); ++cycles; }
      if (!ref) {  // pin the pressure mean (FP64 sum)
        const R mean = (R)(sum64(p) / (double)p.size());
        for (auto& q : p) q = q - mean;
      }
    }
    last_stats[3] = cycles;
    last_stats[4] = outer;
  }
  static double dot64(const std::vector<R>& a, const std::vector<R>& b) {
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (long long i = 0; i < (long long)a.size(); ++i) s += (double)a[i] * (double)b[i];
    return s;
  }

  // ---- FLUID_MAC_PROJECT (fluid.ts:863-911) -------------------------------------------------
  void project() {
#pragma omp parallel for schedule(static)
    for (int z = 0; z < dv.nz; ++z)
      for (int y = 0; y < dv.ny; ++y)
        for (int x = 0; x < dv.nx; ++x) {
          const size_t i = dv.at(x, y, z);
          V3<R> mac = mk(u[i], v[i], w[i]);
          const R pC = p[i];
          // mixed mode: pressure differences of the high-precision pressure
          auto dp = [&](size_t j) { return mixed() ? (R)(p64[j] - p64[i]) : p[j] - pC; };
          if (x < dv.nx - 1) mac.x = mac.x - dp(dv.at(x + 1, y, z)); else mac.x = R(0);
          if (y < dv.ny - 1) mac.y = mac.y - dp(dv.at(x, y + 1, z));
          else if (ref) mac.y = mac.y - (top_pressure(x, z) - pC);
          else mac.y = R(0);
          if (z < dv.nz - 1) mac.z = mac.z - dp(dv.at(x, y, z + 1)); else mac.z = R(0);
          if (ref) mac = ClampV(mac, R(-2), R(2));
          u[i] = st_vel(mac.x); v[i] = st_vel(mac.y); w[i] = st_vel(mac.z);
        }
  }

  // ---- splat helpers (particles.ts:22-24, 234-301) -------------------------------------------
  size_t flat_conc(int x, int y, int z) const { return dc.at(x, y, z); }
  void splat_trilinear(std::vector<uint32_t>& dst, V3<R> uvw, R mass, R minMass) {
    if (mass <= minMass) return;
    const V3<R> dims = cdims();
    const V3<R> coord = uvw * dims - mk(R(0.5), R(0.5), R(0.5));
    const int bx = (int)Floor(coord.x), by = (int)Floor(coord.y), bz = (int)Floor(coord.z);
    const V3<R> f = ClampV(coord - mk((R)bx, (R)by, (R)bz), R(0), R(1));
    const V3<R> omf = mk(R(1), R(1), R(1)) - f;
    const int x0 = ClampI(bx, 0, dc.nx - 1), y0 = ClampI(by, 0, dc.ny - 1), z0 = ClampI(bz, 0, dc.nz - 1);
    const int x1 = ClampI(bx + 1, 0, dc.nx - 1), y1 = ClampI(by + 1, 0, dc.ny - 1), z1 = ClampI(bz + 1, 0, dc.nz - 1);
    const R scale = mass * R(kSplatScale);
    const uint32_t w000 = (uint32_t)Round(scale * omf.x * omf.y * omf.z);
    const uint32_t w100 = (uint32_t)Round(scale * f.x * omf.y * omf.z);
    const uint32_t w010 = (uint32_t)Round(scale * omf.x * f.y * omf.z);
    const uint32_t w110 = (uint32_t)Round(scale * f.x * f.y * omf.z);
    const uint32_t w001 = (uint32_t)Round(scale * omf.x * omf.y * f.z);
    const uint32_t w101 = (uint32_t)Round(scale * f.x * omf.y * f.z);
    const uint32_t w011 = (uint32_t)Round(scale * omf.x * f.y * f.z);
    const uint32_t w111 = (uint32_t)Round(scale * f.x * f.y * f.z);
    auto add = [&](int x, int y, int z, uint32_t val) {
      if (val > 0u) {
        uint32_t* t = &dst[flat_conc(x, y, z)];
#pragma omp atomic
        *t += val;
      }
    };
    add(x0, y0, z0, w000); add(x1, y0, z0, w100); add(x0, y1, z0, w010); add(x1, y1, z0, w110);
    add(x0, y0, z1, w001); add(x1, y0, z1, w101); add(x0, y1, z1, w011); add(x1, y1, z1, w111);
  }

  // ---- hash33 (common.ts:79-83) ------------------------------------------------------------
  static V3<R> hash33(V3<R> p3in) {
    V3<R> p3 = mk(Fract(p3in.x * R(0.1031)), Fract(p3in.y * R(0.1030)), Fract(p3in.z * R(0.0973)));
    const R dd = Dot(p3, mk(p3.y + R(33.33), p3.x + R(33.33), p3.z + R(33.33)));
    p3 = mk(p3.x + dd, p3.y + dd, p3.z + dd);
    const V3<R> a = mk(p3.x + p3.y, p3.x + p3.x, p3.y + p3.x);
    const V3<R> b = mk(p3.z, p3.y, p3.x);
    const V3<R> q = a * b;
    return mk(Fract(q.x), Fract(q.y), Fract(q.z));
  }

  // ---- PARTICLE_EMIT (particles.ts:53-181) ---------------------------------------------------
  uint32_t spawn_count() const {
    if (!ref) return 0u;
    const float sc = U[62] > 0.0f ? U[62] : 0.0f;
    uint32_t n = (uint32_t)sc;
    if (n > 8192u) n = 8192u;  // the engine never packs more (BloodDropEngine.ts:1835)
    return n > cap ? cap : n;
  }
  void parcel_emit() {
    const uint32_t spawnCount = spawn_count();
    if (spawnCount == 0u) return;
    R totalDrain = R(0);
    for (int d = 0; d < kMaxDrops; ++d)
      if (drop(d, 7) > R(0) && drop(d, 6) > R(0.0001)) totalDrain = totalDrain + drop(d, 6);
    if (totalDrain <= R(1e-6)) return;
    const uint32_t cursor = (uint32_t)(U[61] > 0.0f ? U[61] : 0.0f);
    const R surfY = (R)U[40];
    for (uint32_t gid = 0; gid < spawnCount; ++gid) {
      const R targetFrac = ((R)gid + R(0.5)) / (R)(spawnCount > 1u ? spawnCount : 1u) * totalDrain;
      R accum = R(0);
      int chosen = 0;
      for (int d = 0; d < kMaxDrops; ++d) {
        if (drop(d, 7) > R(0) && drop(d, 6) > R(0.0001)) {
          accum = accum + drop(d, 6);
          chosen = d;
          if (accum >= targetFrac) break;
        }
      }
      const R dX = drop(chosen, 0), dY = drop(chosen, 1), dZ = drop(chosen, 2), dRad = drop(chosen, 3);
      const R dDrain = drop(chosen, 6);
      const R seed = Max(drop(chosen, 7), R(0.5));
      const uint32_t ringIdx = (uint32_t)(((uint64_t)cursor + gid) % cap);
      R* op = &parcels[(size_t)ringIdx * 8];
      if (op[3] > R(1e-6)) {
        const V3<R> settle = op[1] < surfY - R(0.32) ? mk(op[0], (R)U[53] + R(0.012), op[2]) : mk(op[0], op[1], op[2]);
        const V3<R> oldUvw = to_uvw(settle);
        if (oldUvw.x > R(0.002) && oldUvw.y > R(0.002) && oldUvw.z > R(0.002) && oldUvw.x < R(0.998) &&
            oldUvw.y < R(0.998) && oldUvw.z < R(0.998)) {
          const V3<R> cd = oldUvw * cdims();
          const int cx = ClampI((int)Floor(cd.x), 0, dc.nx - 1), cy = ClampI((int)Floor(cd.y), 0, dc.ny - 1),
                    cz = ClampI((int)Floor(cd.z), 0, dc.nz - 1);
          const uint32_t fpOld = (uint32_t)Round(op[3] * R(kSplatScale));
          if (fpOld > 0u) splatL[flat_conc(cx, cy, cz)] += fpOld;
        }
      }
      const R seqIdx = (R)ringIdx + seed * R(137.0);
      const V3<R> hsh = hash33(mk((R)gid, (R)U[35] * R(60.0), seed));
      const V3<R> r3 = mk(Fract(seqIdx * R(0.8191725134) + hsh.x * R(0.032)), Fract(seqIdx * R(0.6710436067) + hsh.y * R(0.032)),
                          Fract(seqIdx * R(0.5497004779) + hsh.z * R(0.032)));
      const R theta = R(6.28318530718) * r3.x;
      const R azim = azim_neck(theta, seed);
      const R rDrop = Max(dRad, R(0.010));
      const R emergNorm = (dY - surfY) / Max(rDrop, R(0.018));
      const R nascentCoreFill = Smooth(R(-0.32), R(0.18), emergNorm);
      const R slugWeight = Smooth(R(0.26), R(0.85), dDrain);
      const R wakeThin = Mix(R(0.46), R(1.0), Smooth(R(0.018), R(0.26), dDrain));
      const R rNeck = Mix(R(0.013) * wakeThin, Clamp(rDrop * R(0.84) + R(0.014), R(0.020), R(0.056)), slugWeight) * azim;
      const R innerRing = R(0.37) * slugWeight;
      const bool isCapVeil = slugWeight > R(0.08) && r3.z < R(0.16);
      const R radFracAnnular = Mix(innerRing, R(1.0), Pow(r3.y, Mix(R(0.50), R(0.44), slugWeight)));
      const R radFracCap = Mix(R(0.14) * slugWeight, Max(innerRing * R(1.32), R(0.08)), Sqrt(r3.y));
      const R radFracTorus = isCapVeil ? radFracCap : radFracAnnular;
      const R radFrac = Mix(radFracTorus, Sqrt(r3.y), nascentCoreFill * R(0.82));
      const R r = rNeck * radFrac;
      const R wakeDriftAngle = (R)U[35] * R(1.85) + seed * R(3.17);
      const R driftS = R(0.0038) * (R(1) - slugWeight) * (R(1) - wakeThin * R(0.45));
      const R wdx = Cos(wakeDriftAngle) * driftS, wdz = Sin(wakeDriftAngle * R(0.83) + seed) * driftS;
      const R ct = Cos(theta), stt = Sin(theta);
      const R posX = dX + wdx + ct * r, posZ = dZ + wdz + stt * r;
      R ws[4];
      wave_at(posX, posZ, R(0.002), R(0.998), ws);
      const R localEta = Clamp(ws[0], R(-0.085), R(0.015));
      const R neckTopY = surfY + Min(R(0), localEta) - R(0.0038);
      const R cavitySag = (R(1) - radFrac * radFrac) * (R(0.0085) * slugWeight + R(0.0045) * nascentCoreFill);
      const R zStrat = isCapVeil ? r3.z * R(3.6) : (r3.z - R(0.16) * slugWeight) / Max(R(1) - R(0.16) * slugWeight, R(0.5));
      const R posY = neckTopY - cavitySag - Mix(R(0.0014), R(0.0135), Clamp(zStrat, R(0), R(1)));
      const R smallDropFragility = R(1) - Smooth(R(0.022), R(0.056), rDrop);
      const R rimExposure = Smooth(R(0.58), R(1.0), radFrac);
      const R initLysis = Clamp(R(0.14) * rimExposure + R(0.28) * smallDropFragility * (R(0.45) + R(0.55) * radFrac), R(0), R(0.44));
      const R rf = Max(radFrac, R(0.25));
      const V3<R> tangentDir = mk(-stt * rf, R(-0.80), ct * rf);
      const V3<R> initStretch = Normalize(tangentDir) * R(0.0036);
      op[0] = posX; op[1] = posY; op[2] = posZ; op[3] = R(kParcelMass);
      op[4] = initStretch.x; op[5] = initStretch.y; op[6] = initStretch.z; op[7] = initLysis;
    }
  }

  // ---- sampleVelWorld (particles.ts:201-232) ---------------------------------------------------
  V3<R> sample_vel_world(V3<R> pp, R rouleauxMaturity, R meniscusHold) const {
    const R depth = (R)U[40] - pp.y;
    const V3<R> uvw = ClampV(to_uvw(pp), R(0.002), R(0.998));
    const R settleGate = Mix(R(0.38), R(1.0), Smooth(R(0.002), R(0.055), depth));
    const R rouleauxFall = Mix(R(0.020), R(0.046), Smooth(R(0.04), R(0.42), depth));
    const R monoSettle = rouleauxFall * settleGate;
    const R stackSettle = Mix(R(0.032), R(0.062), Smooth(R(0.04), R(0.48), depth));
    const R surfTailHold = meniscusHold * (R(1) - Smooth(R(0.003), R(0.034), Max(R(0), depth)));
    const R effSettle = Mix(monoSettle, stackSettle, rouleauxMaturity) * Mix(R(1.0), R(0.035), surfTailHold);
    const R deepUnfurl = Smooth(R(0.035), R(0.24), depth);
    V3<R> sub = mk(R(0), R(0), R(0));
    if (deepUnfurl > R(0.001)) {
      const R tPhase = (R)U[35] * R(0.42);
      const R a1 = R(8.4) * pp.x + R(5.2) * pp.y + R(6.6) * pp.z + tPhase;
      const R a2 = R(-7.2) * pp.x + R(6.0) * pp.y + R(9.4) * pp.z - tPhase * R(0.81);
      const R a3 = R(11.5) * pp.x - R(7.5) * pp.y - R(8.5) * pp.z + tPhase * R(1.13);
      const R c1 = Cos(a1), c2 = Cos(a2), s3 = R(0.45) * Sin(a3);
      const V3<R> raw = mk(R(-8.16), R(3.84), R(7.36)) * c1 + mk(R(-8.20), R(-1.38), R(-5.40)) * c2 + mk(R(8.30), R(-1.10), R(12.20)) * s3;
      const R vertTaper = Smooth(R(0.06), R(0.24), depth);
      sub = mk(raw.x, raw.y * vertTaper, raw.z) * (R(0.00028) * deepUnfurl);
    }
    V3<R> vg = sample_center(uvw);
    vg.y = vg.y * Mix(R(1.0), R(0.045), surfTailHold);
    return vg + mk(R(0), -effSettle, R(0)) + sub;
  }

  // ---- PARTICLE_ADVECT_SPLAT (particles.ts:303-462) ---------------------------------------------
  void parcel_advect_ref_one(uint32_t gid) {
    R* q = &parcels[(size_t)gid * 8];
    R mass = q[3];
    if (mass <= R(1e-6)) return;
    const R dtv = dt();
    const R halfXZ = (R)U[52], yMin = (R)U[53], surfY = (R)U[40];
    V3<R> pos = mk(q[0], q[1], q[2]);
    V3<R> stretch = mk(q[4], q[5], q[6]);
    const R rawW = Max(R(0), q[7]);
    R ageTicks = Floor(rawW);
    R lysis = Clamp(rawW - ageTicks, R(0), R(0.98));
    const R parcelAge = ageTicks * (R(1) / R(240));
    const R rouleauxMaturity = Smooth(R(8.5), R(18.0), parcelAge);
    const R tailRank = Fract((R)gid * R(0.7548776662));
    const R meniscusHold = Pow(Smooth(R(0.36), R(0.995), tailRank), R(1.65)) * (R(1) - Smooth(R(5.2), R(10.2), parcelAge));
    const V3<R> v1 = sample_vel_world(pos, rouleauxMaturity, meniscusHold);
    const R speed2 = Dot(v1, v1);
    if (dtv > R(0)) {
      ageTicks = Min(R(8191), ageTicks + Max(R(1), Round(dtv * R(240))));
      const V3<R> v2 = sample_vel_world(pos + R(0.5) * v1 * dtv, rouleauxMaturity, meniscusHold);
      V3<R> vAdv = v2;
      if (speed2 > R(0.0025)) {
        const V3<R> v3 = sample_vel_world(pos + R(0.75) * v2 * dtv, rouleauxMaturity, meniscusHold);
        vAdv = R(2.0 / 9.0) * v1 + R(3.0 / 9.0) * v2 + R(4.0 / 9.0) * v3;
      }
      const R floorSlip = Smooth(yMin + R(0.005), yMin + R(0.042), pos.y);
      const R rXZFloor = Len2(pos.x, pos.z);
      R fox = R(0), foz = R(0);
      if (rXZFloor > R(1e-4)) {
        const R k = R(0.016) * (R(1) - floorSlip) * Smooth(R(0.01), R(0.22), rXZFloor);
        fox = (pos.x / Max(rXZFloor, R(1e-4))) * k;
        foz = (pos.z / Max(rXZFloor, R(1e-4))) * k;
      }
      vAdv = mk(vAdv.x * Mix(R(0.45), R(1.0), floorSlip) + fox, vAdv.y * Mix(R(0.15), R(1.0), floorSlip),
                vAdv.z * Mix(R(0.45), R(1.0), floorSlip) + foz);
      pos = pos + vAdv * dtv;
      pos.y = Clamp(pos.y, yMin + R(0.0055), surfY - R(0.0018));
      if (speed2 > R(2.5e-7) && floorSlip > R(0.15)) {
        const R sLen = Max(Len(stretch), R(1e-5));
        const V3<R> sDir = stretch / sLen;
        const R probeStep = R(0.0065);
        const V3<R> vPlus = sample_vel_world(pos + sDir * probeStep, rouleauxMaturity, meniscusHold);
        const V3<R> vMinus = sample_vel_world(pos - sDir * probeStep, rouleauxMaturity, meniscusHold);
        const V3<R> dVel = (vPlus - vMinus) * (sLen / (R(2) * probeStep));
        stretch = stretch + dVel * dtv;
        const R vMag = Sqrt(speed2);
        if (vMag > R(0.001) && sLen < R(0.006)) stretch = stretch + (v1 / vMag) * (R(0.0022) * dtv);
        const R maxThreadLen = Mix(R(0.0270), R(0.0420), meniscusHold * (R(1) - Smooth(R(0.005), R(0.065), Max(R(0), surfY - pos.y))));
        const R nextLen = Clamp(Len(stretch), R(0.0026), maxThreadLen);
        stretch = (stretch / Max(Len(stretch), R(1e-5))) * nextLen;
      } else if (floorSlip <= R(0.15)) {
        stretch.y = stretch.y * Exp(-dtv * R(5.0));
      }
    }
    const V3<R> uvw = to_uvw(pos);
    const R rHoriz = Len2(pos.x, pos.z);
    const R wallSponge = R(1) - Smooth(halfXZ * R(0.68), halfXZ * R(0.94), rHoriz);
    mass = mass * Mix(R(1.0), wallSponge, Clamp(dtv * R(6.0), R(0), R(1)));
    if (mass <= R(1e-5) || rHoriz >= halfXZ * R(0.95) || uvw.x <= R(0.002) || uvw.x >= R(0.998) || uvw.z <= R(0.002) ||
        uvw.z >= R(0.998) || uvw.y >= R(0.998)) {
      q[3] = R(0);  // p.posAndMass.w = 0; the rest of p is written back unchanged
      return;
    }
    if (dtv > R(0) && pos.y < yMin + R(0.026)) {
      const R settleWeight = R(1) - Smooth(yMin + R(0.005), yMin + R(0.026), pos.y);
      const R dmBed = mass * Clamp(settleWeight * dtv * R(1.65), R(0), R(0.095));
      if (dmBed > R(1e-7)) {
        mass = Max(R(0), mass - dmBed);
        splat_trilinear(splatL, ClampV(uvw, R(0.002), R(0.998)), dmBed * R(0.68), R(1e-7));
      }
      if (mass <= R(1e-5)) {
        q[3] = R(0);
        return;
      }
    }
    const R cellRes = Fract((R)gid * R(0.6180339887) + R(0.17));
    const V3<R> cs = sample_conc_rg(ClampV(uvw, R(0.002), R(0.998)));
    const R cNeighborhood = cs.x + cs.y;
    const R diluteExposure = R(1) - Smooth(R(0.012), R(0.22), cNeighborhood);
    const R ageDispersion = Smooth(R(1.1), R(7.8), parcelAge + diluteExposure * R(2.2) + lysis * R(2.5));
    const R lateDiluteFade = Smooth(R(7.2), R(16.0), parcelAge) * diluteExposure;
    const R midResid = Mix(R(0.07), R(0.20), cellRes);
    const R lateResid = Mix(R(0.014), R(0.052), cellRes);
    const R minIntactMass = R(kParcelMass) * Mix(Mix(R(0.46), R(0.64), cellRes), Mix(midResid, lateResid, lateDiluteFade), ageDispersion);
    const R lysableHeadroom = mass - minIntactMass;
    const R floorShelter = Smooth(yMin + R(0.024), yMin + R(0.062), pos.y);
    if (dtv > R(0) && lysableHeadroom > R(1e-7) && floorShelter > R(0.02)) {
      const R shearActivity = Mix(R(0.22), R(1.0), Smooth(R(0.0005), R(0.0120), speed2));
      const R waterExposure = (R(1) - R(0.72) * Smooth(R(0.016), R(0.30), cNeighborhood)) * floorShelter * shearActivity;
      const R kLysis = (R)U[59];
      lysis = Clamp(lysis + kLysis * (R(1.85) * waterExposure) * dtv, R(0), R(0.98));
      const R fragility = Smooth(R(0.04), R(0.48), lysis) * waterExposure;
      const R dmLysed = Min(lysableHeadroom, mass * Clamp(fragility * kLysis * R(1.95) * dtv, R(0), R(0.16)));
      if (dmLysed > R(1e-7)) {
        mass = Max(R(0), mass - dmLysed);
        splat_trilinear(splatL, ClampV(uvw, R(0.002), R(0.998)), dmLysed, R(1e-7));
      }
    }
    q[0] = pos.x; q[1] = pos.y; q[2] = pos.z; q[3] = mass;
    q[4] = stretch.x; q[5] = stretch.y; q[6] = stretch.z; q[7] = ageTicks + Clamp(lysis, R(0), R(0.98));
    const R sLenNow = Len(stretch);
    if (sLenNow < R(0.0038)) {
      splat_trilinear(splatI, ClampV(uvw, R(0.002), R(0.998)), mass, R(1e-6));
    } else {
      const R sxz = Len2(stretch.x, stretch.z);
      const V3<R> horiz = sxz > R(1e-4) ? mk(-stretch.z, R(0), stretch.x) / Max(sxz, R(1e-5)) : mk(R(1), R(0), R(0));
      const V3<R> sheetCross = Cross(stretch, horiz);
      const R scl = Len(sheetCross);
      const V3<R> crossChoice = scl > R(1e-4) ? sheetCross / Max(scl, R(1e-5)) : horiz;
      const R horizMix = Smooth(R(0.35), R(0.85), (R)std::fabs(stretch.y) / Max(sLenNow, R(1e-5)));
      const V3<R> sheetNorm = Normalize(MixV(crossChoice, horiz, horizMix));
      const R sheetSpan = Clamp(sLenNow * R(0.62), R(0.0032), R(0.0085));
      const V3<R> sheetVec = sheetNorm * sheetSpan;
      const V3<R> uvw0 = ClampV(to_uvw(pos - R(0.42) * stretch), R(0.002), R(0.998));
      const V3<R> uvw1 = ClampV(to_uvw(pos - R(0.14) * stretch + sheetVec), R(0.002), R(0.998));
      const V3<R> uvw2 = ClampV(to_uvw(pos + R(0.14) * stretch - sheetVec), R(0.002), R(0.998));
      const V3<R> uvw3 = ClampV(to_uvw(pos + R(0.42) * stretch), R(0.002), R(0.998));
      splat_trilinear(splatI, uvw0, R(0.21) * mass, R(1e-6));
      splat_trilinear(splatI, uvw1, R(0.29) * mass, R(1e-6));
      splat_trilinear(splatI, uvw2, R(0.29) * mass, R(1e-6));
      splat_trilinear(splatI, uvw3, R(0.21) * mass, R(1e-6));
    }
  }
  // Closed box: plain Ralston RK3 tracer on the centre velocity, clamped to
  // the box interior, 1-point trilinear fixed-point splat of its mass.
  void parcel_advect_box_one(uint32_t gid) {
    R* q = &parcels[(size_t)gid * 8];
    const R mass = q[3];
    if (mass <= R(1e-6)) return;
    const R dtv = dt();
    V3<R> pos = mk(q[0], q[1], q[2]);
    auto vel = [&](V3<R> pp) { return sample_center(ClampV(to_uvw(pp), R(0.002), R(0.998))); };
    const V3<R> v1 = vel(pos);
    const V3<R> v2 = vel(pos + R(0.5) * v1 * dtv);
    const V3<R> v3 = vel(pos + R(0.75) * v2 * dtv);
    const V3<R> vAdv = R(2.0 / 9.0) * v1 + R(3.0 / 9.0) * v2 + R(4.0 / 9.0) * v3;
    pos = pos + vAdv * dtv;
    const V3<R> lo = dmin() + dsize() * R(0.002);
    const V3<R> hi = dmax() - dsize() * R(0.002);
    pos = mk(Clamp(pos.x, lo.x, hi.x), Clamp(pos.y, lo.y, hi.y), Clamp(pos.z, lo.z, hi.z));
    q[0] = pos.x; q[1] = pos.y; q[2] = pos.z;
    splat_trilinear(splatI, ClampV(to_uvw(pos), R(0.002), R(0.998)), mass, R(1e-6));
  }
  uint32_t advect_count() const {
    const uint32_t hw = (uint32_t)(((uint64_t)highWater + 255u) / 256u * 256u);
    return hw < cap ? hw : cap;
  }
  void parcel_advect() {
    const uint32_t n = advect_count();
#pragma omp parallel for schedule(static)
    for (long long g = 0; g < (long long)n; ++g) {
      if (ref) parcel_advect_ref_one((uint32_t)g);
      else parcel_advect_box_one((uint32_t)g);
    }
  }

  // ---- CONC_PREDICT (advect.ts:28-72) -------------------------------------------------------
  void conc_predict() {
    const V3<R> dims = cdims();
    const R dtv = dt();
    const V3<R> dom = dsize();
#pragma omp parallel for schedule(static)
    for (int z = 0; z < dc.nz; ++z)
      for (int y = 0; y < dc.ny; ++y)
        for (int x = 0; x < dc.nx; ++x) {
          const size_t i = dc.at(x, y, z);
          const V3<R> uvw = (mk((R)x, (R)y, (R)z) + mk(R(0.5), R(0.5), R(0.5))) / dims;
          if (ref) {
            if (x == 0 || x >= dc.nx - 1 || z == 0 || z >= dc.nz - 1 || y >= dc.ny - 1) { pred[i] = R(0); continue; }
            const V3<R> v0 = sample_center(uvw);
            const R speed2 = Dot(v0, v0);
            if (speed2 < R(2.5e-5)) { pred[i] = st_dye(conc[1][i]); continue; }
            V3<R> back;
            if (speed2 < R(0.012)) {
              back = ClampV(uvw - (v0 * dtv) / dom, R(0.001), R(0.999));
            } else {
              const V3<R> mid = ClampV(uvw - (R(0.5) * (v0 * dtv)) / dom, R(0.001), R(0.999));
              const V3<R> vMid = sample_center(mid);
              back = ClampV(uvw - (vMid * dtv) / dom, R(0.001), R(0.999));
            }
            pred[i] = st_dye(sample_scalar(dc, conc[1], back));
          } else {
            const V3<R> v0 = sample_center(uvw);
            const V3<R> mid = ClampV(uvw - (R(0.5) * (v0 * dtv)) / dom, R(0.001), R(0.999));
            const V3<R> vMid = sample_center(mid);
            const V3<R> back = ClampV(uvw - (vMid * dtv) / dom, R(0.001), R(0.999));
            pred[i] = st_dye(sample_scalar(dc, conc[0], back));
          }
        }
  }

  // ---- CONC_RESOLVE (advect.ts:81-298) --------------------------------------------------------
  R ldc(const std::vector<R>& a, int x, int y, int z) const {
    return a[dc.at(ClampI(x, 0, dc.nx - 1), ClampI(y, 0, dc.ny - 1), ClampI(z, 0, dc.nz - 1))];
  }
  R intact_raw(int x, int y, int z) const {
    return (R)splatI[dc.at(ClampI(x, 0, dc.nx - 1), ClampI(y, 0, dc.ny - 1), ClampI(z, 0, dc.nz - 1))] * R(1.52587891e-5);
  }
  void conc_resolve_ref() {
    const V3<R> dims = cdims();
    const R dtv = dt();
    const V3<R> dom = dsize();
    const R halfXZ = (R)U[52], yMin = (R)U[53];
    const R sharpness = (R)U[47];
#pragma omp parallel for schedule(static)
    for (int z = 0; z < dc.nz; ++z)
      for (int y = 0; y < dc.ny; ++y)
        for (int x = 0; x < dc.nx; ++x) {
          const size_t i = dc.at(x, y, z);
          auto out = [&](R r, R g, R b, R a) {
            concN[0][i] = st_dye(r); concN[1][i] = st_dye(g); concN[2][i] = st_dye(b); concN[3][i] = st_dye(a);
          };
          if (x == 0 || x >= dc.nx - 1 || z == 0 || z >= dc.nz - 1 || y >= dc.ny - 1) { out(0, 0, 0, 0); continue; }
          const uint32_t rawIntact = splatI[i], rawLysed = splatL[i];
          const bool inFloorZone = y <= 7;
          if (rawIntact == 0u && rawLysed == 0u) {
            const R oct0 = sample_scalar(dc, pred, mk((R)x, (R)y, (R)z) / dims);
            const R oct1 = sample_scalar(dc, pred, (mk((R)x, (R)y, (R)z) + mk(R(1), R(1), R(1))) / dims);
            R bedActive = R(0);
            if (inFloorZone) bedActive = sample_scalar(dc, conc[3], (mk((R)x, (R)y, (R)z) + mk(R(0.5), R(0.5), R(0.5))) / dims);
            if (oct0 + oct1 <= R(1.0e-7) && bedActive <= R(1.0e-6)) { out(0, 0, 0, 0); continue; }
          }
          const R gPred = pred[i];
          const R lapNeighborsG = (ldc(pred, x + 1, y, z) + ldc(pred, x - 1, y, z) + ldc(pred, x, y + 1, z) + ldc(pred, x, y - 1, z) +
                                   ldc(pred, x, y, z + 1) + ldc(pred, x, y, z - 1)) * (R(1) / R(6));
          if (!inFloorZone && rawIntact == 0u && rawLysed == 0u && gPred <= R(1.2e-6) && lapNeighborsG <= R(1.2e-6)) {
            out(0, 0, 0, 0);
            continue;
          }
          R lapIntact = R(0);
          const bool loadNeighborhood = rawIntact > 0u || gPred > R(8.0e-5) || lapNeighborsG > R(8.0e-5);
          if (loadNeighborhood)
            lapIntact = (intact_raw(x + 1, y, z) + intact_raw(x - 1, y, z) + intact_raw(x, y + 1, z) + intact_raw(x, y - 1, z) +
                         intact_raw(x, y, z + 1) + intact_raw(x, y, z - 1)) * (R(1) / R(6));
          const V3<R> uvw = (mk((R)x, (R)y, (R)z) + mk(R(0.5), R(0.5), R(0.5))) / dims;
          const V3<R> pw = to_world(uvw);
          const V3<R> v0 = sample_center(uvw);
          const V3<R> uvwMid = ClampV(uvw - (R(0.5) * (v0 * dtv)) / dom, R(0.001), R(0.999));
          const V3<R> vMid = sample_center(uvwMid);
          const V3<R> uvwBack = ClampV(uvw - (vMid * dtv) / dom, R(0.001), R(0.999));
          const V3<R> uvwFwd = ClampV(uvw + (v0 * dtv) / dom, R(0.001), R(0.999));
          const R gBackEst = sample_scalar(dc, pred, uvwFwd);
          const R gOrig = conc[1][i];
          const R gCorr = gPred + (R(0.45) * sharpness) * (gOrig - gBackEst);
          const V3<R> tc = uvwBack * dims - mk(R(0.5), R(0.5), R(0.5));
          const int bx = (int)Floor(tc.x), by = (int)Floor(tc.y), bz = (int)Floor(tc.z);
          const R s000 = ldc(conc[1], bx, by, bz), s100 = ldc(conc[1], bx + 1, by, bz);
          const R s010 = ldc(conc[1], bx, by + 1, bz), s110 = ldc(conc[1], bx + 1, by + 1, bz);
          const R s001 = ldc(conc[1], bx, by, bz + 1), s101 = ldc(conc[1], bx + 1, by, bz + 1);
          const R s011 = ldc(conc[1], bx, by + 1, bz + 1), s111 = ldc(conc[1], bx + 1, by + 1, bz + 1);
          const R minG = Min(Min(Min(s000, s100), Min(s010, s110)), Min(Min(s001, s101), Min(s011, s111)));
          const R maxG = Max(Max(Max(s000, s100), Max(s010, s110)), Max(Max(s001, s101), Max(s011, s111)));
          R cLysed = Clamp(gCorr, minG, maxG);
          const R diffBlend = Clamp(dtv * R(5.60), R(0), R(0.105));
          cLysed = Mix(cLysed, lapNeighborsG, diffBlend);
          const R upperDilute = Exp(-dtv * Mix(R(0.016), R(0.034), Smooth(yMin + R(0.045), yMin + R(0.26), pw.y)));
          cLysed = cLysed * upperDilute;
          const R dmTransfer = (R)rawLysed * R(1.52587891e-5);
          const R floorBedCapture = R(1) - Smooth(yMin + R(0.018), yMin + R(0.058), pw.y);
          cLysed = cLysed + dmTransfer * (R(1) - floorBedCapture * R(0.72));
          if (cLysed < R(2.5e-6)) cLysed = R(0);
          const R rHoriz = Len2(pw.x, pw.z);
          R cBed = R(0);
          if (inFloorZone) {
            const R bCenter = ldc(conc[3], x, y, z);
            const R bHoriz = R(0.25) * (ldc(conc[3], x + 1, y, z) + ldc(conc[3], x - 1, y, z) + ldc(conc[3], x, y, z + 1) + ldc(conc[3], x, y, z - 1));
            const R bAbove = ldc(conc[3], x, y + 1, z);
            const R bBelow = ldc(conc[3], x, std::max(0, y - 1), z);
            const R spreadAlpha = Clamp(dtv * (R(3.20) + R(6.50) * Min(bCenter, R(0.65))), R(0), R(0.165));
            const R vertDiffuse = Clamp(dtv * R(0.75), R(0), R(0.026));
            const R settleAlpha = Clamp(dtv * R(2.80), R(0), R(0.090));
            const R bedDecay = Exp(-dtv * Mix(R(0.095), R(0.28), Smooth(halfXZ * R(0.35), halfXZ * R(0.78), rHoriz)));
            const R drainedSelf = (y == 0 ? bCenter : bCenter * (R(1) - settleAlpha)) * bedDecay;
            const R settledFromAbove = y >= 7 ? R(0) : bAbove * settleAlpha;
            const R advectedBed = drainedSelf + settledFromAbove;
            const R smoothedBed = Mix(Mix(advectedBed, bHoriz, spreadAlpha), R(0.5) * (bAbove + bBelow), vertDiffuse);
            const R topBedFade = R(1) - R(0.38) * Smooth(R(3.5), R(7.0), (R)y);
            cBed = (smoothedBed + dmTransfer * floorBedCapture * R(0.68)) * topBedFade;
            if (cBed < R(1.0e-6)) cBed = R(0);
          }
          const R wallSponge = R(1) - Smooth(halfXZ * R(0.68), halfXZ * R(0.94), rHoriz);
          const R floorRadialTaper = R(1) - Smooth(halfXZ * R(0.52), halfXZ * R(0.88), rHoriz);
          const R maxBedProfile = R(0.54) * Exp(R(-0.56) * (R)y) * floorRadialTaper;
          cBed = Min(cBed * wallSponge, maxBedProfile);
          const R cParcelRaw = (R)rawIntact * R(1.52587891e-5);
          const R shoulderFeather = rawIntact > 0u ? R(0.36) : R(0.18);
          const R cParcelIntact = Mix(cParcelRaw, lapIntact, shoulderFeather) * wallSponge;
          const R cIntact = cParcelIntact + cBed;
          cLysed = cLysed * wallSponge;
          const R cTotal = cIntact + cLysed;
          R vOx = R(0);
          if (cTotal > R(1.0e-5)) {
            const R fLysis = Clamp(cLysed / Max(cTotal, R(1.0e-5)), R(0), R(1));
            const R intactFrac = R(1) - fLysis;
            const R bedFrac = Smooth(R(0), R(0.85), cBed / Max(cTotal, R(1.0e-5)));
            const R flowSpeed = Len(v0);
            const R convShear = Len(v0 - vMid) / Max(R(0.5) * dtv, R(1.0e-3));
            const R shearDispersion = Smooth(R(0.014), R(0.135), flowSpeed + R(0.38) * convShear);
            const R thinIntactSheet = (R(1) - Smooth(R(0.024), R(0.24), cIntact)) * Smooth(R(0.0006), R(0.0065), cIntact);
            const R activeSheet = thinIntactSheet * (R(0.38) + R(0.62) * shearDispersion) * intactFrac;
            const R rawOx = Clamp(R(0.08) + R(0.62) * activeSheet + R(0.36) * shearDispersion * intactFrac, R(0), R(1));
            vOx = rawOx * (R(1) - R(0.82) * bedFrac);
          }
          out(cIntact, cLysed, vOx, cBed);
        }
    for (int c = 0; c < 4; ++c) conc[c].swap(concN[c]);
  }
  // Closed box: MacCormack correction of the single dye with the 8-tap
  // min/max limiter of CONC_RESOLVE (advect.ts:196-222) and nothing else.
  void dye_resolve_box() {
    const V3<R> dims = cdims();
    const R dtv = dt();
    const V3<R> dom = dsize();
    const R sharpness = (R)cfg.dye_sharpness;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < dc.nz; ++z)
      for (int y = 0; y < dc.ny; ++y)
        for (int x = 0; x < dc.nx; ++x) {
          const size_t i = dc.at(x, y, z);
          const V3<R> uvw = (mk((R)x, (R)y, (R)z) + mk(R(0.5), R(0.5), R(0.5))) / dims;
          const V3<R> v0 = sample_center(uvw);
          const V3<R> uvwMid = ClampV(uvw - (R(0.5) * (v0 * dtv)) / dom, R(0.001), R(0.999));
          const V3<R> vMid = sample_center(uvwMid);
          const V3<R> uvwBack = ClampV(uvw - (vMid * dtv) / dom, R(0.001), R(0.999));
          const V3<R> uvwFwd = ClampV(uvw + (v0 * dtv) / dom, R(0.001), R(0.999));
          const R gBackEst = sample_scalar(dc, pred, uvwFwd);
          const R gOrig = conc[0][i];
          const R gCorr = pred[i] + (R(0.45) * sharpness) * (gOrig - gBackEst);
          const V3<R> tc = uvwBack * dims - mk(R(0.5), R(0.5), R(0.5));
          const int bx = (int)Floor(tc.x), by = (int)Floor(tc.y), bz = (int)Floor(tc.z);
          const R s000 = ldc(conc[0], bx, by, bz), s100 = ldc(conc[0], bx + 1, by, bz);
          const R s010 = ldc(conc[0], bx, by + 1, bz), s110 = ldc(conc[0], bx + 1, by + 1, bz);
          const R s001 = ldc(conc[0], bx, by, bz + 1), s101 = ldc(conc[0], bx + 1, by, bz + 1);
          const R s011 = ldc(conc[0], bx, by + 1, bz + 1), s111 = ldc(conc[0], bx + 1, by + 1, bz + 1);
          const R minG = Min(Min(Min(s000, s100), Min(s010, s110)), Min(Min(s001, s101), Min(s011, s111)));
          const R maxG = Max(Max(Max(s000, s100), Max(s010, s110)), Max(Max(s001, s101), Max(s011, s111)));
          concN[0][i] = st_dye(Clamp(gCorr, minG, maxG));
        }
    conc[0].swap(concN[0]);
  }

  // ---- injection (closed box) ---------------------------------------------------------------------
  void inject_sphere(const float c[3], float radius, float dye, const float vel[3], float sigma, uint64_t seed) {
    inject_pending = kInjectedSteps;
    const V3<R> cc = mk((R)c[0], (R)c[1], (R)c[2]);
    const R rr = (R)radius;
    const V3<R> dims = vdims();
    const V3<R> cdm = cdims();
    for (int z = 0; z < dc.nz; ++z)
      for (int y = 0; y < dc.ny; ++y)
        for (int x = 0; x < dc.nx; ++x) {
          const V3<R> pw = to_world((mk((R)x, (R)y, (R)z) + mk(R(0.5), R(0.5), R(0.5))) / cdm);
          if (Len(pw - cc) <= rr) conc[0][dc.at(x, y, z)] = st_dye((R)dye);
        }
    for (int z = 0; z < dv.nz; ++z)
      for (int y = 0; y < dv.ny; ++y)
        for (int x = 0; x < dv.nx; ++x) {
          const size_t i = dv.at(x, y, z);
          const V3<R> fx = to_world(mk((R)x + R(1), (R)y + R(0.5), (R)z + R(0.5)) / dims);
          const V3<R> fy = to_world(mk((R)x + R(0.5), (R)y + R(1), (R)z + R(0.5)) / dims);
          const V3<R> fz = to_world(mk((R)x + R(0.5), (R)y + R(0.5), (R)z + R(1)) / dims);
          if (x < dv.nx - 1 && Len(fx - cc) <= rr) u[i] = st_vel((R)(vel[0] + sigma * dob_sphere_noise(seed, i, 0)));
          if (y < dv.ny - 1 && Len(fy - cc) <= rr) v[i] = st_vel((R)(vel[1] + sigma * dob_sphere_noise(seed, i, 1)));
          if (z < dv.nz - 1 && Len(fz - cc) <= rr) w[i] = st_vel((R)(vel[2] + sigma * dob_sphere_noise(seed, i, 2)));
        }
  }

  // soft-edged additive drop (dob_inject_sphere_soft)
  void inject_sphere_soft(const float c[3], float radius, float edge, float dye, const float vel[3], float sigma,
                          uint64_t seed) {
    inject_pending = kInjectedSteps;
    const V3<R> cc = mk((R)c[0], (R)c[1], (R)c[2]);
    const R rr = (R)radius, hh = (R)edge;
    const V3<R> dims = vdims();
    const V3<R> cdm = cdims();
    V3<R> g;
    for (int z = 0; z < dc.nz; ++z)
      for (int y = 0; y < dc.ny; ++y)
        for (int x = 0; x < dc.nx; ++x) {
          const V3<R> pw = to_world((mk((R)x, (R)y, (R)z) + mk(R(0.5), R(0.5), R(0.5))) / cdm);
          const R wt = SoftSphere(pw, cc, rr, hh, g);
          const size_t k = dc.at(x, y, z);
          if (wt > R(0)) conc[0][k] = st_dye(conc[0][k] + wt * (R)dye);
        }
    for (int z = 0; z < dv.nz; ++z)
      for (int y = 0; y < dv.ny; ++y)
        for (int x = 0; x < dv.nx; ++x) {
          const size_t i = dv.at(x, y, z);
          const V3<R> fx = to_world(mk((R)x + R(1), (R)y + R(0.5), (R)z + R(0.5)) / dims);
          const V3<R> fy = to_world(mk((R)x + R(0.5), (R)y + R(1), (R)z + R(0.5)) / dims);
          const V3<R> fz = to_world(mk((R)x + R(0.5), (R)y + R(0.5), (R)z + R(1)) / dims);
          R wt = SoftSphere(fx, cc, rr, hh, g);
          if (x < dv.nx - 1 && wt > R(0)) u[i] = st_vel(u[i] + wt * (R)(vel[0] + sigma * dob_sphere_noise(seed, i, 0)));
          wt = SoftSphere(fy, cc, rr, hh, g);
          if (y < dv.ny - 1 && wt > R(0)) v[i] = st_vel(v[i] + wt * (R)(vel[1] + sigma * dob_sphere_noise(seed, i, 1)));
          wt = SoftSphere(fz, cc, rr, hh, g);
          if (z < dv.nz - 1 && wt > R(0)) w[i] = st_vel(w[i] + wt * (R)(vel[2] + sigma * dob_sphere_noise(seed, i, 2)));
        }
  }

  // ---- statistics -------------------------------------------------------------------------------
  double max_div() const {
    const double scale = ref ? 1.0 : (double)cfg.dt / (double)cfg.dx;
    double m = 0.0;
#pragma omp parallel for reduction(max : m) schedule(static)
    for (int z = 0; z < dv.nz; ++z)
      for (int y = 0; y < dv.ny; ++y)
        for (int x = 0; x < dv.nx; ++x) {
          double d = (double)divergence(x, y, z);
          if (ref && y == dv.ny - 1) continue;  // the top row carries the free-surface flux
          m = std::max(m, std::fabs(d) * scale);
        }
    return m;
  }

  // ---- one step in the reference's order (BloodDropEngine.ts:1855-2111) ----------------------
  void run_stage(int st) {
    switch (st) {
      case DOB_STAGE_ADVECT_MAC: advect_mac(); break;
      case DOB_STAGE_MAC_TO_CENTER: mac_to_center(); break;
      case DOB_STAGE_CURL: curl_stage(); break;
      case DOB_STAGE_CASSON_FORCES: casson_forces(); break;
      case DOB_STAGE_MAC_RHS: mac_rhs(); break;
      case DOB_STAGE_PRESSURE_SOLVE: pressure_solve(); break;
      case DOB_STAGE_PROJECT: project(); break;
      case DOB_STAGE_CLEAR_SPLATS:
        std::fill(splatI.begin(), splatI.end(), 0u);
        std::fill(splatL.begin(), splatL.end(), 0u);
        break;
      case DOB_STAGE_PARCEL_EMIT: parcel_emit(); break;
      case DOB_STAGE_PARCEL_ADVECT: parcel_advect(); break;
      case DOB_STAGE_CONC_PREDICT: conc_predict(); break;
      case DOB_STAGE_CONC_RESOLVE:
        if (ref) conc_resolve_ref(); else dye_resolve_box();
        break;
      default: break;
    }
  }
  // steps left that run cfg.mg_cycles_injected V-cycles (FP32 pressure): an
  // injection covers the injection step and the next, as the library does
  static constexpr int kInjectedSteps = 2;
  int inject_pending = 0;
  int cycles_override = 0;
  void step(bool want_stats) {
    const bool injected = inject_pending > 0 && cfg.mg_cycles_injected > 0 && !mixed() &&
                          cfg.mg_cycles_injected != cfg.mg_cycles;
    if (inject_pending > 0) --inject_pending;
    if (ref) {  // BloodDropEngine.ts:1832-1840: the high-water mark grows by the spawn count first
      const uint64_t hw = (uint64_t)highWater + spawn_count();
      highWater = (uint32_t)(hw < cap ? hw : cap);
    }
    if (flag(DOB_PHYS_WAVE)) wave_step();  // BloodDropEngine.ts:1886-1912, before the advection
    advect_mac();
    mac_to_center();
    if (flag(DOB_PHYS_VORT_CONF)) curl_stage();
    casson_forces();
    mac_rhs();
    if (want_stats) last_stats[0] = sqrt(dot64(rhs, rhs));
    cycles_override = injected ? cfg.mg_cycles_injected : 0;
    pressure_solve();
    cycles_override = 0;
    if (want_stats) last_stats[1] = mixed() ? residual64(nullptr, nullptr) : residual_l2(p, rhs, nullptr);
    project();
    if (want_stats) last_stats[2] = max_div();
    mac_to_center();
    std::fill(splatI.begin(), splatI.end(), 0u);
    std::fill(splatL.begin(), splatL.end(), 0u);
    parcel_emit();
    parcel_advect();
    conc_predict();
    if (ref) conc_resolve_ref(); else dye_resolve_box();
  }

#include "dob_oracle_adjoint.inc"
#include "dob_oracle_wave.inc"
#include "dob_oracle_light.inc"
#include "dob_oracle_render.inc"
};

struct AnySim {
  bool f64;
  Sim<float>* sf = nullptr;
  Sim<double>* sd = nullptr;
};

template <class R> std::vector<R>* adj_array(Sim<R>& s, int field) {
  switch (field) {
    case DOB_FIELD_ADJ_VEL_U: return &s.au;
    case DOB_FIELD_ADJ_VEL_V: return &s.av;
    case DOB_FIELD_ADJ_VEL_W: return &s.aw;
    case DOB_FIELD_ADJ_VEL_U2: return &s.au2;
    case DOB_FIELD_ADJ_VEL_V2: return &s.av2;
    case DOB_FIELD_ADJ_VEL_W2: return &s.aw2;
    case DOB_FIELD_ADJ_CONC: return &s.ac;
    case DOB_FIELD_ADJ_CONC2: return &s.ac2;
    case DOB_FIELD_ADJ_PRED: return &s.apred;
    case DOB_FIELD_ADJ_PRESSURE: return &s.ap;
    case DOB_FIELD_ADJ_RHS: return &s.arhs;
    default: return nullptr;
  }
}

template <class R> int set_field(Sim<R>& s, int field, const void* host, size_t bytes) {
  const size_t N = s.dv.n(), Nc = s.dc.n();
  auto put = [&](std::vector<R>& a, size_t n) -> int {
    if (bytes != n * sizeof(float)) return DOB_EINVAL;
    const float* f = (const float*)host;
    for (size_t i = 0; i < n; ++i) a[i] = (R)f[i];
    return DOB_OK;
  };
  auto put4 = [&](std::vector<R>* a, int nch, size_t n) -> int {
    if (bytes != n * nch * sizeof(float)) return DOB_EINVAL;
    const float* f = (const float*)host;
    for (size_t i = 0; i < n; ++i)
      for (int c = 0; c < nch; ++c) a[c][i] = (R)f[i * nch + c];
    return DOB_OK;
  };
  switch (field) {
    case DOB_FIELD_VEL_U: return put(s.u, N);
    case DOB_FIELD_VEL_V: return put(s.v, N);
    case DOB_FIELD_VEL_W: return put(s.w, N);
    case DOB_FIELD_VEL_CENTER: return put4(s.cen, 4, N);
    case DOB_FIELD_CURL: return put4(s.curl, 4, N);
    case DOB_FIELD_PRESSURE: {
      const int rc = put(s.p, N);
      if (rc == DOB_OK && s.mixed()) for (size_t i = 0; i < N; ++i) s.p64[i] = (double)s.p[i];
      return rc;
    }
    case DOB_FIELD_RHS: return put(s.rhs, N);
    case DOB_FIELD_CONC: return s.nconc == 4 ? put4(s.conc, 4, Nc) : put(s.conc[0], Nc);
    case DOB_FIELD_CONC_PRED: return put(s.pred, Nc);
    case DOB_FIELD_SPLAT_INTACT:
    case DOB_FIELD_SPLAT_LYSED: {
      if (bytes != Nc * 4) return DOB_EINVAL;
      auto& d = field == DOB_FIELD_SPLAT_INTACT ? s.splatI : s.splatL;
      memcpy(d.data(), host, bytes);
      return DOB_OK;
    }
    case DOB_FIELD_WAVE:
      if (bytes != s.wave.size() * 4) return DOB_EINVAL;
      memcpy(s.wave.data(), host, bytes);
      return DOB_OK;
    default: break;
  }
  if (field >= DOB_FIELD_ADJ_VEL_U && field <= DOB_FIELD_ADJ_RHS) {
    s.adj_alloc();
    if (field == DOB_FIELD_ADJ_CENTER) {
      if (bytes != N * 4 * sizeof(float)) return DOB_EINVAL;
      const float* f = (const float*)host;
      for (size_t i = 0; i < N; ++i)
        for (int c = 0; c < 3; ++c) s.acen[c][i] = (R)f[i * 4 + c];
      return DOB_OK;
    }
    std::vector<R>* a = adj_array(s, field);
    return put(*a, a->size());
  }
  return DOB_EINVAL;
}

template <class R> int get_field(Sim<R>& s, int field, void* host, size_t bytes) {
  const size_t N = s.dv.n(), Nc = s.dc.n();
  auto get = [&](const std::vector<R>& a, size_t n) -> int {
    if (bytes != n * sizeof(float)) return DOB_EINVAL;
    float* f = (float*)host;
    for (size_t i = 0; i < n; ++i) f[i] = (float)a[i];
    return DOB_OK;
  };
  auto get4 = [&](const std::vector<R>* a, int nch, size_t n) -> int {
    if (bytes != n * nch * sizeof(float)) return DOB_EINVAL;
    float* f = (float*)host;
    for (size_t i = 0; i < n; ++i)
      for (int c = 0; c < nch; ++c) f[i * nch + c] = (float)a[c][i];
    return DOB_OK;
  };
  switch (field) {
    case DOB_FIELD_VEL_U: return get(s.u, N);
    case DOB_FIELD_VEL_V: return get(s.v, N);
    case DOB_FIELD_VEL_W: return get(s.w, N);
    case DOB_FIELD_VEL_CENTER: return get4(s.cen, 4, N);
    case DOB_FIELD_CURL: return get4(s.curl, 4, N);
    case DOB_FIELD_PRESSURE:
      if (s.mixed()) {
        if (bytes != N * sizeof(float)) return DOB_EINVAL;
        for (size_t i = 0; i < N; ++i) ((float*)host)[i] = (float)s.p64[i];
        return DOB_OK;
      }
      return get(s.p, N);
    case DOB_FIELD_RHS: return get(s.rhs, N);
    case DOB_FIELD_CONC: return s.nconc == 4 ? get4(s.conc, 4, Nc) : get(s.conc[0], Nc);
    case DOB_FIELD_CONC_PRED: return get(s.pred, Nc);
    case DOB_FIELD_SPLAT_INTACT:
    case DOB_FIELD_SPLAT_LYSED: {
      if (bytes != Nc * 4) return DOB_EINVAL;
      const auto& d = field == DOB_FIELD_SPLAT_INTACT ? s.splatI : s.splatL;
      memcpy(host, d.data(), bytes);
      return DOB_OK;
    }
    case DOB_FIELD_WAVE:
      if (bytes != s.wave.size() * 4) return DOB_EINVAL;
      memcpy(host, s.wave.data(), bytes);
      return DOB_OK;
    case DOB_FIELD_LIGHT:
      if (s.light.size() != 4 * N) return DOB_ESTATE;
      return get(s.light, 4 * N);
    case DOB_FIELD_BRICKS:
    case DOB_FIELD_BRICKS_RAW: {
      const auto& b = field == DOB_FIELD_BRICKS ? s.bricks : s.brickRaw;
      if (b.empty()) return DOB_ESTATE;
      return get(b, b.size());
    }
    case DOB_FIELD_DIVERGENCE: {
      if (bytes != N * sizeof(float)) return DOB_EINVAL;
      float* f = (float*)host;
      for (int z = 0; z < s.dv.nz; ++z)
        for (int y = 0; y < s.dv.ny; ++y)
          for (int x = 0; x < s.dv.nx; ++x) f[s.dv.at(x, y, z)] = (float)s.divergence(x, y, z);
      return DOB_OK;
    }
    default: break;
  }
  if (field >= DOB_FIELD_ADJ_VEL_U && field <= DOB_FIELD_ADJ_RHS) {
    s.adj_alloc();
    if (field == DOB_FIELD_ADJ_CENTER) {
      if (bytes != N * 4 * sizeof(float)) return DOB_EINVAL;
      float* f = (float*)host;
      for (size_t i = 0; i < N; ++i) {
        for (int c = 0; c < 3; ++c) f[i * 4 + c] = (float)s.acen[c][i];
        f[i * 4 + 3] = 0.0f;
      }
      return DOB_OK;
    }
    const std::vector<R>* a = adj_array(s, field);
    return get(*a, a->size());
  }
  return DOB_EINVAL;
}
// Channel arrays of a field for the double-precision interface: returns the
// channel count (0 if the field has no FP64 access).
template <class R> int field_arrays(Sim<R>& s, int field, std::vector<R>* a[4]) {
  switch (field) {
    case DOB_FIELD_VEL_U: a[0] = &s.u; return 1;
    case DOB_FIELD_VEL_V: a[0] = &s.v; return 1;
    case DOB_FIELD_VEL_W: a[0] = &s.w; return 1;
    case DOB_FIELD_VEL_CENTER: for (int c = 0; c < 4; ++c) a[c] = &s.cen[c]; return 4;
    case DOB_FIELD_PRESSURE: a[0] = &s.p; return 1;
    case DOB_FIELD_RHS: a[0] = &s.rhs; return 1;
    case DOB_FIELD_CONC: if (s.nconc != 1) return 0; a[0] = &s.conc[0]; return 1;
    case DOB_FIELD_CONC_PRED: a[0] = &s.pred; return 1;
    default: break;
  }
  if (field >= DOB_FIELD_ADJ_VEL_U && field <= DOB_FIELD_ADJ_RHS && field != DOB_FIELD_ADJ_CENTER) {
    s.adj_alloc();
    a[0] = adj_array(s, field);
    return 1;
  }
  return 0;
}
// double-precision field access (interleaved channels like the float API)
template <class R> int get_field64(Sim<R>& s, int field, double* host, size_t n) {
  if (field == DOB_FIELD_PRESSURE && s.mixed()) {  // the defect loop's high-precision pressure
    if (n != s.p64.size()) return DOB_EINVAL;
    for (size_t i = 0; i < n; ++i) host[i] = s.p64[i];
    return DOB_OK;
  }
  std::vector<R>* a[4];
  const int nch = field_arrays(s, field, a);
  if (nch == 0 || n != a[0]->size() * nch) return DOB_EINVAL;
  for (size_t i = 0; i < a[0]->size(); ++i)
    for (int c = 0; c < nch; ++c) host[i * nch + c] = (double)(*a[c])[i];
  return DOB_OK;
}
template <class R> int set_field64(Sim<R>& s, int field, const double* host, size_t n) {
  if (field == DOB_FIELD_PRESSURE && s.mixed()) {
    if (n != s.p64.size()) return DOB_EINVAL;
    for (size_t i = 0; i < n; ++i) { s.p64[i] = host[i]; s.p[i] = (R)host[i]; }
    return DOB_OK;
  }
  std::vector<R>* a[4];
  const int nch = field_arrays(s, field, a);
  if (nch == 0 || n != a[0]->size() * nch) return DOB_EINVAL;
  for (size_t i = 0; i < a[0]->size(); ++i)
    for (int c = 0; c < nch; ++c) (*a[c])[i] = (R)host[i * nch + c];
  return DOB_OK;
}

bool valid_config(const dob_config* c) {
  if (!c || c->struct_size != sizeof(dob_config)) return false;
  if (c->nx < 4 || c->ny < 4 || c->nz < 4) return false;
  if (c->dye_refine != 1 && c->dye_refine != 2) return false;
  if (c->mg_levels < 1 || c->mg_levels > 10) return false;
  const uint32_t m = 1u << c->mg_levels;  // even dims on every level, like the library
  if (c->nx % m || c->ny % m || c->nz % m) return false;
  if (c->mg_coarse_sweeps < -1) return false;
  if (c->mg_coarse_sweeps == -1 &&
      (uint64_t)(c->nx >> (c->mg_levels - 1)) * (c->ny >> (c->mg_levels - 1)) * (c->nz >> (c->mg_levels - 1)) > 4096)
    return false;
  if (c->bc_mode != DOB_BC_REFERENCE && c->bc_mode != DOB_BC_CLOSED_BOX) return false;
  if (c->precision_mode < 0 || c->precision_mode > 2) return false;
  if (c->parcel_capacity < 1) return false;
  return true;
}

}  // namespace

struct orc_sim {
  AnySim a;
};

template <class R> int set_par(Sim<R>* s, const float* p, uint32_t n, uint32_t off) {
  if ((uint64_t)off + n > s->cap) return DOB_EINVAL;
  for (size_t i = 0; i < (size_t)n * 8; ++i) s->parcels[(size_t)off * 8 + i] = (R)p[i];
  const uint32_t hw = off + n;
  if (hw > s->highWater) s->highWater = hw;
  return DOB_OK;
}
template <class R> int get_par(Sim<R>* s, float* p, uint32_t n, uint32_t off) {
  if ((uint64_t)off + n > s->cap) return DOB_EINVAL;
  for (size_t i = 0; i < (size_t)n * 8; ++i) p[i] = (float)s->parcels[(size_t)off * 8 + i];
  return DOB_OK;
}


#define DISPATCH(s, call) ((s)->a.f64 ? (s)->a.sd->call : (s)->a.sf->call)

extern "C" {

orc_sim* orc_create(const dob_config* cfg, int fp64) {
  if (!valid_config(cfg)) return nullptr;
  orc_sim* s = new orc_sim();
  s->a.f64 = fp64 != 0;
  if (s->a.f64) s->a.sd = new Sim<double>(*cfg, true);
  else s->a.sf = new Sim<float>(*cfg, false);
  DISPATCH(s, reset());
  return s;
}
void orc_destroy(orc_sim* s) {
  if (!s) return;
  delete s->a.sf;
  delete s->a.sd;
  delete s;
}
int orc_reset(orc_sim* s) { DISPATCH(s, reset()); return DOB_OK; }
int orc_set_uniforms(orc_sim* s, const float u[128]) {
  if (s->a.f64) memcpy(s->a.sd->U, u, 512); else memcpy(s->a.sf->U, u, 512);
  return DOB_OK;
}
int orc_inject_sphere(orc_sim* s, const float c[3], float r, float dye, const float vel[3], float sigma, uint64_t seed) {
  if (DISPATCH(s, ref)) return DOB_ESTATE;
  DISPATCH(s, inject_sphere(c, r, dye, vel, sigma, seed));
  return DOB_OK;
}
int orc_inject_sphere_soft(orc_sim* s, const float c[3], float r, float edge, float dye, const float vel[3],
                           float sigma, uint64_t seed) {
  if (DISPATCH(s, ref)) return DOB_ESTATE;
  if (!(r > 0.0f) || !(edge > 0.0f)) return DOB_EINVAL;
  DISPATCH(s, inject_sphere_soft(c, r, edge, dye, vel, sigma, seed));
  return DOB_OK;
}
int orc_set_parcels(orc_sim* s, const float* p, uint32_t n, uint32_t off) {
  return s->a.f64 ? set_par(s->a.sd, p, n, off) : set_par(s->a.sf, p, n, off);
}
int orc_get_parcels(orc_sim* s, float* p, uint32_t n, uint32_t off) {
  return s->a.f64 ? get_par(s->a.sd, p, n, off) : get_par(s->a.sf, p, n, off);
}
int orc_set_high_water(orc_sim* s, uint32_t hw) {
  if (s->a.f64) s->a.sd->highWater = std::min(hw, s->a.sd->cap);
  else s->a.sf->highWater = std::min(hw, s->a.sf->cap);
  return DOB_OK;
}
int orc_set_field(orc_sim* s, int field, const void* host, size_t bytes) {
  return s->a.f64 ? set_field(*s->a.sd, field, host, bytes) : set_field(*s->a.sf, field, host, bytes);
}
int orc_get_field(orc_sim* s, int field, void* host, size_t bytes) {
  return s->a.f64 ? get_field(*s->a.sd, field, host, bytes) : get_field(*s->a.sf, field, host, bytes);
}
int orc_step(orc_sim* s, int nsteps, double* stats) {
  if (nsteps < 0) return DOB_EINVAL;
  for (int k = 0; k < nsteps; ++k) DISPATCH(s, step(stats != nullptr));
  // DOB_PHYS_LIGHTING: the lighting passes once after the frame's steps
  const dob_config& cfg = s->a.f64 ? s->a.sd->cfg : s->a.sf->cfg;
  if (nsteps > 0 && cfg.bc_mode == DOB_BC_REFERENCE && (cfg.physics_flags & DOB_PHYS_LIGHTING)) DISPATCH(s, light_volume());
  if (stats) {
    const double* ls = s->a.f64 ? s->a.sd->last_stats : s->a.sf->last_stats;
    for (int i = 0; i < 5; ++i) stats[i] = ls[i];
  }
  return DOB_OK;
}
int orc_run_stage(orc_sim* s, int stage) {
  if (stage < 0 || stage >= DOB_STAGE_COUNT) return DOB_EINVAL;
  DISPATCH(s, run_stage(stage));
  return DOB_OK;
}
void orc_set_threads(int n) {
  g_threads = n;
  if (n > 0) omp_set_num_threads(n);
}
int orc_get_threads(void) { return omp_get_max_threads(); }

// The light volume and brick passes (lighting.ts:19-240).
int orc_light_volume(orc_sim* s) { return DISPATCH(s, light_volume()); }
int orc_render_plume(orc_sim* s, const float* lut, int width, int height, uint16_t* out) {
  if (!s || !lut || !out || width < 1 || height < 1) return DOB_EINVAL;
  return DISPATCH(s, render_plume(lut, width, height, out));
}

// The wave substep on the simulation's wave field (wave.ts:55-388).
int orc_wave_step(orc_sim* s) {
  if (s->a.f64) s->a.sd->wave_step(); else s->a.sf->wave_step();
  return DOB_OK;
}
// Unitary 2-D transform of a 512x512 complex field (interleaved re, im; x
// fastest) by the wave passes: rows then columns forward, columns then rows
// inverse.
int orc_wave_fft2(float* data, int inverse) {
  if (!data) return DOB_EINVAL;
  const size_t n = (size_t)2 * kWaveN * kWaveN;
  std::vector<float> a(data, data + n), b(n);
  if (!inverse) { Sim<float>::wave_fft_lines(a, 2, b, true, false); Sim<float>::wave_fft_lines(b, 2, a, false, false); }
  else { Sim<float>::wave_fft_lines(a, 2, b, false, true); Sim<float>::wave_fft_lines(b, 2, a, true, true); }
  memcpy(data, a.data(), n * sizeof(float));
  return DOB_OK;
}
int orc_adjoint_stage(orc_sim* s, int stage) { return DISPATCH(s, adjoint_stage(stage)); }
int orc_tape_forward(orc_sim* s, int nsteps) { return DISPATCH(s, tape_forward(nsteps)); }
int orc_tape_backward(orc_sim* s, const float* dye_grad, size_t bytes) {
  const size_t nc = s->a.f64 ? s->a.sd->dc.n() : s->a.sf->dc.n();
  if (!dye_grad || bytes != nc * sizeof(float)) return DOB_EINVAL;
  return DISPATCH(s, tape_backward(dye_grad));
}
int orc_sphere_impulse(orc_sim* s, const float c[3], float radius, const float vel[3], double* out) {
  if (!out) return DOB_EINVAL;
  *out = DISPATCH(s, sphere_impulse(c, radius, vel));
  return DOB_OK;
}
int orc_sphere_soft_grad(orc_sim* s, const float c[3], float radius, float edge, float dye, const float vel[3],
                         float sigma, uint64_t seed, double out[4]) {
  if (!out || !(radius > 0.0f) || !(edge > 0.0f)) return DOB_EINVAL;
  DISPATCH(s, sphere_soft_grad(c, radius, edge, dye, vel, sigma, seed, out));
  return DOB_OK;
}
int orc_coarse_inverse(int nx, int ny, int nz, double h2, int ref, int method, double* out) {
  if (nx < 1 || ny < 1 || nz < 1 || !out || (size_t)nx * ny * nz > 4096) return DOB_EINVAL;
  Dims c;
  c.nx = nx; c.ny = ny; c.nz = nz;
  const std::vector<double> m = method ? cinv_separable(c, h2, ref) : cinv_direct(c, h2, ref);
  memcpy(out, m.data(), m.size() * sizeof(double));
  return DOB_OK;
}
int orc_get_field64(orc_sim* s, int field, double* host, size_t n) {
  return s->a.f64 ? get_field64(*s->a.sd, field, host, n) : get_field64(*s->a.sf, field, host, n);
}
int orc_set_field64(orc_sim* s, int field, const double* host, size_t n) {
  return s->a.f64 ? set_field64(*s->a.sd, field, host, n) : set_field64(*s->a.sf, field, host, n);
}

int orc_eval_math(int fn, const float* x, const float* y, float* out, uint32_t n) {
  for (uint32_t i = 0; i < n; ++i) {
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
      case 7: r = dob_round_f16(a); break;
      case 8: r = dob_round_bf16(a); break;
      default: return DOB_EINVAL;
    }
    out[i] = r;
  }
  return DOB_OK;
}

}  // extern "C"
