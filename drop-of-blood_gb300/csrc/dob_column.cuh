// dob_column.cuh — z-column addressing of the closed-box stencil kernels
// (k_box.cu).
//
// Block 32 x 8: a warp is 32 consecutive cells of one row and every thread
// walks ZC planes of its (x, y) column.  z-neighbours are kept in registers
// from plane to plane, x-neighbours come from the neighbouring lanes by warp
// shuffles (edge lanes load them), y-neighbours are loads of the adjacent
// rows, which the neighbouring warps of the block bring into L1.  Offsets
// are 32-bit (grids have fewer than 2^31 cells).
#pragma once

#include "dob_device.cuh"

namespace dob {
namespace column_detail {
constexpr unsigned kFull = 0xffffffffu;
}

// Cell of this thread, clamped into the grid (lanes past the last column or
// row compute a copy of the edge cell and store nothing, so every lane takes
// part in the shuffles).
struct Col {
  int lane, x, y, z0, zend;
  bool valid;
  uint32_t sy, sz, i;  // row and plane strides, index of (x, y, z0)
};
template <int ZC>
__device__ __forceinline__ Col column(const Grid& g) {
  Col c;
  c.lane = threadIdx.x;
  const int xr = blockIdx.x * 32 + threadIdx.x, yr = blockIdx.y * 8 + threadIdx.y;
  c.valid = xr < g.nx && yr < g.ny;
  c.x = xr < g.nx ? xr : g.nx - 1;
  c.y = yr < g.ny ? yr : g.ny - 1;
  c.z0 = blockIdx.z * ZC;
  c.zend = min(c.z0 + ZC, g.nz);
  c.sy = (uint32_t)g.nx;
  c.sz = (uint32_t)g.nx * (uint32_t)g.ny;
  c.i = (uint32_t)c.z0 * c.sz + (uint32_t)c.y * c.sy + (uint32_t)c.x;
  return c;
}
// value of cell x - 1 (clamped: x = 0 gives the own value) and x + 1
template <class S>
__device__ __forceinline__ float x_minus(const Col& c, float own, const S* a, uint32_t i) {
  const float sh = __shfl_up_sync(column_detail::kFull, own, 1);
  if (c.x == 0) return own;
  return c.lane == 0 ? ldf(a + i - 1) : sh;
}
template <class S>
__device__ __forceinline__ float x_plus(const Col& c, const Grid& g, float own, const S* a, uint32_t i) {
  const float sh = __shfl_down_sync(column_detail::kFull, own, 1);
  if (c.x == g.nx - 1) return own;
  return c.lane == 31 ? ldf(a + i + 1) : sh;
}
template <class VS>
__device__ __forceinline__ dob_v3 ld3(const VS* u, const VS* v, const VS* w, uint32_t j) {
  return v3(ldf(u + j), ldf(v + j), ldf(w + j));
}

}  // namespace dob
