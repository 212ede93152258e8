// Device helpers shared by the single-cloud and the batched build kernels.
#pragma once

#include "owm_internal.cuh"

namespace owm {

__device__ __forceinline__ uint32_t spread_bits16(uint32_t x) {
  x &= 0x0000ffffu;
  x = (x | (x << 8)) & 0x00ff00ffu;
  x = (x | (x << 4)) & 0x0f0f0f0fu;
  x = (x | (x << 2)) & 0x33333333u;
  x = (x | (x << 1)) & 0x55555555u;
  return x;
}

// Per-leaf reduction state: exact int64-key bounding box, count and the
// (z, id)-minimum with its sorted position.
struct LeafAcc {
  int64_t xmin, xmax, ymin, ymax, zmin;
  uint32_t idmin, posmin, count;
  __device__ __forceinline__ void init() {
    xmin = ymin = 0x7FFFFFFFFFFFFFFFll;
    xmax = ymax = (int64_t)0x8000000000000000ull;
    zmin = 0x7FFFFFFFFFFFFFFFll;
    idmin = 0xFFFFFFFFu;
    posmin = 0xFFFFFFFFu;
    count = 0;
  }
  __device__ __forceinline__ void add(int64_t x, int64_t y, int64_t z, uint32_t id, uint32_t pos) {
    xmin = min(xmin, x);
    xmax = max(xmax, x);
    ymin = min(ymin, y);
    ymax = max(ymax, y);
    if (zid_less(z, id, zmin, idmin)) {
      zmin = z;
      idmin = id;
      posmin = pos;
    }
    ++count;
  }
  // reduce with lanes lane^o for o in [1, width)
  __device__ __forceinline__ void reduce(int width) {
    for (int o = width >> 1; o >= 1; o >>= 1) {
      int64_t a = __shfl_xor_sync(0xffffffffu, xmin, o);
      int64_t b = __shfl_xor_sync(0xffffffffu, xmax, o);
      int64_t c = __shfl_xor_sync(0xffffffffu, ymin, o);
      int64_t d = __shfl_xor_sync(0xffffffffu, ymax, o);
      int64_t z = __shfl_xor_sync(0xffffffffu, zmin, o);
      uint32_t id = __shfl_xor_sync(0xffffffffu, idmin, o);
      uint32_t ps = __shfl_xor_sync(0xffffffffu, posmin, o);
      uint32_t ct = __shfl_xor_sync(0xffffffffu, count, o);
      xmin = min(xmin, a);
      xmax = max(xmax, b);
      ymin = min(ymin, c);
      ymax = max(ymax, d);
      if (zid_less(z, id, zmin, idmin)) {
        zmin = z;
        idmin = id;
        posmin = ps;
      }
      count += ct;
    }
  }
};

__device__ __forceinline__ void write_leaf(Node* nd, const LeafAcc& a, int32_t first, double ox, double oy) {
  Node n;
  n.x0 = __double2float_rd(__dsub_rd(dkey_inv(a.xmin), ox));
  n.y0 = __double2float_rd(__dsub_rd(dkey_inv(a.ymin), oy));
  n.x1 = __double2float_ru(__dsub_ru(dkey_inv(a.xmax), ox));
  n.y1 = __double2float_ru(__dsub_ru(dkey_inv(a.ymax), oy));
  n.zmin = a.zmin;
  n.min_id = a.idmin;
  n.min_pos = a.posmin;
  n.count = a.count;
  n.left = first;
  n.escape = kEnd;
  n.right = -1;
  *nd = n;
}

// Loads one input point as order keys; returns false if a coordinate is not
// finite (the reference's comparisons are undefined there: such input is
// rejected through the context's status word).
__device__ __forceinline__ bool load_point(const double* __restrict__ xyz, uint32_t src, int64_t& x, int64_t& y,
                                           int64_t& z) {
  const double* p = xyz + 3 * (int64_t)src;
  const double dx = __ldg(p), dy = __ldg(p + 1), dz = __ldg(p + 2);
  x = dkey(dx);
  y = dkey(dy);
  z = dkey(dz);
  const uint64_t e = 0x7FF0000000000000ull;
  return ((__double_as_longlong(dx) & e) != e) & ((__double_as_longlong(dy) & e) != e) &
         ((__double_as_longlong(dz) & e) != e);
}


}  // namespace owm
