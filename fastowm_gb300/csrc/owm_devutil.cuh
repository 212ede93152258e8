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
  // Reduces over aligned segments of `width` lanes (a power of two <= 32);
  // every lane of the warp calls this, and every lane of a segment ends with
  // the segment's result.  Uses the warp reduction unit (redux.sync, 32-bit)
  // instead of a shuffle tree: a 64-bit min/max is the high words' signed
  // min/max, then the low words' unsigned min/max over the lanes whose high
  // word won.  (z, id) stays lexicographic: min z, then min id among the
  // lanes holding it; the winner's sorted position comes from its lane.
  __device__ __forceinline__ void reduce(int width) {
    const int lane = threadIdx.x & 31;
    const uint32_t mask = width >= 32 ? 0xFFFFFFFFu : (((1u << width) - 1u) << (lane & ~(width - 1)));
    xmin = seg_min64(mask, xmin);
    xmax = seg_max64(mask, xmax);
    ymin = seg_min64(mask, ymin);
    ymax = seg_max64(mask, ymax);
    const int64_t zm = seg_min64(mask, zmin);
    const uint32_t im = __reduce_min_sync(mask, zmin == zm ? idmin : 0xFFFFFFFFu);
    const uint32_t win = __ballot_sync(mask, zmin == zm && idmin == im) & mask;
    posmin = __shfl_sync(mask, posmin, __ffs(win) - 1);
    zmin = zm;
    idmin = im;
    count = __reduce_add_sync(mask, count);
  }
  static __device__ __forceinline__ int64_t seg_min64(uint32_t mask, int64_t v) {
    const int32_t hi = (int32_t)(v >> 32);
    const int32_t mh = __reduce_min_sync(mask, hi);
    const uint32_t ml = __reduce_min_sync(mask, hi == mh ? (uint32_t)v : 0xFFFFFFFFu);
    return (int64_t)(((uint64_t)(uint32_t)mh << 32) | ml);
  }
  static __device__ __forceinline__ int64_t seg_max64(uint32_t mask, int64_t v) {
    const int32_t hi = (int32_t)(v >> 32);
    const int32_t mh = __reduce_max_sync(mask, hi);
    const uint32_t ml = __reduce_max_sync(mask, hi == mh ? (uint32_t)v : 0u);
    return (int64_t)(((uint64_t)(uint32_t)mh << 32) | ml);
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

// Segment-cooperative form: every lane of an aligned segment of `width` lanes
// (a power of two) calls this with the segment's reduced accumulator, and the
// segment's first lane stores the node when `store`.  The four FP64 box
// roundings run on four lanes at once -- FP64 issue is scarce on GB300 --
// all as round-down: the upper bounds use ru(v - o) = -rd(o - v), which gives
// the same bits as write_leaf.
__device__ __forceinline__ void write_leaf_seg(Node* nd, const LeafAcc& a, int32_t first, double ox, double oy,
                                               int width, bool store) {
  const int lane = threadIdx.x & 31;
  const int base = lane & ~(width - 1);
  if (width < 4) {
    if (store && lane == base) write_leaf(nd, a, first, ox, oy);
    return;
  }
  const uint32_t mask = width >= 32 ? 0xFFFFFFFFu : (((1u << width) - 1u) << base);
  const int c = lane - base;  // lanes c = 0..3 of the segment: x0, y0, x1, y1
  const double p = c == 0 ? dkey_inv(a.xmin) : c == 1 ? dkey_inv(a.ymin) : c == 2 ? ox : oy;
  const double q = c == 0 ? ox : c == 1 ? oy : c == 2 ? dkey_inv(a.xmax) : dkey_inv(a.ymax);
  float v = __double2float_rd(__dsub_rd(p, q));
  if (c >= 2) v = 0.0f - v;  // exact; 0 - (+0) keeps +0
  const float x0 = __shfl_sync(mask, v, base), y0 = __shfl_sync(mask, v, base + 1);
  const float x1 = __shfl_sync(mask, v, base + 2), y1 = __shfl_sync(mask, v, base + 3);
  if (store && lane == base) {
    Node n;
    n.x0 = x0;
    n.y0 = y0;
    n.x1 = x1;
    n.y1 = y1;
    n.zmin = a.zmin;
    n.min_id = a.idmin;
    n.min_pos = a.posmin;
    n.count = a.count;
    n.left = first;
    n.escape = kEnd;
    n.right = -1;
    *nd = n;
  }
}

// Read-only 16-byte load whose L2 miss asks for 64 bytes (the prefetch-size
// hint), for gathers of random points.
__device__ __forceinline__ double2 ldg_l2_64(const double2* p) {
  double2 r;
  asm("ld.global.nc.L2::64B.v2.f64 {%0, %1}, [%2];" : "=d"(r.x), "=d"(r.y) : "l"(p));
  return r;
}

// load_point with wide aligned reads instead of three 8-byte ones, for AoS
// records of kStride doubles.  kStride 4 (a cloud's 32-byte records, x, y, z,
// pad): the point is one aligned 32-byte sector, read at once.  kStride 3 (plain
// 24-byte points): the point lies in the 32 bytes from the 16-byte boundary at
// or below x, which straddle two sectors for half the points; needs kXyzSlack
// readable bytes after the last point.  xyz 16-byte aligned (32 for kStride 4).
// Both take the 64-byte hint: without it a random miss fetched more (123
// instead of 67 bytes read per point, 32-byte records, 24 M points).
template <int kStride>
__device__ __forceinline__ bool load_point16(const double* __restrict__ xyz, uint32_t src, int64_t& x, int64_t& y,
                                             int64_t& z) {
  static_assert(kStride == 3 || kStride == 4, "records of 3 or 4 doubles");
  double dx, dy, dz;
  if (kStride == 4) {
    // one 32-byte load; it bypasses L1, which then keeps the tables that the
    // callers look up per point (1.2% off the build gather at 100 M points)
    asm("ld.global.nc.L1::no_allocate.L2::64B.v4.f64 {%0, %1, %2, _}, [%3];"
        : "=d"(dx), "=d"(dy), "=d"(dz)
        : "l"(xyz + 4 * (int64_t)src));
  } else {
    const int64_t e = 3 * (int64_t)src;
    const int odd = (int)(e & 1);
    const double2* w = reinterpret_cast<const double2*>(xyz + (e - odd));
    const double2 a = ldg_l2_64(w), b = ldg_l2_64(w + 1);
    dx = odd ? a.y : a.x;
    dy = odd ? b.x : a.y;
    dz = odd ? b.y : b.x;
  }
  x = dkey(dx);
  y = dkey(dy);
  z = dkey(dz);
  const uint64_t m = 0x7FF0000000000000ull;
  return ((__double_as_longlong(dx) & m) != m) & ((__double_as_longlong(dy) & m) != m) &
         ((__double_as_longlong(dz) & m) != m);
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
