// Stage-3 cell query by one warp per cell (single clouds and batches).
#pragma once

#include "owm_devutil.cuh"
#include "owm_query.cuh"

namespace owm {

// Stage 3 has threshold 1 and, after the LLP marks, only a few cells left to
// answer (those no LLP falls in), so the per-lane walk (k_query) leaves a handful
// of lanes walking alone, one dependent node load after another.  Here the
// whole warp answers one cell: a shared-memory stack holds the nodes still to
// test, and each round the warp pops up to 32 of them and tests them at once:
//   * outside, or (once some point is known inside) unable to beat the best
//     (z, id): dropped;
//   * strictly inside: its memoised (z, id)-min is a candidate;
//   * partial, but its memoised min point lies strictly inside the cell: that
//     point is the minimum of the subtree's inside points, a candidate;
//   * otherwise a partial internal node pushes its two children and a partial
//     leaf is scanned by the whole warp.
// The result is the (z, id)-minimum of the points strictly inside, or kNone
// when there is none: the same as the per-lane walk with threshold 1.  The
// stack never overflows for a hierarchy of depth <= 63 (each round leaves at
// most 32 entries behind per level); on overflow, or past the round bound, the
// walk sets kStatusWalkBound and stops.

constexpr int kS3Stack = 2304;   // node stack entries per warp (the kernels run 2, 4 or 8 warps per block)

__device__ __forceinline__ int64_t cq_shfl64(int64_t v, int src) { return __shfl_sync(0xffffffffu, v, src); }

// Record r of the points a tree without point arrays was built from, as
// order keys (T.perm set: point p of the sorted order is record T.perm[p]).
__device__ __forceinline__ void cq_record(const TreeView& T, uint32_t r, int64_t& x, int64_t& y, int64_t& z) {
  if (T.rec_stride == 4)
    load_point16<4>(T.rec, r, x, y, z);
  else
    load_point16<3>(T.rec, r, x, y, z);
}
// x, y of a node's min point: sorted position p, id `id` (its record + 1).
template <bool kPerm>
__device__ __forceinline__ void cq_min_point_xy(const TreeView& T, int64_t p, uint32_t id, int64_t& x, int64_t& y) {
  if (kPerm) {  // the id names the record: no permutation read
    int64_t z;
    cq_record(T, id - 1u, x, y, z);
  } else {
    x = __ldg(T.xk + p);
    y = __ldg(T.yk + p);
  }
}

// The whole warp answers the cell with edge tables ex, ey over tree T; st is
// this warp's kS3Stack-entry shared stack.  Returns the result on every lane.
// kPerm: T keeps no point arrays (T.perm is set).
template <bool kPerm>
__device__ __forceinline__ uint32_t cell_min_warp(const TreeView& T, const Edge& ex, const Edge& ey, int32_t* st,
                                                  uint32_t* status, int lane) {
  const uint32_t lt = (1u << lane) - 1u;
  const int32_t first_leaf = T.nleaves - 1;
  int64_t bz = kZSentinel;  // warp-uniform best
  uint32_t bid = 0;
  bool any = false;         // some point strictly inside
  if (lane == 0) st[0] = T.root;
  int top = 1;
  __syncwarp();
  // every node is popped at most once (or the test limit, walk_limit)
  const int64_t round_bound = T.walk_limit > 0 ? (int64_t)T.walk_limit : 2 * (int64_t)T.nleaves + 16;
  for (int64_t round = 0; top > 0; ++round) {
    if (round >= round_bound) {
      if (lane == 0) atomicOr(status, kStatusWalkBound);
      break;
    }
    const int m = top < 32 ? top : 32;
    const int32_t nodei = lane < m ? st[top - m + lane] : kEnd;
    top -= m;
    __syncwarp();  // every lane has read its entry before pushes reuse the slots
    int64_t cz = 0x7FFFFFFFFFFFFFFFll;
    uint32_t cid = 0xFFFFFFFFu;
    bool cand = false, push = false, scan = false;
    int32_t c0 = 0, c1 = 0;
    if (nodei != kEnd) {
      const uint4* np = reinterpret_cast<const uint4*>(T.nodes + nodei);
      const float4 b = __ldg(reinterpret_cast<const float4*>(np));
      const uint4 mw = __ldg(np + 1);
      const uint4 cw = __ldg(np + 2);
      const int64_t nz = (int64_t)(((uint64_t)mw.y << 32) | mw.x);
      const uint32_t nid = mw.z, npos = mw.w;
      const bool outside = b.z <= ex.lo_dn || b.x >= ex.hi_up || b.w <= ey.lo_dn || b.y >= ey.hi_up;
      const bool inside = !outside && b.x > ex.lo_up && b.z < ex.hi_dn && b.y > ey.lo_up && b.w < ey.hi_dn;
      const bool improve = zid_less(nz, nid, bz, bid);
      if (inside) {
        cand = true;
      } else if (!outside && (improve || !any)) {
        int64_t mx, my;
        cq_min_point_xy<kPerm>(T, npos, nid, mx, my);
        if (mx > ex.lo_k && mx < ex.hi_k && my > ey.lo_k && my < ey.hi_k) {
          cand = true;
        } else if (nodei >= first_leaf) {
          scan = true;
        } else {
          push = true;
          c0 = (int32_t)cw.y;  // left
          c1 = (int32_t)cw.w;  // right
        }
      }
      if (cand) {
        cz = nz;
        cid = nid;
      }
    }
    // candidates of this round
    if (__any_sync(0xffffffffu, cand)) {
      any = true;
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) {
        const int64_t z2 = cq_shfl64(cz, lane ^ o);
        const uint32_t i2 = __shfl_xor_sync(0xffffffffu, cid, o);
        if (zid_less(z2, i2, cz, cid)) {
          cz = z2;
          cid = i2;
        }
      }
      if (zid_less(cz, cid, bz, bid)) {
        bz = cz;
        bid = cid;
      }
    }
    // partial leaves, one at a time by the whole warp
    uint32_t want = __ballot_sync(0xffffffffu, scan);
    while (want) {
      const int src = __ffs(want) - 1;
      want &= want - 1;
      const int32_t leafi = __shfl_sync(0xffffffffu, nodei, src);
      const Node* lp = T.nodes + leafi;
      const int32_t first = __ldg(&lp->left);
      const uint32_t c = __ldg(&lp->count);
      int64_t mz = 0x7FFFFFFFFFFFFFFFll;
      uint32_t mid = 0xFFFFFFFFu;
      bool seen = false;
      // kU * 32 points per chunk, every load issued before any test: one
      // memory latency per chunk (with kPerm two, the permutation entries
      // first; 256 points a chunk, so a leaf of up to 256 points takes one)
      constexpr int kU = kPerm ? 8 : 4;
      for (uint32_t o = 0; o < c; o += 32 * kU) {
        int64_t x[kU], y[kU], z[kU];
        uint32_t id[kU];
        if (kPerm) {
          uint32_t src[kU];
#pragma unroll
          for (int u = 0; u < kU; ++u) {
            const uint32_t k = o + u * 32 + lane;
            src[u] = k < c ? __ldg(T.perm + (int64_t)first + k) : 0xFFFFFFFFu;  // positions < 2^31
          }
#pragma unroll
          for (int u = 0; u < kU; ++u) {
            if (src[u] != 0xFFFFFFFFu) {
              cq_record(T, src[u], x[u], y[u], z[u]);
              id[u] = src[u] + 1u;
            } else {
              x[u] = ex.lo_k;  // fails the strict test
              y[u] = z[u] = 0;
              id[u] = 0;
            }
          }
        } else {
#pragma unroll
          for (int u = 0; u < kU; ++u) {
            const uint32_t k = o + u * 32 + lane;
            if (k < c) {
              const int64_t q = (int64_t)first + k;
              x[u] = __ldg(T.xk + q);
              y[u] = __ldg(T.yk + q);
              z[u] = __ldg(T.zk + q);
              id[u] = __ldg(T.pid + q);
            } else {
              x[u] = ex.lo_k;  // fails the strict test
              y[u] = z[u] = 0;
              id[u] = 0;
            }
          }
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          if (x[u] > ex.lo_k && x[u] < ex.hi_k && y[u] > ey.lo_k && y[u] < ey.hi_k) {
            seen = true;
            if (zid_less(z[u], id[u], mz, mid)) {
              mz = z[u];
              mid = id[u];
            }
          }
        }
      }
      if (__any_sync(0xffffffffu, seen)) {
        any = true;
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) {
          const int64_t z2 = cq_shfl64(mz, lane ^ o);
          const uint32_t i2 = __shfl_xor_sync(0xffffffffu, mid, o);
          if (zid_less(z2, i2, mz, mid)) {
            mz = z2;
            mid = i2;
          }
        }
        if (zid_less(mz, mid, bz, bid)) {
          bz = mz;
          bid = mid;
        }
      }
    }
    // children of partial internal nodes
    const uint32_t pm = __ballot_sync(0xffffffffu, push);
    const int npush = 2 * __popc(pm);
    if (top + npush > kS3Stack) {
      if (lane == 0) atomicOr(status, kStatusWalkBound);
      break;
    }
    if (push) {
      const int at = top + 2 * __popc(pm & lt);
      st[at] = c1;
      st[at + 1] = c0;
    }
    top += npush;
    __syncwarp();
  }
  return any ? bid : kNone;
}

}  // namespace owm
