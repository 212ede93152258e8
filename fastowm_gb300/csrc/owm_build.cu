// Spatial index build on the device: the GB300 replacement of the reference's
// parallel_qtree + storeMinAndNumPoints (CPP-TBB-CPU/src/optim3_func.cpp:
// 220-307).
//
//   k_morton          quantise (x, y) on the square root domain, interleave
//                     (2D Morton / quadtree order), one key of 16-24 bits per
//                     point (choose_key_bits)
//   radix_sort        stable LSD sort of (key, input position)
//   k_gather_leaves   permute the points into sorted order as exact
//                     order-preserving int64 keys + 1-based id, and reduce each
//                     leaf of L points (count, outward float box, (z,id)-min)
//                     with warp shuffles -- one pass over the points
//   k_leaf_starts /   leaves = quadtree cells of half-side <= min_radius
//   k_leaf_reduce     (min-radius policy) or any other leaf partition
//   k_leaf_keys       the key of every leaf's first point, packed
//   k_karras          binary radix hierarchy over the leaves (Karras 2012) on
//                     64-bit (leaf Morton key, leaf index) codes
//   k_refit           bottom-up atomic refit: internal count, box and
//                     (z, id)-min -- the reference's O3 memo (storeMinAndNumPoints)
//                     -- and the depth-first "escape" link of every node, so
//                     that queries walk the tree without a stack
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "owm_build.cuh"
#include "owm_classes.cuh"
#include "owm_devutil.cuh"

namespace owm {

namespace {

// Quadtree order key: x bit above y bit at each level, like the
// reference's quadrant index (x >= cx) << 1 | (y >= cy) (optim3_func.cpp:92-100).
// Integer form: when the domain's ends share sign and exponent, the order key
// of a double is linear in its value over the domain, so the cell index is
// (key(v) - key(lo)) >> shift -- no FP64 arithmetic at all.
template <int kStride>
__global__ void k_morton_int(const double* __restrict__ xyz, int64_t n, int64_t kx0, int64_t ky0, int shx, int shy,
                             int bits, uint32_t* __restrict__ keys) {
  const int64_t qmax = (1ll << bits) - 1;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t qx = (dkey(__ldg(xyz + kStride * i)) - kx0) >> shx;
    int64_t qy = (dkey(__ldg(xyz + kStride * i + 1)) - ky0) >> shy;
    qx = qx < 0 ? 0 : (qx > qmax ? qmax : qx);
    qy = qy < 0 ? 0 : (qy > qmax ? qmax : qy);
    keys[i] = (spread_bits16((uint32_t)qx) << 1) | spread_bits16((uint32_t)qy);
  }
}

// General form (domain spans exponents): scaled FP64 offsets.
template <int kStride>
__global__ void k_morton(const double* __restrict__ xyz, int64_t n, double ox, double oy, double scale,
                         int bits, uint32_t* __restrict__ keys) {
  const float qmax = (float)((1u << bits) - 1u);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double x = __ldg(xyz + kStride * i), y = __ldg(xyz + kStride * i + 1);
    float fx = (float)((x - ox) * scale), fy = (float)((y - oy) * scale);
    fx = fminf(fmaxf(fx, 0.0f), qmax);
    fy = fminf(fmaxf(fy, 0.0f), qmax);
    keys[i] = (spread_bits16((uint32_t)fx) << 1) | spread_bits16((uint32_t)fy);
  }
}

// Morton key of one point, integer form (k_morton_int) and FP64 form
// (k_morton), for the counting variant below.
// x and y of a point at p: one 16-byte load from a compact x, y array
// (stride 2), two 8-byte loads from plain points.
template <int kStride>
__device__ __forceinline__ double2 load_xy(const double* __restrict__ p) {
  if (kStride == 2) return __ldg(reinterpret_cast<const double2*>(p));
  return make_double2(__ldg(p), __ldg(p + 1));
}

struct MortonIntKey {
  int64_t kx0, ky0, qmax;
  int shx, shy;
  __device__ __forceinline__ uint32_t operator()(double2 v) const {
    int64_t qx = (dkey(v.x) - kx0) >> shx;
    int64_t qy = (dkey(v.y) - ky0) >> shy;
    qx = qx < 0 ? 0 : (qx > qmax ? qmax : qx);
    qy = qy < 0 ? 0 : (qy > qmax ? qmax : qy);
    return (spread_bits16((uint32_t)qx) << 1) | spread_bits16((uint32_t)qy);
  }
};
struct MortonFpKey {
  double ox, oy, scale;
  float qmax;
  __device__ __forceinline__ uint32_t operator()(double2 v) const {
    float fx = (float)((v.x - ox) * scale), fy = (float)((v.y - oy) * scale);
    fx = fminf(fmaxf(fx, 0.0f), qmax);
    fy = fminf(fmaxf(fy, 0.0f), qmax);
    return (spread_bits16((uint32_t)fx) << 1) | spread_bits16((uint32_t)fy);
  }
};

// Morton keys of part blockIdx.x of a large sort (sort_part_range), with the
// part's counts of the sort's first digit (key & dmask0) into
// counts[d * gridDim.x + blockIdx.x]: the first radix pass then needs no
// separate read of the keys.
template <class KeyOf, int kStride>
__global__ void __launch_bounds__(256) k_morton_counts(const double* __restrict__ xyz, int64_t n, KeyOf key_of,
                                                       int64_t ntiles, uint32_t dmask0, uint32_t* __restrict__ keys,
                                                       uint32_t* __restrict__ counts) {
  __shared__ uint32_t h[8][256];
  for (int i = threadIdx.x; i < 8 * 256; i += 256) (&h[0][0])[i] = 0;
  __syncthreads();
  int64_t b, e;
  sort_part_range(n, ntiles, gridDim.x, blockIdx.x, &b, &e);
  uint32_t* hw = h[threadIdx.x >> 5];
  int64_t i = b + threadIdx.x;
  for (; i + 3 * 256 < e; i += 4 * 256) {  // four points in flight per thread
    uint32_t k[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) k[u] = key_of(load_xy<kStride>(xyz + kStride * (i + u * 256)));
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      keys[i + u * 256] = k[u];
      atomicAdd(hw + (k[u] & dmask0), 1u);
    }
  }
  for (; i < e; i += 256) {
    const uint32_t k = key_of(load_xy<kStride>(xyz + kStride * i));
    keys[i] = k;
    atomicAdd(hw + (k & dmask0), 1u);
  }
  __syncthreads();
  {
    const int d = threadIdx.x;
    uint32_t s = 0;
#pragma unroll
    for (int w = 0; w < 8; ++w) s += h[w][d];
    counts[(int64_t)d * gridDim.x + blockIdx.x] = s;
  }
}

// One warp per unit of max(L, 32) sorted positions.  L in {1,2,4,...,256}.
// Without kCls the sorted points go to the SoA arrays xk, yk, zk, pid.  With
// kCls (the whole-path run, whose only later reader of points is stage 3's
// cell walk, which then reads them through the permutation) nothing is
// stored: 28 bytes a point less to write (100 M points: 2.53 -> 2.39 ms).
// With kCls, every chunk of 32 gathered points is also folded into the
// stage-1 window classes while the point is in registers (about 0.45 ms of
// the kernel's 2.5 ms at 100 M points, nearly all of it the sub-cell lookups
// and the warp votes; the atomics take about 0.07 ms).
// At most 40 registers a thread (a few bytes spill): 3 blocks of 512 (48
// warps) per SM instead of 2 at the 63 registers the compiler would take; the
// kernel waits on random DRAM reads, and the extra resident warps keep more of
// them in flight (100 M points: 2.84 -> 2.55 ms; 48 registers 2.69, 36 and 32
// registers 2.63).  Launched with at most 512 threads.
template <int L, bool kCls, int kStride>
__global__ void __maxnreg__(40) k_gather_leaves(const double* __restrict__ xyz, const uint32_t* __restrict__ perm,
                                                       int64_t n, int32_t nleaves, double ox, double oy,
                                                       int64_t* __restrict__ xk, int64_t* __restrict__ yk,
                                                       int64_t* __restrict__ zk, uint32_t* __restrict__ pid,
                                                       Node* __restrict__ leaves, uint32_t* __restrict__ status,
                                                       ClassArgs A) {
  constexpr int kUnit = L < 32 ? 32 : L;
  constexpr int kSeg = L < 32 ? L : 32;
  bool finite = true;
  const int lane = threadIdx.x & 31;
  const int64_t nunits = (n + kUnit - 1) / kUnit;
  for (int64_t u = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < nunits;
       u += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    LeafAcc acc;
    acc.init();
    // the next chunk's permutation entry is in flight while a chunk is folded
    uint32_t s_nxt = u * kUnit + lane < n ? __ldg(perm + u * kUnit + lane) : 0u;
#pragma unroll
    for (int c = 0; c < kUnit; c += 32) {
      int64_t pos = u * kUnit + c + lane;
      const bool valid = pos < n;
      int64_t x = 0, y = 0, z = 0;
      const uint32_t src = s_nxt;
      if (c + 32 < kUnit) s_nxt = pos + 32 < n ? __ldg(perm + pos + 32) : 0u;
      if (valid) {
        finite &= load_point16<kStride>(xyz, src, x, y, z);
        if (!kCls) {
          xk[pos] = x;
          yk[pos] = y;
          zk[pos] = z;
          pid[pos] = src + 1;
        }
        acc.add(x, y, z, src + 1, (uint32_t)pos);
      }
      if (kCls) {
        if (!__all_sync(0xffffffffu, valid)) {  // ragged tail: idle lanes borrow lane 0's point
          const int64_t bx = __shfl_sync(0xffffffffu, x, 0), by = __shfl_sync(0xffffffffu, y, 0);
          if (!valid) {
            x = bx;
            y = by;
            z = 0;
          }
        }
        cls_aggregate_warp(A, valid, x, y, z, src + 1, lane);
      }
    }
    acc.reduce(kSeg);
    {
      const int64_t first = u * kUnit + (lane & ~(kSeg - 1));  // L < 32: segment start; else lane 0's
      write_leaf_seg(leaves + (first < n ? first / L : 0), acc, (int32_t)first, ox, oy, kSeg, first < n);
    }
  }
  if (!finite) atomicOr(status, 1u);
}

template <int kStride>
__global__ void k_gather(const double* __restrict__ xyz, const uint32_t* __restrict__ perm, int64_t n,
                         int64_t* __restrict__ xk, int64_t* __restrict__ yk, int64_t* __restrict__ zk,
                         uint32_t* __restrict__ pid, uint32_t* __restrict__ status) {
  bool finite = true;
  for (int64_t pos = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; pos < n;
       pos += (int64_t)gridDim.x * blockDim.x) {
    uint32_t src = __ldg(perm + pos);
    int64_t x, y, z;
    finite &= load_point16<kStride>(xyz, src, x, y, z);
    xk[pos] = x;
    yk[pos] = y;
    zk[pos] = z;
    pid[pos] = src + 1;
  }
  if (!finite) atomicOr(status, 1u);
}

// flag[pos] = 1 where a new leaf starts: the quadtree cell (key >> cell_shift)
// changes, or the current run reached max_leaf points from its cell start.
__global__ void k_leaf_flags(const uint32_t* __restrict__ keys, int64_t n, int cell_shift,
                             uint32_t* __restrict__ flags) {
  for (int64_t pos = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; pos < n;
       pos += (int64_t)gridDim.x * blockDim.x) {
    uint32_t f = 1;
    if (pos > 0) {
      uint32_t a = cell_shift >= 32 ? 0u : keys[pos] >> cell_shift;
      uint32_t b = cell_shift >= 32 ? 0u : keys[pos - 1] >> cell_shift;
      f = a != b;
    }
    flags[pos] = f;
  }
}

__global__ void k_leaf_starts(const uint32_t* __restrict__ flags, const uint32_t* __restrict__ scan, int64_t n,
                              int32_t* __restrict__ starts) {
  for (int64_t pos = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; pos < n;
       pos += (int64_t)gridDim.x * blockDim.x) {
    if (flags[pos]) starts[scan[pos]] = (int32_t)pos;
  }
}

// One warp per leaf of any size; starts has nleaves+1 entries (last = n).
__global__ void k_leaf_reduce(const int64_t* __restrict__ xk, const int64_t* __restrict__ yk,
                              const int64_t* __restrict__ zk, const uint32_t* __restrict__ pid,
                              const int32_t* __restrict__ starts, int32_t nleaves, double ox, double oy,
                              Node* __restrict__ leaves) {
  const int lane = threadIdx.x & 31;
  for (int64_t li = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; li < nleaves;
       li += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    int32_t b = starts[li], e = starts[li + 1];
    LeafAcc acc;
    acc.init();
    for (int32_t p = b + lane; p < e; p += 32) acc.add(xk[p], yk[p], zk[p], pid[p], (uint32_t)p);
    acc.reduce(32);
    write_leaf_seg(leaves + li, acc, b, ox, oy, 32, true);
  }
}

__device__ __forceinline__ int32_t leaf_first(int32_t li, int32_t L, const int32_t* starts) {
  return starts ? starts[li] : li * L;
}

__device__ __forceinline__ int delta(const uint32_t* __restrict__ mk, int32_t L, const int32_t* __restrict__ starts,
                                     int32_t nl, int32_t i, int32_t j) {
  if (j < 0 || j >= nl) return -1;
  uint64_t a = ((uint64_t)__ldg(mk + leaf_first(i, L, starts)) << 32) | (uint32_t)i;
  uint64_t b = ((uint64_t)__ldg(mk + leaf_first(j, L, starts)) << 32) | (uint32_t)j;
  return __clzll((long long)(a ^ b));
}

// Key of every leaf's first point, packed (the hierarchy's binary searches
// then share cache lines instead of reading one sector per key).
__global__ void k_leaf_keys(const uint32_t* __restrict__ mk, int32_t L, const int32_t* __restrict__ starts,
                            int32_t nl, uint32_t* __restrict__ lk) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nl) lk[i] = __ldg(mk + leaf_first(i, L, starts));
}

// Karras (2012), Sec. 4: internal node i covers leaves [min(i,j), max(i,j)]
// and splits after gamma.  Internal nodes are 0..nl-2, leaf li is nl-1+li.
// Also readies k_refit: the root's parent is -1 and every internal node's
// arrival counter starts at 0.
__global__ void k_karras(const uint32_t* __restrict__ mk, int32_t L, const int32_t* __restrict__ starts, int32_t nl,
                         Node* __restrict__ nodes, int32_t* __restrict__ parent, int32_t* __restrict__ right_of,
                         int32_t* __restrict__ last_of, int32_t* __restrict__ flags) {
  int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nl - 1) return;
  flags[i] = 0;
  if (i == 0) parent[0] = -1;  // no node has the root as a child
  int d = delta(mk, L, starts, nl, i, i + 1) - delta(mk, L, starts, nl, i, i - 1) > 0 ? 1 : -1;
  int dmin = delta(mk, L, starts, nl, i, i - d);
  int32_t lmax = 2;
  while (delta(mk, L, starts, nl, i, i + lmax * d) > dmin) lmax <<= 1;
  int32_t l = 0;
  for (int32_t t = lmax >> 1; t >= 1; t >>= 1)
    if (delta(mk, L, starts, nl, i, i + (l + t) * d) > dmin) l += t;
  int32_t j = i + l * d;
  int dnode = delta(mk, L, starts, nl, i, j);
  int32_t s = 0;
  for (int32_t div = 2;; div <<= 1) {
    int32_t t = (l + div - 1) / div;
    if (delta(mk, L, starts, nl, i, i + (s + t) * d) > dnode) s += t;
    if (t <= 1) break;
  }
  int32_t gamma = i + s * d + (d < 0 ? -1 : 0);
  int32_t lo = min(i, j), hi = max(i, j);
  int32_t left = (lo == gamma) ? (nl - 1 + gamma) : gamma;
  int32_t right = (hi == gamma + 1) ? (nl - 1 + gamma + 1) : gamma + 1;
  nodes[i].left = left;
  nodes[i].right = right;
  parent[left] = i;
  parent[right] = i;
  right_of[gamma] = right;
  last_of[i] = hi;
}

// escape(node covering leaves [a, b]) = right child of the split after b
// (the unique internal node whose left subtree ends at b), or end.
__device__ __forceinline__ int32_t escape_of(int32_t last, const int32_t* __restrict__ right_of, int32_t nl) {
  return last >= nl - 1 ? kEnd : __ldg(right_of + last);
}

__device__ __forceinline__ void load_summary(const Node* p, float4& box, int64_t& z, uint32_t& id, uint32_t& pos,
                                             uint32_t& cnt) {
  // L2 loads: the sibling's summary was written by another thread of this grid
  box = __ldcg(reinterpret_cast<const float4*>(p));
  z = __ldcg(&p->zmin);
  id = __ldcg(&p->min_id);
  pos = __ldcg(&p->min_pos);
  cnt = __ldcg(&p->count);
}

// Bottom-up refit; every node also gets its escape link here (the thread
// that starts at a leaf, and the second arrival at an internal node).
__device__ __forceinline__ int32_t arrive_acq_rel(int32_t* f) {
  int32_t old;
  asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], 1;" : "=r"(old) : "l"(f) : "memory");
  return old;
}

__global__ void k_refit(Node* __restrict__ nodes, const int32_t* __restrict__ parent, int32_t* __restrict__ flags,
                        const int32_t* __restrict__ right_of, const int32_t* __restrict__ last_of, int32_t nl) {
  int32_t li = blockIdx.x * blockDim.x + threadIdx.x;
  if (li >= nl) return;
  nodes[nl - 1 + li].escape = escape_of(li, right_of, nl);
  int32_t n = parent[nl - 1 + li];
  // a root path has at most nl-1 internal nodes; the bound guards corruption
  for (int32_t guard = 0; n >= 0 && guard < nl; ++guard) {
    // acquire-release arrival: the first arriver's summary stores are
    // released by its increment and acquired by the second arriver's, which
    // then reads both children from L2
    if (arrive_acq_rel(flags + n) == 0) return;  // sibling not done yet
    const Node* a = nodes + __ldcg(&nodes[n].left);
    const Node* b = nodes + __ldcg(&nodes[n].right);
    float4 ba, bb;
    int64_t za, zb;
    uint32_t ia, ib, pa, pb, ca, cb;
    load_summary(a, ba, za, ia, pa, ca);
    load_summary(b, bb, zb, ib, pb, cb);
    Node* o = nodes + n;
    float4 box = make_float4(fminf(ba.x, bb.x), fminf(ba.y, bb.y), fmaxf(ba.z, bb.z), fmaxf(ba.w, bb.w));
    __stcg(reinterpret_cast<float4*>(o), box);
    bool bl = zid_less(zb, ib, za, ia);
    __stcg(&o->zmin, bl ? zb : za);
    __stcg(&o->min_id, bl ? ib : ia);
    __stcg(&o->min_pos, bl ? pb : pa);
    __stcg(&o->count, ca + cb);
    o->escape = escape_of(__ldg(last_of + n), right_of, nl);
    n = parent[n];
  }
}

// Sum of children == count for every internal node (checkNumPoints).
__global__ void k_check_counts(const Node* __restrict__ nodes, int32_t nl, int32_t* __restrict__ bad) {
  int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nl - 1) return;
  const Node& n = nodes[i];
  const Node& a = nodes[n.left];
  const Node& b = nodes[n.right];
  bool ok = n.count == a.count + b.count;
  bool zok = !zid_less(a.zmin, a.min_id, n.zmin, n.min_id) && !zid_less(b.zmin, b.min_id, n.zmin, n.min_id);
  bool box_ok = n.x0 <= a.x0 && n.x0 <= b.x0 && n.y0 <= a.y0 && n.y0 <= b.y0 && n.x1 >= a.x1 && n.x1 >= b.x1 &&
                n.y1 >= a.y1 && n.y1 >= b.y1;
  if (!(ok && zok && box_ok)) atomicAdd(bad, 1);
}

int grid_for(int64_t n, int block) {
  int64_t g = (n + block - 1) / block;
  if (g > 152 * 32) g = 152 * 32;
  if (g < 1) g = 1;
  return (int)g;
}

template <int L, int kStride>
void launch_gather_leaves(const double* xyz, const uint32_t* perm, int64_t n, int32_t nl, double ox, double oy,
                          TreeStore* t, uint32_t* status, cudaStream_t s, const ClassArgs* cls) {
  constexpr int kUnit = L < 32 ? 32 : L;
  int64_t nunits = (n + kUnit - 1) / kUnit;
  int64_t warps = nunits;
  const int gb = t->gather_block;  // 128, 256 or 512 threads
  int64_t blocks = (warps * 32 + gb - 1) / gb;
  // one warp per unit (no grid-stride reuse): the resident warps then work on
  // neighbouring units, which measured 12-15% faster than 16 blocks per SM
  if (blocks > (int64_t)152 * 1024 * 256 / gb) blocks = (int64_t)152 * 1024 * 256 / gb;
  if (cls) {
    OWM_LAUNCH("k_gather_leaves", s, k_gather_leaves<L, true, kStride><<<(unsigned)blocks, gb, 0, s>>>(
        xyz, perm, n, nl, ox, oy, t->xk, t->yk, t->zk, t->pid, t->nodes + (nl - 1), status, *cls));
  } else {
    ClassArgs none;
    std::memset(&none, 0, sizeof(none));
    OWM_LAUNCH("k_gather_leaves", s, k_gather_leaves<L, false, kStride><<<(unsigned)blocks, gb, 0, s>>>(
        xyz, perm, n, nl, ox, oy, t->xk, t->yk, t->zk, t->pid, t->nodes + (nl - 1), status, none));
  }
}

template <int kStride>
int gather_leaves_for(int32_t L, const double* xyz, const uint32_t* perm, int64_t n, int32_t nl, double ox, double oy,
                      TreeStore* t, uint32_t* status, cudaStream_t s, const ClassArgs* cls) {
  switch (L) {
    case 1: launch_gather_leaves<1, kStride>(xyz, perm, n, nl, ox, oy, t, status, s, cls); break;
    case 2: launch_gather_leaves<2, kStride>(xyz, perm, n, nl, ox, oy, t, status, s, cls); break;
    case 4: launch_gather_leaves<4, kStride>(xyz, perm, n, nl, ox, oy, t, status, s, cls); break;
    case 8: launch_gather_leaves<8, kStride>(xyz, perm, n, nl, ox, oy, t, status, s, cls); break;
    case 16: launch_gather_leaves<16, kStride>(xyz, perm, n, nl, ox, oy, t, status, s, cls); break;
    case 32: launch_gather_leaves<32, kStride>(xyz, perm, n, nl, ox, oy, t, status, s, cls); break;
    case 64: launch_gather_leaves<64, kStride>(xyz, perm, n, nl, ox, oy, t, status, s, cls); break;
    case 128: launch_gather_leaves<128, kStride>(xyz, perm, n, nl, ox, oy, t, status, s, cls); break;
    case 256: launch_gather_leaves<256, kStride>(xyz, perm, n, nl, ox, oy, t, status, s, cls); break;
    default:
      return OWM_EINVAL;  // unreachable: leaf_size() gives powers of two up to 256
  }
  return OWM_OK;
}

}  // namespace

bool morton_int_shifts(double lo, double hi, int bits, int64_t* klo, int* shift) {
  int64_t a = dkey(lo), b = dkey(hi);
  int64_t ba, bb;
  std::memcpy(&ba, &lo, 8);
  std::memcpy(&bb, &hi, 8);
  // same sign and same exponent field: keys are linear in the value
  if ((ba >> 52) != (bb >> 52) || lo <= 0.0) return false;
  uint64_t span = (uint64_t)(b - a);
  int len = 0;
  while (len < 64 && (span >> len) != 0) ++len;
  *klo = a;
  *shift = len > bits ? len - bits : 0;
  return true;
}

int choose_key_bits(int64_t n, int policy, double side, float min_radius, int32_t leaf) {
  int b;
  if (policy == OWM_TREE_MIN_RADIUS && min_radius > 0.0f) {
    b = n <= (1 << 18) ? 8 : 12;
    // quadtree depth where half-side <= 2*min_radius (insertPoint's split
    // rule, optim3_func.cpp:107: split while radius*0.5 > minRadius)
    double r = side * 0.5;
    int d = 0;
    while (r * 0.5 > (double)min_radius && d < 16) {
      r *= 0.5;
      ++d;
    }
    if (d > b) b = d <= 12 ? 12 : 16;
  } else {
    // Leaves are runs of `leaf` points in key order.  The fewest bits per
    // axis (8..12) that leave at most half a leaf of points per finest cell
    // of an evenly spread cloud keep every leaf compact; fewer key bits make
    // the last sort digit narrower (20 bits: 8 + 8 + 4).
    const int64_t per_cell = std::max<int32_t>(leaf / 2, 1);
    b = 8;
    while (b < 12 && n > per_cell * ((int64_t)1 << (2 * b))) ++b;
  }
  return 2 * b;
}

size_t tree_scratch_bytes(int64_t n) {
  size_t a = 0;
  auto add = [&](size_t bytes) { a += (bytes + 255) & ~(size_t)255; };
  add((size_t)n * 4);  // keys0
  add((size_t)n * 4);  // keys1
  add((size_t)n * 4);  // vals0
  add((size_t)n * 4);  // vals1
  add(radix_sort_temp_bytes(n));
  add((size_t)(n + 1) * 4);  // leaf starts
  add((size_t)(2 * n + 2) * 4);  // parent
  add((size_t)(n + 1) * 4);      // flags / right_of
  add((size_t)(n + 1) * 4);      // right_of
  add((size_t)(n + 1) * 4);      // last_of
  add(scan_temp_bytes(n) + 64);
  return a + 1024;
}

int build_tree(const PointsView& pts, int64_t n, const owm_bbox& bb, const owm_tree_cfg& cfg, TreeStore* t,
               void* scratch, size_t scratch_bytes, uint32_t* status, cudaStream_t s, int64_t* launches,
               const ClassArgs* cls, bool* fused, cudaEvent_t cls_ready, cudaEvent_t gather_done) {
  if (fused) *fused = false;
  t->perm = nullptr;  // set again below when the gather keeps no point arrays
  t->rec = nullptr;
  t->rec_stride = 0;
  const int stride = pts.rec_stride;
  const double* d_xyz = pts.rec;
  if (n <= 0 || n >= 0x7FFFFFFFLL || (stride != 3 && stride != 4) || (pts.xy_stride != 2 && pts.xy_stride != 3))
    return OWM_EINVAL;
  // the gather reads 16-byte words; a 32-byte record is one sector
  if ((reinterpret_cast<uintptr_t>(d_xyz) & (stride == 4 ? 31u : 15u)) != 0) return OWM_EINVAL;
  const double* d_xy = pts.xy;
  const bool xy2 = pts.xy_stride == 2;  // the Morton pass reads x, y from a compact array
  if (scratch_bytes < tree_scratch_bytes(n)) return OWM_ENOMEM;
  char* sp = static_cast<char*>(scratch);
  auto take = [&](size_t bytes) {
    void* p = sp;
    sp += (bytes + 255) & ~(size_t)255;
    return p;
  };
  uint32_t* k0 = (uint32_t*)take((size_t)n * 4);
  uint32_t* k1 = (uint32_t*)take((size_t)n * 4);
  uint32_t* v0 = (uint32_t*)take((size_t)n * 4);
  uint32_t* v1 = (uint32_t*)take((size_t)n * 4);
  size_t sort_bytes = radix_sort_temp_bytes(n);
  void* sort_tmp = take(sort_bytes);
  int32_t* starts = (int32_t*)take((size_t)(n + 1) * 4);
  int32_t* parent = (int32_t*)take((size_t)(2 * n + 2) * 4);
  int32_t* flags = (int32_t*)take((size_t)(n + 1) * 4);
  int32_t* right_of = (int32_t*)take((size_t)(n + 1) * 4);
  int32_t* last_of = (int32_t*)take((size_t)(n + 1) * 4);
  void* scan_tmp = take(scan_temp_bytes(n) + 64);

  // Square root domain like the reference's quadtree (getRadius/getCenter,
  // optim3_func.cpp:6-26): centre of the bbox, half-side = max half-extent.
  double rx = (bb.max_x - bb.min_x) * 0.5, ry = (bb.max_y - bb.min_y) * 0.5;
  double R = rx >= ry ? rx : ry;
  if (!(R > 0.0)) R = 0.5;
  double ox = bb.min_x + rx - R, oy = bb.min_y + ry - R;
  int key_bits = choose_key_bits(n, cfg.policy, 2.0 * R, cfg.min_radius, leaf_size(cfg.max_number));
  int bits_axis = key_bits / 2;
  double scale = (double)(1u << bits_axis) / (2.0 * R);
  t->ox = bb.min_x;  // float boxes are offsets from the bbox corner
  t->oy = bb.min_y;
  t->key_bits = key_bits;
  t->n = n;

  int shx = 0, shy = 0;
  int64_t kx0 = 0, ky0 = 0;
  // large sorts: the Morton pass also counts the first radix digit, in the
  // sort's count-table layout at the start of its temp
  const RadixSortPlan plan = radix_sort_plan(n);
  uint32_t* first_counts = static_cast<uint32_t*>(sort_tmp);
  if (morton_int_shifts(ox, ox + 2.0 * R, bits_axis, &kx0, &shx) &&
      morton_int_shifts(oy, oy + 2.0 * R, bits_axis, &ky0, &shy)) {
    if (plan.parts) {
      const MortonIntKey kf{kx0, ky0, (1ll << bits_axis) - 1, shx, shy};
      const uint32_t dm0 = (1u << radix_digit_bits(key_bits, 0, radix_ranked_widths(n, key_bits))) - 1u;
      if (xy2)
        OWM_LAUNCH("k_morton", s, k_morton_counts<MortonIntKey, 2><<<(unsigned)plan.parts, 256, 0, s>>>(
            d_xy, n, kf, plan.ntiles, dm0, k0, first_counts));
      else
        OWM_LAUNCH("k_morton", s, k_morton_counts<MortonIntKey, 3><<<(unsigned)plan.parts, 256, 0, s>>>(
            d_xy, n, kf, plan.ntiles, dm0, k0, first_counts));
    } else if (xy2) {
      OWM_LAUNCH("k_morton", s, k_morton_int<2><<<grid_for(n, 256), 256, 0, s>>>(d_xy, n, kx0, ky0, shx, shy, bits_axis, k0));
    } else {
      OWM_LAUNCH("k_morton", s, k_morton_int<3><<<grid_for(n, 256), 256, 0, s>>>(d_xy, n, kx0, ky0, shx, shy, bits_axis, k0));
    }
  } else {
    if (plan.parts) {
      const MortonFpKey kf{ox, oy, scale, (float)((1u << bits_axis) - 1u)};
      const uint32_t dm0 = (1u << radix_digit_bits(key_bits, 0, radix_ranked_widths(n, key_bits))) - 1u;
      if (xy2)
        OWM_LAUNCH("k_morton", s, k_morton_counts<MortonFpKey, 2><<<(unsigned)plan.parts, 256, 0, s>>>(
            d_xy, n, kf, plan.ntiles, dm0, k0, first_counts));
      else
        OWM_LAUNCH("k_morton", s, k_morton_counts<MortonFpKey, 3><<<(unsigned)plan.parts, 256, 0, s>>>(
            d_xy, n, kf, plan.ntiles, dm0, k0, first_counts));
    } else if (xy2) {
      OWM_LAUNCH("k_morton", s, k_morton<2><<<grid_for(n, 256), 256, 0, s>>>(d_xy, n, ox, oy, scale, bits_axis, k0));
    } else {
      OWM_LAUNCH("k_morton", s, k_morton<3><<<grid_for(n, 256), 256, 0, s>>>(d_xy, n, ox, oy, scale, bits_axis, k0));
    }
  }
  count_launch(launches);
  bool alt = false;
  OWM_CUDA_TRY(
      radix_sort(k0, v0, k1, v1, n, key_bits, true, sort_tmp, sort_bytes, s, &alt, launches, plan.parts > 0, status));
  const uint32_t* mk = alt ? k1 : k0;
  const uint32_t* perm = alt ? v1 : v0;

  int32_t L = leaf_size(cfg.max_number);
  int32_t nl;
  const int32_t* lstarts = nullptr;
  bool fixed = cfg.policy == OWM_TREE_MAX_NUMBER;
  if (fixed) {
    nl = (int32_t)((n + L - 1) / L);
  } else {
    // min-radius leaves: runs of equal cell key at the leaf depth
    double r = R;
    int d = 0;
    while (r * 0.5 > (double)cfg.min_radius && d < bits_axis) {
      r *= 0.5;
      ++d;
    }
    int cell_shift = 2 * (bits_axis - d);
    uint32_t* fl = reinterpret_cast<uint32_t*>(flags);  // reuse as scratch, [n]
    uint32_t* sc = reinterpret_cast<uint32_t*>(parent);  // [n] + total
    OWM_LAUNCH("k_leaf_flags", s, k_leaf_flags<<<grid_for(n, 256), 256, 0, s>>>(mk, n, cell_shift, fl));
    count_launch(launches);
    OWM_CUDA_TRY(exclusive_scan_u32(fl, sc, n, sc + n, scan_tmp, scan_temp_bytes(n) + 64, s, launches));
    OWM_LAUNCH("k_leaf_starts", s, k_leaf_starts<<<grid_for(n, 256), 256, 0, s>>>(fl, sc, n, starts));
    count_launch(launches);
    uint32_t h_nl = 0;
    OWM_CUDA_TRY(cudaMemcpyAsync(&h_nl, sc + n, 4, cudaMemcpyDeviceToHost, s));
    OWM_CUDA_TRY(cudaStreamSynchronize(s));
    nl = (int32_t)h_nl;
    OWM_CUDA_TRY(cudaMemcpyAsync(starts + nl, &n, 4, cudaMemcpyHostToDevice, s));  // n < 2^31
    OWM_CUDA_TRY(cudaStreamSynchronize(s));
    lstarts = starts;
    L = 0;
  }
  int64_t nnodes = 2 * (int64_t)nl - 1;
  if (t->node_cap < nnodes || t->point_cap < n) return OWM_ENOMEM;
  t->nleaves = nl;
  t->root = 0;

  if (fixed) {
    if (cls && cls_ready) OWM_CUDA_TRY(cudaStreamWaitEvent(s, cls_ready, 0));
    const int grc = stride == 4 ? gather_leaves_for<4>(L, d_xyz, perm, n, nl, t->ox, t->oy, t, status, s, cls)
                                : gather_leaves_for<3>(L, d_xyz, perm, n, nl, t->ox, t->oy, t, status, s, cls);
    if (grc) return grc;
    count_launch(launches);
    if (cls) {  // the class-fold gather keeps no point arrays: points through the permutation
      t->perm = perm;
      t->rec = d_xyz;
      t->rec_stride = stride;
    }
    if (fused && cls) *fused = true;
    if (cls && gather_done) OWM_CUDA_TRY(cudaEventRecord(gather_done, s));
  } else {
    if (stride == 4)
      OWM_LAUNCH("k_gather", s, k_gather<4><<<grid_for(n, 256), 256, 0, s>>>(d_xyz, perm, n, t->xk, t->yk, t->zk, t->pid, status));
    else
      OWM_LAUNCH("k_gather", s, k_gather<3><<<grid_for(n, 256), 256, 0, s>>>(d_xyz, perm, n, t->xk, t->yk, t->zk, t->pid, status));
    count_launch(launches);
    int64_t blocks = ((int64_t)nl * 32 + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    OWM_LAUNCH("k_leaf_reduce", s, k_leaf_reduce<<<(unsigned)blocks, 256, 0, s>>>(t->xk, t->yk, t->zk, t->pid, lstarts, nl, t->ox, t->oy,
                                                    t->nodes + (nl - 1)));
    count_launch(launches);
  }

  if (nl > 1) {
    // the sort's other key buffer is free now: leaf keys there
    uint32_t* lk = alt ? k0 : k1;
    OWM_LAUNCH("k_leaf_keys", s, k_leaf_keys<<<(nl + 255) / 256, 256, 0, s>>>(mk, L, lstarts, nl, lk));
    OWM_LAUNCH("k_karras", s, k_karras<<<(nl - 1 + 255) / 256, 256, 0, s>>>(lk, 1, nullptr, nl, t->nodes, parent,
                                                                           right_of, last_of, flags));
    OWM_LAUNCH("k_refit", s, k_refit<<<(nl + 255) / 256, 256, 0, s>>>(t->nodes, parent, flags, right_of, last_of, nl));
    count_launch(launches, 3);
  }
  t->max_leaf = fixed ? L : -1;
  OWM_CUDA_TRY(cudaGetLastError());
  return OWM_OK;
}

int check_tree(const TreeStore* t, int32_t* d_bad, cudaStream_t s, int64_t* launches, int32_t* h_bad) {
  OWM_CUDA_TRY(cudaMemsetAsync(d_bad, 0, 4, s));
  if (t->nleaves > 1) {
    k_check_counts<<<(t->nleaves - 1 + 255) / 256, 256, 0, s>>>(t->nodes, t->nleaves, d_bad);
    count_launch(launches);
  }
  OWM_CUDA_TRY(cudaMemcpyAsync(h_bad, d_bad, 4, cudaMemcpyDeviceToHost, s));
  OWM_CUDA_TRY(cudaStreamSynchronize(s));
  return OWM_OK;
}

}  // namespace owm
