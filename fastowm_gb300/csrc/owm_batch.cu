// Batched tiles: many independent clouds (own bbox, Wsize, overlap, Bsize and
// leaf size) built and queried together with one launch per step instead of
// one launch sequence per tile.
//
//   * all points are sorted once on a (tile, Morton) key, so every tile's
//     points stay in their own contiguous range;
//   * leaves, Karras hierarchies, escape links and refits of all tiles are
//     built by single launches that find their tile by binary search over
//     per-tile offsets;
//   * stage 1 by exact window classes: per-tile class tables built by two
//     launches, every point folded into its tile's sub-cell counters inside
//     the gather, then batched row and window reductions (a tile that
//     asks for the tree walk switches the whole batch to the persistent walk);
//   * stage 3 (and the stage-1 walk) is one persistent query launch: warps
//     pull 4 x 8 window patches of any tile from one work counter, which
//     balances uneven tiles;
//   * stage 2 sorts all window results on a (tile, id) key;
//   * the device part can be captured once into a CUDA graph and replayed
//     while the tile shapes repeat.
// Results per tile are exactly those of owm_run on that tile alone (ids are
// 1-based within the tile).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "owm_batch.cuh"
#include "owm_cellq.cuh"
#include "owm_classes.cuh"
#include "owm_devutil.cuh"

namespace owm {

namespace {

// Largest t in [0, ntiles) with off[t] <= x (off has ntiles+1 entries,
// off[0] = 0, off[ntiles] > x): the tile that owns global index x.
template <class T>
__device__ __forceinline__ int tile_of(const T* __restrict__ off, int ntiles, int64_t x) {
  int lo = 0, hi = ntiles - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if ((int64_t)__ldg(off + mid) <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__global__ void k_b_morton(const double* __restrict__ xyz, int64_t n, const int64_t* __restrict__ pt_off,
                           const TileMeta* __restrict__ meta, int ntiles, int mbits, uint32_t* __restrict__ keys) {
  const float qmax = (float)((1u << mbits) - 1u);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int t = tile_of(pt_off, ntiles, i);
    const TileMeta& m = meta[t];
    const double x = __ldg(xyz + 3 * i), y = __ldg(xyz + 3 * i + 1);
    uint32_t qx, qy;
    if (m.mint) {  // order keys are linear over the tile's domain: no FP64 arithmetic
      const int64_t qm = (1ll << mbits) - 1;
      int64_t a = (dkey(x) - m.mkx0) >> m.mshx, b = (dkey(y) - m.mky0) >> m.mshy;
      qx = (uint32_t)(a < 0 ? 0 : (a > qm ? qm : a));
      qy = (uint32_t)(b < 0 ? 0 : (b > qm ? qm : b));
    } else {
      float fx = (float)((x - m.mox) * m.mscale), fy = (float)((y - m.moy) * m.mscale);
      qx = (uint32_t)fminf(fmaxf(fx, 0.0f), qmax);
      qy = (uint32_t)fminf(fmaxf(fy, 0.0f), qmax);
    }
    keys[i] = ((uint32_t)t << (2 * mbits)) | (spread_bits16(qx) << 1) | spread_bits16(qy);
  }
}

// (tile, Morton) key of point i of tile m (the tile's integer or FP64 form).
struct TileKey {
  int64_t kx0, ky0, qm;
  double ox, oy, scale;
  float qmax;
  int shx, shy, mint;
  uint32_t tile_bits_key;  // t << (2 * mbits)
  __device__ __forceinline__ void load(const TileMeta& m, int t, int mbits) {
    kx0 = m.mkx0;
    ky0 = m.mky0;
    shx = m.mshx;
    shy = m.mshy;
    mint = m.mint;
    ox = m.mox;
    oy = m.moy;
    scale = m.mscale;
    qm = (1ll << mbits) - 1;
    qmax = (float)((1u << mbits) - 1u);
    tile_bits_key = (uint32_t)t << (2 * mbits);
  }
  __device__ __forceinline__ uint32_t operator()(const double* __restrict__ p) const {
    const double x = __ldg(p), y = __ldg(p + 1);
    uint32_t qx, qy;
    if (mint) {  // order keys are linear over the tile's domain: no FP64 arithmetic
      const int64_t a = (dkey(x) - kx0) >> shx, b = (dkey(y) - ky0) >> shy;
      qx = (uint32_t)(a < 0 ? 0 : (a > qm ? qm : a));
      qy = (uint32_t)(b < 0 ? 0 : (b > qm ? qm : b));
    } else {
      const float fx = (float)((x - ox) * scale), fy = (float)((y - oy) * scale);
      qx = (uint32_t)fminf(fmaxf(fx, 0.0f), qmax);
      qy = (uint32_t)fminf(fmaxf(fy, 0.0f), qmax);
    }
    return tile_bits_key | (spread_bits16(qx) << 1) | spread_bits16(qy);
  }
};

// Keys of part blockIdx.x of the batch's sort (sort_part_range, contiguous
// points), with the part's counts of the first radix digit into
// counts[d * gridDim.x + blockIdx.x].  Each thread finds its tile once and
// walks forward with the tile's key parameters in registers.
// At most 32 registers a thread (4 bytes spill): 8 blocks of 256 per SM, so
// the batch's 4 x 304 sort parts run in one wave (48 registers: 5 blocks, two
// waves; 1.59 -> 1.28 ms for the 512-tile batch).  Launched with 256 threads.
__global__ void __maxnreg__(32) k_b_morton_counts(const double* __restrict__ xyz, int64_t n,
                                                         const int64_t* __restrict__ pt_off,
                                                         const TileMeta* __restrict__ meta, int ntiles, int mbits,
                                                         int64_t ntiles_sort, uint32_t dmask0, uint32_t* __restrict__ keys,
                                                         uint32_t* __restrict__ counts) {
  __shared__ uint32_t h[8][256];
  for (int i = threadIdx.x; i < 8 * 256; i += 256) (&h[0][0])[i] = 0;
  __syncthreads();
  int64_t b, e;
  sort_part_range(n, ntiles_sort, gridDim.x, blockIdx.x, &b, &e);
  uint32_t* hw = h[threadIdx.x >> 5];
  int64_t i = b + threadIdx.x;
  if (i < e) {
    int t = tile_of(pt_off, ntiles, i);
    int64_t tend = __ldg(pt_off + t + 1);
    TileKey key;
    key.load(meta[t], t, mbits);
    for (; i < e;) {
      while (i >= tend) {  // next tile (tiles are contiguous; empty ones skipped)
        ++t;
        tend = __ldg(pt_off + t + 1);
        key.load(meta[t], t, mbits);
      }
      if (i + 3 * 256 < e && i + 3 * 256 < tend) {  // four points of this tile in flight
        uint32_t k[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) k[u] = key(xyz + 3 * (i + u * 256));
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          keys[i + u * 256] = k[u];
          atomicAdd(hw + (k[u] & dmask0), 1u);
        }
        i += 4 * 256;
      } else {
        const uint32_t k = key(xyz + 3 * i);
        keys[i] = k;
        atomicAdd(hw + (k & dmask0), 1u);
        i += 256;
      }
    }
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

// One warp per global leaf: gather its points into sorted order as keys and
// reduce the leaf summary.  At most 40 registers a thread (a few bytes spill)
// so that more warps wait on the point reads at once: 8.01 -> 6.91 ms for the
// 512-tile batch (59 registers before; 48 registers 7.08 ms).  Launched with
// at most 512 threads.
__global__ void __maxnreg__(40) k_b_gather_leaves(const double* __restrict__ xyz,
                                                         const uint32_t* __restrict__ perm,
                                                         const TileMeta* __restrict__ meta,
                                                         const int32_t* __restrict__ leaf_off, int ntiles,
                                                         int64_t total_leaves, int64_t* __restrict__ xk,
                                                         int64_t* __restrict__ yk, int64_t* __restrict__ zk,
                                                         uint32_t* __restrict__ pid, Node* __restrict__ nodes,
                                                         uint32_t* __restrict__ status,
                                                         const ClassArgs* __restrict__ cls) {
  const int lane = threadIdx.x & 31;
  bool finite = true;
  for (int64_t g = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; g < total_leaves;
       g += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int t = tile_of(leaf_off, ntiles, g);
    const TileMeta& m = meta[t];
    const int32_t j = (int32_t)(g - m.leaf_off);
    const int32_t first = j * m.leaf;
    const int32_t cnt = min(m.leaf, m.n - first);
    LeafAcc acc;
    acc.init();
    for (int32_t c0 = 0; c0 < cnt; c0 += 32) {  // warp-uniform: the class fold needs whole warps
      const int32_t lp = first + c0 + lane;
      const bool valid = c0 + lane < cnt;
      int64_t x = 0, y = 0, z = 0;
      uint32_t id = 0;
      if (valid) {
        const int64_t gp = m.pt_off + lp;
        const uint32_t src = __ldg(perm + gp);
        finite &= load_point(xyz, src, x, y, z);
        id = (uint32_t)((int64_t)src - m.pt_off + 1);
        xk[gp] = x;
        yk[gp] = y;
        zk[gp] = z;
        pid[gp] = id;
        acc.add(x, y, z, id, (uint32_t)lp);
      }
      if (cls) {
        if (!__all_sync(0xffffffffu, valid)) {  // short leaf: idle lanes borrow lane 0's point
          const int64_t bx = __shfl_sync(0xffffffffu, x, 0), by = __shfl_sync(0xffffffffu, y, 0);
          if (!valid) {
            x = bx;
            y = by;
            z = 0;
          }
        }
        cls_aggregate_warp(cls[t], valid, x, y, z, id, lane);
      }
    }
    acc.reduce(32);
    write_leaf_seg(nodes + m.node_off + (m.nleaves - 1) + j, acc, first, m.ox, m.oy, 32, true);
  }
  if (!finite) atomicOr(status, kStatusNonFinite);
}

// ---- stage 1 by window classes, all tiles per launch ----------------------
// Grid y = tile.  Edge keys of the tile's window columns and rows.
__global__ void k_bc_split(const ClassArgs* __restrict__ cls, const TileMeta* __restrict__ meta,
                           const Edge* __restrict__ E_wx, const Edge* __restrict__ E_wy) {
  const ClassArgs& A = cls[blockIdx.y];
  const TileMeta& m = meta[blockIdx.y];
  const int32_t nmax = max(A.nx, A.ny);
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nmax; i += gridDim.x * blockDim.x) {
    if (i < A.nx) {
      const Edge e = E_wx[m.ex_off + i];
      const_cast<int64_t*>(A.Lx)[i] = e.lo_k;
      const_cast<int64_t*>(A.Rx)[i] = e.hi_k;
    }
    if (i < A.ny) {
      const Edge e = E_wy[m.ey_off + i];
      const_cast<int64_t*>(A.Ly)[i] = e.lo_k;
      const_cast<int64_t*>(A.Ry)[i] = e.hi_k;
    }
  }
}

// Grid y = tile.  s-ranges of the windows and the class tables.
__global__ void k_bc_prep(const ClassArgs* __restrict__ cls) {
  const ClassArgs& A = cls[blockIdx.y];
  const int32_t nmax = max(max(A.nx, A.ny), max(A.qx, A.qy));
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nmax; i += gridDim.x * blockDim.x) {
    if (i < A.nx) cls_range_one(A.Lx, A.Rx, A.nx, i, A.sxl + i, A.sxh + i);
    if (i < A.ny) cls_range_one(A.Ly, A.Ry, A.ny, i, A.syl + i, A.syh + i);
    if (i < A.qx) const_cast<ClsCell*>(A.tabx)[i] = cls_table_one(A.Lx, A.Rx, A.nx, A.kx0, A.shx, i);
    if (i < A.qy) const_cast<ClsCell*>(A.taby)[i] = cls_table_one(A.Ly, A.Ry, A.ny, A.ky0, A.shy, i);
  }
}

__global__ void k_bc_rows(const ClassArgs* __restrict__ cls, const int64_t* __restrict__ rows_off, int ntiles,
                          int64_t total) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (int64_t)gridDim.x * blockDim.x) {
    const int t = tile_of(rows_off, ntiles, k);
    cls_row_one(cls[t], k - __ldg(rows_off + t));
  }
}

__global__ void k_bc_windows(const ClassArgs* __restrict__ cls, const TileMeta* __restrict__ meta,
                             const int64_t* __restrict__ win_off, int ntiles, int64_t total,
                             uint32_t* __restrict__ win) {
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < total; w += (int64_t)gridDim.x * blockDim.x) {
    const int t = tile_of(win_off, ntiles, w);
    const int64_t off = __ldg(win_off + t);
    win[off + cls_window_slot(cls[t], w - off)] = cls_window_one(cls[t], w - off, meta[t].thr);
  }
}

// lk: packed leaf keys (k_b_leaf_keys), lk[m.leaf_off + i] for leaf i of tile m.
__device__ __forceinline__ int bdelta(const uint32_t* __restrict__ lk, const TileMeta& m, int32_t i, int32_t j) {
  if (j < 0 || j >= m.nleaves) return -1;
  uint64_t a = ((uint64_t)__ldg(lk + m.leaf_off + i) << 32) | (uint32_t)i;
  uint64_t b = ((uint64_t)__ldg(lk + m.leaf_off + j) << 32) | (uint32_t)j;
  return __clzll((long long)(a ^ b));
}

// Key of every leaf's first point, packed over all tiles.
__global__ void k_b_leaf_keys(const uint32_t* __restrict__ mk, const TileMeta* __restrict__ meta,
                              const int32_t* __restrict__ leaf_off, int ntiles, int64_t total_leaves,
                              uint32_t* __restrict__ lk) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total_leaves) return;
  const int t = tile_of(leaf_off, ntiles, g);
  const TileMeta& m = meta[t];
  lk[g] = __ldg(mk + m.pt_off + (g - m.leaf_off) * m.leaf);
}

// Karras (2012) per tile; indices stored local to the tile.
// Also readies k_b_refit: each tile's root has parent -1 and every internal
// node's arrival counter starts at 0.
__global__ void k_b_karras(const uint32_t* __restrict__ lk, const TileMeta* __restrict__ meta,
                           const int32_t* __restrict__ int_off, int ntiles, int64_t total_internal,
                           Node* __restrict__ nodes, int32_t* __restrict__ parent, int32_t* __restrict__ right_of,
                           int32_t* __restrict__ last_of, int32_t* __restrict__ flags) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= total_internal) return;
  const int t = tile_of(int_off, ntiles, q);
  const TileMeta& m = meta[t];
  const int32_t i = (int32_t)(q - m.int_off);
  const int32_t nl = m.nleaves;
  flags[q] = 0;
  if (i == 0) parent[m.node_off] = -1;  // no node of the tile has its root as a child
  int d = bdelta(lk, m, i, i + 1) - bdelta(lk, m, i, i - 1) > 0 ? 1 : -1;
  int dmin = bdelta(lk, m, i, i - d);
  int32_t lmax = 2;
  while (bdelta(lk, m, i, i + lmax * d) > dmin) lmax <<= 1;
  int32_t l = 0;
  for (int32_t s = lmax >> 1; s >= 1; s >>= 1)
    if (bdelta(lk, m, i, i + (l + s) * d) > dmin) l += s;
  int32_t j = i + l * d;
  int dnode = bdelta(lk, m, i, j);
  int32_t s = 0;
  for (int32_t div = 2;; div <<= 1) {
    int32_t st = (l + div - 1) / div;
    if (bdelta(lk, m, i, i + (s + st) * d) > dnode) s += st;
    if (st <= 1) break;
  }
  int32_t gamma = i + s * d + (d < 0 ? -1 : 0);
  int32_t lo = min(i, j), hi = max(i, j);
  int32_t left = (lo == gamma) ? (nl - 1 + gamma) : gamma;
  int32_t right = (hi == gamma + 1) ? (nl - 1 + gamma + 1) : gamma + 1;
  Node* base = nodes + m.node_off;
  base[i].left = left;
  base[i].right = right;
  parent[m.node_off + left] = i;
  parent[m.node_off + right] = i;
  right_of[m.leaf_off + gamma] = right;
  last_of[m.int_off + i] = hi;
}

// Arrival at a node of the bottom-up refit: the first arriver's summary
// stores are released by its increment and acquired by the second arriver's,
// which then reads both children from L2.
__device__ __forceinline__ int32_t arrive_acq_rel(int32_t* f) {
  int32_t old;
  asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], 1;" : "=r"(old) : "l"(f) : "memory");
  return old;
}

// Bottom-up refit of every tile's hierarchy; every node also gets its escape
// link (the right child of the split after its last leaf, or end) from the
// thread that starts at a leaf or arrives second at an internal node.
__global__ void k_b_refit(Node* __restrict__ nodes, const int32_t* __restrict__ parent, int32_t* __restrict__ flags,
                          const int32_t* __restrict__ right_of, const int32_t* __restrict__ last_of,
                          const TileMeta* __restrict__ meta, const int32_t* __restrict__ leaf_off, int ntiles,
                          int64_t total_leaves) {
  int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total_leaves) return;
  const int t = tile_of(leaf_off, ntiles, g);
  const TileMeta& m = meta[t];
  Node* base = nodes + m.node_off;
  const int32_t li = (int32_t)(g - m.leaf_off);
  const int32_t nl = m.nleaves;
  base[nl - 1 + li].escape = li >= nl - 1 ? kEnd : __ldg(right_of + m.leaf_off + li);
  if (nl <= 1) return;  // a one-leaf tile: the leaf is the root
  int32_t n = parent[m.node_off + nl - 1 + li];
  for (int32_t guard = 0; n >= 0 && guard < m.nleaves; ++guard) {
    // acquire-release arrival (see arrive_acq_rel)
    if (arrive_acq_rel(flags + m.int_off + n) == 0) return;
    const Node* a = base + __ldcg(&base[n].left);
    const Node* b = base + __ldcg(&base[n].right);
    float4 ba = __ldcg(reinterpret_cast<const float4*>(a)), bb = __ldcg(reinterpret_cast<const float4*>(b));
    int64_t za = __ldcg(&a->zmin), zb = __ldcg(&b->zmin);
    uint32_t ia = __ldcg(&a->min_id), ib = __ldcg(&b->min_id);
    uint32_t pa = __ldcg(&a->min_pos), pb = __ldcg(&b->min_pos);
    uint32_t ca = __ldcg(&a->count), cb = __ldcg(&b->count);
    Node* o = base + n;
    __stcg(reinterpret_cast<float4*>(o),
           make_float4(fminf(ba.x, bb.x), fminf(ba.y, bb.y), fmaxf(ba.z, bb.z), fmaxf(ba.w, bb.w)));
    bool bl = zid_less(zb, ib, za, ia);
    __stcg(&o->zmin, bl ? zb : za);
    __stcg(&o->min_id, bl ? ib : ia);
    __stcg(&o->min_pos, bl ? pb : pa);
    __stcg(&o->count, ca + cb);
    const int32_t last = __ldg(last_of + m.int_off + n);
    o->escape = last >= nl - 1 ? kEnd : __ldg(right_of + m.leaf_off + last);
    n = parent[m.node_off + n];
  }
}

// Stage 3 of all tiles: one warp per grid cell of any tile (cell_off gives
// each tile's first cell), answered by the tile's stage-3 job; marked cells
// are skipped at once.
template <int kW>
__global__ void __launch_bounds__(kW * 32) k_b_query_cells(const QueryJob* __restrict__ jobs,
                                                             const int64_t* __restrict__ cell_off, int ntiles,
                                                             int64_t total_cells) {
  extern __shared__ int32_t stack_all[];  // [kW][kS3Stack]
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int64_t c = (int64_t)blockIdx.x * kW + wib;
  if (c >= total_cells) return;  // warp-uniform
  const int t = tile_of(cell_off, ntiles, c);
  const QueryJob& J = jobs[t];
  const int64_t k = c - __ldg(cell_off + t);
  if (J.skip && J.skip[k]) {
    if (lane == 0) J.out[k] = kNone;
    return;
  }
  const uint32_t r =
      cell_min_warp<false>(J.tree, J.ex[k % J.ncols], J.ey[k / J.ncols], stack_all + wib * kS3Stack, J.status, lane);
  if (lane == 0) J.out[k] = r;
}

template <int kW>
cudaError_t launch_b_query_cells(const QueryJob* jobs, const int64_t* cell_off, int ntiles, int64_t total_cells,
                                 cudaStream_t s) {
  static bool configured = false;  // per template instance
  const size_t smem = (size_t)kW * kS3Stack * sizeof(int32_t);
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(k_b_query_cells<kW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  OWM_LAUNCH("k_query_s3_batch", s, (k_b_query_cells<kW><<<(unsigned)((total_cells + kW - 1) / kW), kW * 32, smem, s>>>(
      jobs, cell_off, ntiles, total_cells)));
  return cudaGetLastError();
}

__device__ __forceinline__ Edge bedge(double lo, double hi, double o) {
  Edge e;
  e.lo_k = dkey(lo);
  e.hi_k = dkey(hi);
  e.lo_dn = __double2float_rd(__dsub_rd(lo, o));
  e.lo_up = __double2float_ru(__dsub_ru(lo, o));
  e.hi_dn = __double2float_rd(__dsub_rd(hi, o));
  e.hi_up = __double2float_ru(__dsub_ru(hi, o));
  return e;
}

// Edge tables of every tile: kind 0 = stage-1 windows, 1 = stage-3 cells;
// axis 0 = x, 1 = y.  Same arithmetic as the single-cloud k_edges.
__global__ void k_b_edges(int kind, int axis, const TileMeta* __restrict__ meta, const int32_t* __restrict__ off,
                          int ntiles, int64_t total, Edge* __restrict__ out) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= total) return;
  const int t = tile_of(off, ntiles, e);
  const TileMeta& m = meta[t];
  const int32_t i = (int32_t)(e - off[t]);
  const double mn = axis ? m.min_y : m.min_x;
  const double o = axis ? m.oy : m.ox;
  double c, r;
  if (kind) {
    r = (double)(float)m.bhalf;
    c = __dadd_rn(__dadd_rn(mn, (double)m.bhalf), (double)(i * m.bsize));
  } else {
    r = (double)(float)m.whalf;
    double init = __dadd_rn(__dsub_rn(mn, (double)m.whalf), m.displace);
    c = __dadd_rn(init, __dmul_rn((double)i, m.displace));
  }
  out[e] = bedge(__dsub_rn(c, r), __dadd_rn(c, r), o);
}

__global__ void k_b_s2_keys(const uint32_t* __restrict__ win, int64_t n, const int64_t* __restrict__ win_off,
                            int ntiles, int idbits, uint32_t none, uint32_t* __restrict__ keys) {
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < n; w += (int64_t)gridDim.x * blockDim.x) {
    int t = tile_of(win_off, ntiles, w);
    uint32_t v = win[w];
    keys[w] = ((uint32_t)t << idbits) | (v == kNone ? none : v);
  }
}

__global__ void k_b_s2_flags(const uint32_t* __restrict__ keys, int64_t n, int idbits, uint32_t none,
                             const TileMeta* __restrict__ meta, uint32_t* __restrict__ flags,
                             uint32_t* __restrict__ tile_count) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    uint32_t k = keys[i];
    uint32_t t = k >> idbits;
    bool f = (k & none) != none;  // overlap 0: every valid minimum
    if (meta[t].need_dup) f = f && (i == 0 || keys[i - 1] != k) && (i + 1 < n && keys[i + 1] == k);
    flags[i] = f ? 1u : 0u;
    if (f) atomicAdd(tile_count + t, 1u);
  }
}

// Stage 2 of a batch whose tiles all have overlap > 0, by occupancy bitmaps:
// tile t owns words [bm_off[t], bm_off[t+1]) for its ids 0..n, so emitting
// the set bits in word order lists the LLPs tile by tile, ids ascending --
// the (tile, id)-sorted list with every id of run length >= 2 (the first
// atomic OR of an id's bit returns the old word; a second occurrence sets
// the bit in `twice`).
__global__ void k_b_s2_mark(const uint32_t* __restrict__ win, int64_t nw, const int64_t* __restrict__ win_off,
                            int ntiles, const TileMeta* __restrict__ meta, uint32_t* __restrict__ once,
                            uint32_t* __restrict__ twice) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nw; i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t v = win[i];
    if (v == kNone) continue;
    const TileMeta& m = meta[tile_of(win_off, ntiles, i)];
    if (v > (uint32_t)m.n) continue;  // not an id of the tile (cannot happen)
    const int64_t idx = m.bm_word * 32 + v;
    const uint32_t bit = 1u << (idx & 31);
    const uint32_t old = atomicOr(once + (idx >> 5), bit);
    if (old & bit) atomicOr(twice + (idx >> 5), bit);
  }
}

__global__ void k_b_s2_popc(const uint32_t* __restrict__ bm, int64_t nw, uint32_t* __restrict__ cnt) {
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < nw; w += (int64_t)gridDim.x * blockDim.x)
    cnt[w] = (uint32_t)__popc(bm[w]);
}

__global__ void k_b_s2_emit(const uint32_t* __restrict__ bm, const uint32_t* __restrict__ pos, int64_t nw,
                            const int64_t* __restrict__ bm_off, int ntiles, int idbits, uint32_t* __restrict__ llp) {
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < nw; w += (int64_t)gridDim.x * blockDim.x) {
    uint32_t b = bm[w];
    if (!b) continue;
    const int t = tile_of(bm_off, ntiles, w);
    const uint32_t base = (uint32_t)((w - bm_off[t]) * 32);
    uint32_t p = pos[w];
    while (b) {
      llp[p++] = ((uint32_t)t << idbits) | (base + (uint32_t)(__ffs(b) - 1));
      b &= b - 1;
    }
  }
}

// LLPs per tile: the scanned word counts at the tile's word boundaries.
__global__ void k_b_s2_tilecount(const uint32_t* __restrict__ pos, const int64_t* __restrict__ bm_off, int ntiles,
                                 int64_t nw, const uint32_t* __restrict__ total, uint32_t* __restrict__ cnt) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ntiles; t += gridDim.x * blockDim.x) {
    const uint32_t a = bm_off[t] < nw ? pos[bm_off[t]] : *total;
    const uint32_t b = bm_off[t + 1] < nw ? pos[bm_off[t + 1]] : *total;
    cnt[t] = b - a;
  }
}

__global__ void k_b_compact(const uint32_t* __restrict__ vals, const uint32_t* __restrict__ flags,
                            const uint32_t* __restrict__ pos, int64_t n, uint32_t* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (flags[i]) out[pos[i]] = vals[i];
}

__global__ void k_b_s3_mark(const double* __restrict__ xyz, const uint32_t* __restrict__ llp,
                            const uint32_t* __restrict__ nllp, int64_t cap, int idbits,
                            const TileMeta* __restrict__ meta, const Edge* __restrict__ cell_ex,
                            const Edge* __restrict__ cell_ey, uint8_t* __restrict__ mark) {
  const int64_t n = min((int64_t)*nllp, cap);
  const uint32_t mask = (idbits >= 32) ? 0xFFFFFFFFu : ((1u << idbits) - 1u);
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t key = llp[k];
    const TileMeta& m = meta[key >> idbits];
    if (m.bsize == 0 || m.ncg <= 0) continue;
    const uint32_t id = key & mask;
    double x = 0.0, y = 0.0;  // id 0 = sentinel {0, 0, DBL_MAX}
    if (id > 0) {
      x = xyz[3 * (m.pt_off + id - 1)];
      y = xyz[3 * (m.pt_off + id - 1) + 1];
    }
    const int64_t xk = dkey(x), yk = dkey(y);
    double fi = floor((x - m.min_x) / (double)m.bsize), fj = floor((y - m.min_y) / (double)m.bsize);
    if (!(fi > -4.0 && fi < (double)m.ncg + 4.0 && fj > -4.0 && fj < (double)m.nrg + 4.0)) continue;
    const int32_t ic = (int32_t)fi, jc = (int32_t)fj;
    const Edge* ex = cell_ex + m.cx_off;
    const Edge* ey = cell_ey + m.cy_off;
    for (int32_t jj = max(jc - 1, 0); jj <= min(jc + 1, m.nrg - 1); ++jj) {
      if (!(yk > ey[jj].lo_k && yk < ey[jj].hi_k)) continue;
      for (int32_t ii = max(ic - 1, 0); ii <= min(ic + 1, m.ncg - 1); ++ii)
        if (xk > ex[ii].lo_k && xk < ex[ii].hi_k) mark[m.cell_off + (int64_t)jj * m.ncg + ii] = 1;
    }
  }
}

__global__ void k_b_flag_cells(const uint32_t* __restrict__ cellmin, int64_t n, const int64_t* __restrict__ cell_off,
                               int ntiles, uint32_t* __restrict__ flags, uint32_t* __restrict__ tile_count) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    bool f = cellmin[i] != kNone;
    flags[i] = f ? 1u : 0u;
    if (f) atomicAdd(tile_count + tile_of(cell_off, ntiles, i), 1u);
  }
}

// Per tile t: out[out_off[t] ..] = its stage-3 ids, then its LLPs.
__global__ void k_b_assemble(const uint32_t* __restrict__ s3, const uint32_t* __restrict__ s3_off,
                             const uint32_t* __restrict__ llp, const uint32_t* __restrict__ llp_off, int idbits,
                             int ntiles, int64_t* __restrict__ out, int64_t* __restrict__ out_off) {
  const uint32_t mask = (idbits >= 32) ? 0xFFFFFFFFu : ((1u << idbits) - 1u);
  const int64_t n3 = s3_off[ntiles], nl = llp_off[ntiles];
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n3 + nl + ntiles + 1;
       k += (int64_t)gridDim.x * blockDim.x) {
    if (k < n3) {
      int t = tile_of(s3_off, ntiles, k);
      out[(int64_t)s3_off[t] + llp_off[t] + (k - s3_off[t])] = s3[k];
    } else if (k < n3 + nl) {
      int64_t q = k - n3;
      int t = tile_of(llp_off, ntiles, q);
      out[(int64_t)s3_off[t + 1] + llp_off[t] + (q - llp_off[t])] = llp[q] & mask;
    } else {
      int64_t t = k - n3 - nl;
      out_off[t] = (int64_t)s3_off[t] + llp_off[t];
    }
  }
}

int gsz(int64_t n, int block = 256) {
  int64_t g = (n + block - 1) / block;
  return (int)std::max<int64_t>(1, std::min<int64_t>(g, 152 * 32));
}

size_t a256(size_t b) { return (b + 255) & ~(size_t)255; }

int bits_for(uint64_t v) {  // smallest b with 2^b > v
  int b = 0;
  while (b < 64 && ((uint64_t)1 << b) <= v) ++b;
  return b;
}

// Everything a batch needs, derived on the host from the tile shapes.
struct Plan {
  int32_t ntiles = 0;
  int64_t npts = 0, nleaves = 0, nnodes = 0, ninternal = 0, nwin = 0, ncell = 0;
  int64_t ex = 0, ey = 0, cx = 0, cy = 0;
  int tile_bits = 1, mbits = 8, idbits = 1;
  std::vector<TileMeta> meta;
  std::vector<int64_t> pt_off, win_off, cell_off;
  // stage 2 by bitmaps when every tile has overlap > 0 (ids 0..n per tile, word-aligned)
  bool s2_bitmap = true;
  int64_t bm_words = 0;
  std::vector<int64_t> bm_off;
  size_t o_bm1 = 0, o_bm2 = 0, o_bmc = 0, o_bmp = 0, o_bmt = 0, o_bmoff = 0;
  std::vector<int32_t> leaf_off, node_off, int_off, ex_off, ey_off, cx_off, cy_off;
  // stage 1 by window classes (when no tile asks for the tree walk)
  struct ClsLayout {
    size_t tabx, taby, Lx, Rx, Ly, Ry, sxl, sxh, syl, syh, rc, rz, ri;  // byte offsets in the misc region
    int64_t sub_off;                                                   // first sub-cell of the tile
  };
  bool classes = false;
  std::vector<ClassArgs> cls;      // per-tile geometry (pointers are set at launch)
  std::vector<ClsLayout> clay;
  std::vector<int64_t> rows_off;   // prefix of (window columns x sub-cell rows)
  int64_t nsub = 0, rows_total = 0;
  size_t cls_misc = 0;
  int32_t cls_grid_x = 1;          // blocks per tile of the class prepare launches
  size_t o_cls = 0, o_rowsoff = 0, o_ccount = 0, o_czid = 0, o_cmisc = 0;
  // buffer offsets (bytes) inside the batch buffer
  size_t o_xyz, o_k0, o_k1, o_v0, o_v1, o_sort, o_xk, o_yk, o_zk, o_pid, o_nodes, o_parent, o_flags, o_right,
      o_last, o_edges, o_win, o_s2k0, o_s2k1, o_s2f, o_s2p, o_s2t, o_llp, o_mark, o_cmin, o_cf, o_cp, o_ct, o_s3,
      o_meta, o_jobs1, o_jobs3, o_ptoff, o_leafoff, o_nodeoff, o_intoff, o_exoff, o_eyoff, o_cxoff, o_cyoff,
      o_winoff, o_celloff, o_cnt2, o_cnt3, o_llpoff, o_s3off, o_out, o_outoff, o_words, total;
};

int make_plan(const owm_tile_desc* td, int32_t ntiles, const BatchRun& br, Plan* P) {
  P->ntiles = ntiles;
  P->meta.resize(ntiles);
  P->pt_off.assign(ntiles + 1, 0);
  P->bm_off.assign(ntiles + 1, 0);
  P->s2_bitmap = true;
  P->bm_words = 0;
  P->win_off.assign(ntiles + 1, 0);
  P->cell_off.assign(ntiles + 1, 0);
  for (auto* v : {&P->leaf_off, &P->node_off, &P->int_off, &P->ex_off, &P->ey_off, &P->cx_off, &P->cy_off})
    v->assign(ntiles + 1, 0);
  P->tile_bits = std::max(1, bits_for((uint64_t)ntiles - 1));
  // Morton bits per axis: fit (tile, Morton) keys in 24 bits (three 8-bit
  // sort passes) while that leaves at least 7 bits per axis (128 x 128 cells
  // per tile); else use up to 32 bits.  Seeds do not depend on it.
  P->mbits = (24 - P->tile_bits) / 2 >= 7 ? (24 - P->tile_bits) / 2 : std::min(16, (32 - P->tile_bits) / 2);
  P->classes = true;
  for (int32_t t = 0; t < ntiles; ++t) P->classes &= td[t].cfg.stage1_walk == 0;
  if (P->classes) {
    P->cls.assign(ntiles, ClassArgs{});
    P->clay.assign(ntiles, Plan::ClsLayout{});
    P->rows_off.assign(ntiles + 1, 0);
  }
  int32_t cls_span = 1;
  int64_t maxn = 0;
  for (int32_t t = 0; t < ntiles; ++t) {
    const owm_tile_desc& d = td[t];
    if (!d.xyz || d.n <= 0 || d.n >= 0x7FFFFFFFLL) return OWM_EINVAL;
    if (validate_tree_cfg(&d.cfg.tree) != OWM_OK || d.cfg.tree.policy != OWM_TREE_MAX_NUMBER) return OWM_EINVAL;
    owm_bbox bb = d.bbox;
    if (!(bb.min_x <= bb.max_x)) {
      if (is_device_ptr(d.xyz)) return OWM_EINVAL;  // device tiles must carry their bbox
      owm_bbox_of(d.xyz, d.n, &bb);
    }
    owm_params p;
    int rc = owm_params_compute(&bb, d.n, d.cfg.wsize, d.cfg.overlap, d.cfg.bsize, &p);
    if (rc) return rc;
    maxn = std::max<int64_t>(maxn, d.n);
    TileMeta& m = P->meta[t];
    std::memset(&m, 0, sizeof(m));
    m.pt_off = P->npts;
    m.n = (int32_t)d.n;
    m.leaf = leaf_size(br.leaf_for(d.n, d.cfg.tree.max_number));
    int32_t nl = (int32_t)((d.n + m.leaf - 1) / m.leaf);
    m.leaf_off = (int32_t)P->nleaves;
    m.nleaves = nl;
    m.node_off = (int32_t)P->nnodes;
    m.int_off = (int32_t)P->ninternal;
    double rx = (bb.max_x - bb.min_x) * 0.5, ry = (bb.max_y - bb.min_y) * 0.5;
    double R = rx >= ry ? rx : ry;
    if (!(R > 0.0)) R = 0.5;
    m.mox = bb.min_x + rx - R;
    m.moy = bb.min_y + ry - R;
    m.mscale = (double)(1u << P->mbits) / (2.0 * R);
    m.mint = (morton_int_shifts(m.mox, m.mox + 2.0 * R, P->mbits, &m.mkx0, &m.mshx) &&
              morton_int_shifts(m.moy, m.moy + 2.0 * R, P->mbits, &m.mky0, &m.mshy))
                 ? 1
                 : 0;
    m.ox = bb.min_x;
    m.oy = bb.min_y;
    m.min_x = bb.min_x;
    m.min_y = bb.min_y;
    m.displace = p.displace;
    m.ncols = (int32_t)p.ncols;
    m.nrows = (int32_t)p.nrows;
    m.ncg = (int32_t)p.ncols_grid;
    m.nrg = (int32_t)p.nrows_grid;
    m.whalf = ((uint16_t)p.wsize) / 2;
    m.bhalf = ((uint16_t)p.bsize) / 2;
    m.bsize = (uint16_t)p.bsize;
    m.thr = p.min_num_points;
    m.need_dup = p.overlap > 0.0 ? 1 : 0;
    if (!m.need_dup) P->s2_bitmap = false;  // overlap 0 keeps every valid minimum: the sort path
    m.bm_word = P->bm_words;
    P->bm_off[t] = P->bm_words;
    P->bm_words += ((int64_t)d.n + 1 + 31) / 32;
    m.win_off = P->nwin;
    m.cell_off = P->ncell;
    m.ex_off = (int32_t)P->ex;
    m.ey_off = (int32_t)P->ey;
    m.cx_off = (int32_t)P->cx;
    m.cy_off = (int32_t)P->cy;
    P->pt_off[t] = P->npts;
    P->leaf_off[t] = m.leaf_off;
    P->node_off[t] = m.node_off;
    P->int_off[t] = m.int_off;
    P->win_off[t] = P->nwin;
    P->cell_off[t] = P->ncell;
    P->ex_off[t] = (int32_t)P->ex;
    P->ey_off[t] = (int32_t)P->ey;
    P->cx_off[t] = (int32_t)P->cx;
    P->cy_off[t] = (int32_t)P->cy;
    P->npts += d.n;
    P->nleaves += nl;
    P->nnodes += 2 * (int64_t)nl - 1;
    P->ninternal += nl - 1;
    P->nwin += p.ncells;
    P->ncell += p.bsize > 0 ? p.ngrid : 0;
    P->ex += p.ncols;
    P->ey += p.nrows;
    P->cx += p.bsize > 0 ? p.ncols_grid : 0;
    P->cy += p.bsize > 0 ? p.nrows_grid : 0;
    if (P->classes) {
      ClassArgs& a = P->cls[t];
      std::memset(&a, 0, sizeof(a));
      a.nx = (int32_t)p.ncols;
      a.ny = (int32_t)p.nrows;
      a.tx = 2 * a.nx + 1;
      a.ty = 2 * a.ny + 1;
      if (!cls_table_geometry(bb.min_x, bb.max_x, p.displace, &a.kx0, &a.shx, &a.qx)) a.qx = 0;
      if (!cls_table_geometry(bb.min_y, bb.max_y, p.displace, &a.ky0, &a.shy, &a.qy)) a.qy = 0;
      Plan::ClsLayout& l = P->clay[t];
      auto piece = [&](size_t bytes) {
        size_t r = P->cls_misc;
        P->cls_misc += (bytes + 31) & ~(size_t)31;  // 32-byte table cells
        return r;
      };
      const size_t nx = (size_t)a.nx, ny = (size_t)a.ny, rows = nx * (size_t)a.ty;
      l.tabx = piece((size_t)a.qx * sizeof(ClsCell));
      l.taby = piece((size_t)a.qy * sizeof(ClsCell));
      l.Lx = piece(nx * 8);
      l.Rx = piece(nx * 8);
      l.Ly = piece(ny * 8);
      l.Ry = piece(ny * 8);
      l.sxl = piece(nx * 4);
      l.sxh = piece(nx * 4);
      l.syl = piece(ny * 4);
      l.syh = piece(ny * 4);
      l.rc = piece(rows * 4);
      l.rz = piece(rows * 8);
      l.ri = piece(rows * 4);
      l.sub_off = P->nsub;
      P->nsub += (int64_t)a.tx * a.ty;
      P->rows_off[t] = P->rows_total;
      P->rows_total += (int64_t)rows;
      cls_span = std::max(cls_span, std::max(std::max(a.nx, a.ny), std::max(a.qx, a.qy)));
    }
  }
  if (P->classes) {
    P->rows_off[ntiles] = P->rows_total;
    P->cls_grid_x = std::min(64, (cls_span + 255) / 256);
  }
  P->pt_off[ntiles] = P->npts;
  P->bm_off[ntiles] = P->bm_words;
  P->leaf_off[ntiles] = (int32_t)P->nleaves;
  P->node_off[ntiles] = (int32_t)P->nnodes;
  P->int_off[ntiles] = (int32_t)P->ninternal;
  P->win_off[ntiles] = P->nwin;
  P->cell_off[ntiles] = P->ncell;
  P->ex_off[ntiles] = (int32_t)P->ex;
  P->ey_off[ntiles] = (int32_t)P->ey;
  P->cx_off[ntiles] = (int32_t)P->cx;
  P->cy_off[ntiles] = (int32_t)P->cy;
  if (P->npts >= 0xFFFFFFFFLL || P->nnodes >= 0x7FFFFFFFLL) return OWM_ERANGE;
  P->idbits = std::max(1, bits_for((uint64_t)maxn + 1));
  if (P->tile_bits + P->idbits > 32) return OWM_ERANGE;  // split the batch

  size_t o = 0;
  auto take = [&](size_t bytes) {
    size_t r = o;
    o += a256(bytes);
    return r;
  };
  const int64_t N = P->npts, NW = std::max<int64_t>(P->nwin, 1), NC = std::max<int64_t>(P->ncell, 1);
  const int64_t T1 = ntiles + 1;
  P->o_xyz = take((size_t)N * 24);
  P->o_k0 = take((size_t)N * 4);
  P->o_k1 = take((size_t)N * 4);
  P->o_v0 = take((size_t)N * 4);
  P->o_v1 = take((size_t)N * 4);
  P->o_sort = take(radix_sort_temp_bytes(N));
  P->o_xk = take((size_t)N * 8);
  P->o_yk = take((size_t)N * 8);
  P->o_zk = take((size_t)N * 8);
  P->o_pid = take((size_t)N * 4);
  P->o_nodes = take((size_t)P->nnodes * sizeof(Node));
  P->o_parent = take((size_t)P->nnodes * 4);
  P->o_flags = take((size_t)std::max<int64_t>(P->ninternal, 1) * 4);
  P->o_right = take((size_t)P->nleaves * 4);
  P->o_last = take((size_t)std::max<int64_t>(P->ninternal, 1) * 4);
  P->o_edges = take((size_t)(P->ex + P->ey + P->cx + P->cy + 1) * sizeof(Edge));
  P->o_win = take((size_t)NW * 4);
  P->o_s2k0 = take((size_t)NW * 4);
  P->o_s2k1 = take((size_t)NW * 4);
  P->o_s2f = take((size_t)NW * 4);
  P->o_s2p = take((size_t)NW * 4);
  P->o_s2t = take(a256(radix_sort_temp_bytes(NW)) + scan_temp_bytes(std::max(NW, NC)) + 256);
  P->o_llp = take((size_t)NW * 4);
  if (P->s2_bitmap) {
    const int64_t BW = std::max<int64_t>(P->bm_words, 1);
    P->o_bm1 = take((size_t)BW * 4);
    P->o_bm2 = take((size_t)BW * 4);  // adjacent to o_bm1: one memset clears both
    P->o_bmc = take((size_t)BW * 4);
    P->o_bmp = take((size_t)BW * 4);
    P->o_bmt = take(scan_temp_bytes(BW) + 256);
    P->o_bmoff = take((size_t)T1 * 8);
  }
  P->o_mark = take((size_t)NC);
  P->o_cmin = take((size_t)NC * 4);
  P->o_cf = take((size_t)NC * 4);
  P->o_cp = take((size_t)NC * 4);
  P->o_ct = take(scan_temp_bytes(NC) + 256);
  P->o_s3 = take((size_t)NC * 4);
  P->o_meta = take((size_t)ntiles * sizeof(TileMeta));
  P->o_jobs1 = take((size_t)ntiles * sizeof(QueryJob));
  P->o_jobs3 = take((size_t)ntiles * sizeof(QueryJob));
  P->o_ptoff = take((size_t)T1 * 8);
  P->o_leafoff = take((size_t)T1 * 4);
  P->o_nodeoff = take((size_t)T1 * 4);
  P->o_intoff = take((size_t)T1 * 4);
  P->o_exoff = take((size_t)T1 * 4);
  P->o_eyoff = take((size_t)T1 * 4);
  P->o_cxoff = take((size_t)T1 * 4);
  P->o_cyoff = take((size_t)T1 * 4);
  P->o_winoff = take((size_t)T1 * 8);
  P->o_celloff = take((size_t)T1 * 8);
  P->o_cnt2 = take((size_t)T1 * 4);
  P->o_cnt3 = take((size_t)T1 * 4);
  P->o_llpoff = take((size_t)T1 * 4);
  P->o_s3off = take((size_t)T1 * 4);
  P->o_out = take((size_t)(NW + NC + 1) * 8);
  P->o_outoff = take((size_t)T1 * 8);
  P->o_words = take(256);
  if (P->classes) {
    P->o_cls = take((size_t)ntiles * sizeof(ClassArgs));
    P->o_rowsoff = take((size_t)T1 * 8);
    P->o_ccount = take((size_t)std::max<int64_t>(P->nsub, 1) * 4);
    P->o_czid = take((size_t)std::max<int64_t>(P->nsub, 1) * 16);
    P->o_cmisc = take(std::max<size_t>(P->cls_misc, 16));
  }
  P->total = o;
  return OWM_OK;
}

}  // namespace

int BatchRun::init(int dev, cudaStream_t s) {
  device = dev;
  OWM_CUDA_TRY(cudaSetDevice(dev));
  if (s) {
    stream = s;
  } else {
    OWM_CUDA_TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    own_stream = true;
  }
  OWM_CUDA_TRY(cudaEventCreateWithFlags(&done, cudaEventDisableTiming));
  OWM_CUDA_TRY(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
  for (cudaEvent_t* e : {&ev_fork, &ev_cls, &ev_gather, &ev_join})
    OWM_CUDA_TRY(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  return OWM_OK;
}

void BatchRun::destroy() {
  cudaSetDevice(device);
  if (stream) cudaStreamSynchronize(stream);
  if (graph) cudaGraphExecDestroy(graph);
  graph = nullptr;
  mem.release(stream);
  if (stream) cudaStreamSynchronize(stream);
  if (h_off) cudaFreeHost(h_off);
  h_off = nullptr;
  if (h_stage) cudaFreeHost(h_stage);
  h_stage = nullptr;
  stage_cap = 0;
  if (done) cudaEventDestroy(done);
  done = nullptr;
  if (side) {
    cudaStreamSynchronize(side);
    cudaStreamDestroy(side);
  }
  side = nullptr;
  for (cudaEvent_t* e : {&ev_fork, &ev_cls, &ev_gather, &ev_join}) {
    if (*e) cudaEventDestroy(*e);
    *e = nullptr;
  }
  if (own_stream && stream) cudaStreamDestroy(stream);
  stream = nullptr;
  cudaGetLastError();
}

int BatchRun::leaf_for(int64_t n, int32_t requested) const {
  for (int32_t k = 0; k < nclass; ++k)
    if (n <= class_bound[k]) return class_leaf[k];
  return requested;
}

size_t BatchRun::estimate_bytes(const owm_tile_desc* t, int32_t ntiles) {
  BatchRun tmp;
  Plan P;
  if (make_plan(t, ntiles, tmp, &P) != OWM_OK) return (size_t)-1;
  return P.total;
}

int BatchRun::launch(const owm_tile_desc* td, int32_t ntiles) {
  if (!td || ntiles <= 0) return OWM_EINVAL;
  OWM_CUDA_TRY(cudaSetDevice(device));
  Plan P;
  int rc = make_plan(td, ntiles, *this, &P);
  if (rc) return rc;
  bytes_needed = P.total;
  if (P.total > mem.cap && graph) {  // buffers move: the captured graph is stale
    cudaGraphExecDestroy(graph);
    graph = nullptr;
    graph_sig.clear();
  }
  rc = mem.reserve(P.total, stream);
  if (rc) return rc;
  if (cap_tiles < ntiles + 1) {
    if (h_off) cudaFreeHost(h_off);
    h_off = nullptr;
    OWM_CUDA_TRY(cudaMallocHost(&h_off, (size_t)(ntiles + 2) * 8));  // + the status word
    cap_tiles = ntiles + 1;
  }
  // Per-batch tables go through pinned staging: a copy from pageable memory
  // would first wait for this stream's queued point copies, holding the
  // caller (the server's worker) for the whole transfer.
  const size_t T1 = (size_t)ntiles + 1;
  const size_t stage_need = 20 * 16 + (size_t)ntiles * (sizeof(TileMeta) + 2 * sizeof(QueryJob) + sizeof(ClassArgs)) +
                            T1 * (8 * 5 + 4 * 7);
  if (stage_cap < stage_need) {
    if (h_stage) cudaFreeHost(h_stage);
    h_stage = nullptr;
    OWM_CUDA_TRY(cudaMallocHost(&h_stage, stage_need));
    stage_cap = stage_need;
  }
  size_t stage_off = 0;
  auto stage_copy = [&](void* dst, const void* src, size_t bytes) -> cudaError_t {
    char* h = h_stage + stage_off;
    stage_off += (bytes + 15) & ~(size_t)15;
    std::memcpy(h, src, bytes);
    return cudaMemcpyAsync(dst, h, bytes, cudaMemcpyHostToDevice, stream);
  };
  tiles.clear();
  char* B = static_cast<char*>(mem.ptr);
  auto at = [&](size_t off) { return B + off; };
  double* xyz = (double*)at(P.o_xyz);
  const int64_t N = P.npts;
  // tiles already back to back in one device buffer are used in place
  // (on this device: the kernels read them directly)
  bool in_place = device_ptr_on(td[0].xyz, device);
  for (int32_t t = 1; t < ntiles && in_place; ++t) in_place = td[t].xyz == td[0].xyz + 3 * P.pt_off[t];
  if (in_place) xyz = const_cast<double*>(td[0].xyz);
  // points in (host or device sources)
  for (int32_t t = 0; t < ntiles; ++t) {
    if (!in_place)
      OWM_CUDA_TRY(cudaMemcpyAsync(xyz + 3 * P.pt_off[t], td[t].xyz, (size_t)td[t].n * 24, cudaMemcpyDefault, stream));
    TileHost th;
    th.xyz = td[t].xyz;
    owm_bbox bb = td[t].bbox;
    if (!(bb.min_x <= bb.max_x)) owm_bbox_of(td[t].xyz, td[t].n, &bb);
    owm_params_compute(&bb, td[t].n, td[t].cfg.wsize, td[t].cfg.overlap, td[t].cfg.bsize, &th.p);
    th.tree = td[t].cfg.tree;
    tiles.push_back(th);
  }
  TileMeta* d_meta = (TileMeta*)at(P.o_meta);
  int64_t* d_ptoff = (int64_t*)at(P.o_ptoff);
  int32_t* d_leafoff = (int32_t*)at(P.o_leafoff);
  int32_t* d_nodeoff = (int32_t*)at(P.o_nodeoff);
  int32_t* d_intoff = (int32_t*)at(P.o_intoff);
  int32_t* d_exoff = (int32_t*)at(P.o_exoff);
  int32_t* d_eyoff = (int32_t*)at(P.o_eyoff);
  int32_t* d_cxoff = (int32_t*)at(P.o_cxoff);
  int32_t* d_cyoff = (int32_t*)at(P.o_cyoff);
  int64_t* d_winoff = (int64_t*)at(P.o_winoff);
  int64_t* d_celloff = (int64_t*)at(P.o_celloff);
  OWM_CUDA_TRY(stage_copy(d_meta, P.meta.data(), (size_t)ntiles * sizeof(TileMeta)));
  OWM_CUDA_TRY(stage_copy(d_ptoff, P.pt_off.data(), T1 * 8));
  OWM_CUDA_TRY(stage_copy(d_leafoff, P.leaf_off.data(), T1 * 4));
  OWM_CUDA_TRY(stage_copy(d_nodeoff, P.node_off.data(), T1 * 4));
  OWM_CUDA_TRY(stage_copy(d_intoff, P.int_off.data(), T1 * 4));
  OWM_CUDA_TRY(stage_copy(d_exoff, P.ex_off.data(), T1 * 4));
  OWM_CUDA_TRY(stage_copy(d_eyoff, P.ey_off.data(), T1 * 4));
  OWM_CUDA_TRY(stage_copy(d_cxoff, P.cx_off.data(), T1 * 4));
  OWM_CUDA_TRY(stage_copy(d_cyoff, P.cy_off.data(), T1 * 4));
  OWM_CUDA_TRY(stage_copy(d_winoff, P.win_off.data(), T1 * 8));
  OWM_CUDA_TRY(stage_copy(d_celloff, P.cell_off.data(), T1 * 8));
  int64_t* d_bmoff = P.s2_bitmap ? (int64_t*)at(P.o_bmoff) : nullptr;
  if (P.s2_bitmap) OWM_CUDA_TRY(stage_copy(d_bmoff, P.bm_off.data(), T1 * 8));

  // query jobs (host-built: pointers are known here)
  TreeView base_view;
  int64_t* xk = (int64_t*)at(P.o_xk);
  int64_t* yk = (int64_t*)at(P.o_yk);
  int64_t* zk = (int64_t*)at(P.o_zk);
  uint32_t* pid = (uint32_t*)at(P.o_pid);
  Node* nodes = (Node*)at(P.o_nodes);
  Edge* edges = (Edge*)at(P.o_edges);
  Edge* E_wx = edges;
  Edge* E_wy = E_wx + P.ex;
  Edge* E_cx = E_wy + P.ey;
  Edge* E_cy = E_cx + P.cx;
  uint32_t* win = (uint32_t*)at(P.o_win);
  uint8_t* mark = (uint8_t*)at(P.o_mark);
  uint32_t* cmin = (uint32_t*)at(P.o_cmin);
  uint32_t* words = (uint32_t*)at(P.o_words);
  d_status = words;  // [0] status, [1] LLP total, [2] s3 total, [4..5] queue counter (8-byte aligned)
  unsigned long long* qnext = reinterpret_cast<unsigned long long*>(words + 4);
  std::vector<QueryJob> j1(ntiles), j3(ntiles);
  int64_t w1 = 0, w3 = 0;
  for (int32_t t = 0; t < ntiles; ++t) {
    const TileMeta& m = P.meta[t];
    TreeView v;
    v.xk = xk + m.pt_off;
    v.yk = yk + m.pt_off;
    v.zk = zk + m.pt_off;
    v.pid = pid + m.pt_off;
    v.nodes = nodes + m.node_off;
    v.nleaves = m.nleaves;
    v.root = 0;
    v.ox = m.ox;
    v.oy = m.oy;
    QueryJob& a = j1[t];
    a.tree = v;
    a.ex = E_wx + m.ex_off;
    a.ey = E_wy + m.ey_off;
    a.ncols = m.ncols;
    a.nrows = m.nrows;
    a.thr = m.thr;
    a.cell_order = 0;
    a.patch_lx = patch_log2(tuning.walk_patch_x);
    a.skip = nullptr;
    a.out = win + m.win_off;
    a.status = words;
    a.warp_begin = w1;
    w1 += job_warps(m.ncols, m.nrows, a.patch_lx);
    QueryJob& b = j3[t];
    b = a;
    b.ex = E_cx + m.cx_off;
    b.ey = E_cy + m.cy_off;
    b.ncols = m.bsize > 0 ? m.ncg : 0;
    b.nrows = m.bsize > 0 ? m.nrg : 0;
    b.thr = 1;
    b.cell_order = 1;
    b.skip = mark + m.cell_off;
    b.out = cmin + m.cell_off;
    b.warp_begin = w3;
    w3 += job_warps(b.ncols, b.nrows, b.patch_lx);
  }
  (void)base_view;
  QueryJob* d_j1 = (QueryJob*)at(P.o_jobs1);
  QueryJob* d_j3 = (QueryJob*)at(P.o_jobs3);
  OWM_CUDA_TRY(stage_copy(d_j1, j1.data(), (size_t)ntiles * sizeof(QueryJob)));
  OWM_CUDA_TRY(stage_copy(d_j3, j3.data(), (size_t)ntiles * sizeof(QueryJob)));
  ClassArgs* d_cls = nullptr;
  int64_t* d_rowsoff = nullptr;
  if (P.classes) {
    std::vector<ClassArgs> A(P.cls);
    char* misc = at(P.o_cmisc);
    for (int32_t t = 0; t < ntiles; ++t) {
      const Plan::ClsLayout& l = P.clay[t];
      ClassArgs& a = A[t];
      a.tabx = reinterpret_cast<const ClsCell*>(misc + l.tabx);
      a.taby = reinterpret_cast<const ClsCell*>(misc + l.taby);
      a.Lx = reinterpret_cast<const int64_t*>(misc + l.Lx);
      a.Rx = reinterpret_cast<const int64_t*>(misc + l.Rx);
      a.Ly = reinterpret_cast<const int64_t*>(misc + l.Ly);
      a.Ry = reinterpret_cast<const int64_t*>(misc + l.Ry);
      a.sxl = reinterpret_cast<int32_t*>(misc + l.sxl);
      a.sxh = reinterpret_cast<int32_t*>(misc + l.sxh);
      a.syl = reinterpret_cast<int32_t*>(misc + l.syl);
      a.syh = reinterpret_cast<int32_t*>(misc + l.syh);
      a.rc = reinterpret_cast<uint32_t*>(misc + l.rc);
      a.rz = reinterpret_cast<unsigned long long*>(misc + l.rz);
      a.ri = reinterpret_cast<uint32_t*>(misc + l.ri);
      a.count = reinterpret_cast<uint32_t*>(at(P.o_ccount)) + l.sub_off;
      a.zid = reinterpret_cast<ulonglong2*>(at(P.o_czid)) + l.sub_off;
    }
    d_cls = reinterpret_cast<ClassArgs*>(at(P.o_cls));
    d_rowsoff = reinterpret_cast<int64_t*>(at(P.o_rowsoff));
    OWM_CUDA_TRY(stage_copy(d_cls, A.data(), (size_t)ntiles * sizeof(ClassArgs)));
    OWM_CUDA_TRY(stage_copy(d_rowsoff, P.rows_off.data(), T1 * 8));
  }

  int64_t* d_out = (int64_t*)at(P.o_out);
  int64_t* d_outoff = (int64_t*)at(P.o_outoff);
  this->d_out = d_out;
  this->d_out_off = d_outoff;

  // ---- device work (graph-capturable: no host sync, fixed shapes) ----
  std::string sig;
  if (use_graphs) {
    sig.assign(reinterpret_cast<const char*>(P.meta.data()), P.meta.size() * sizeof(TileMeta));
    sig.append(reinterpret_cast<const char*>(&mem.ptr), sizeof(void*));
    sig.append(reinterpret_cast<const char*>(&xyz), sizeof(void*));
    sig.append(reinterpret_cast<const char*>(&P.total), sizeof(P.total));
    // the class regions' layout (table sizes follow each tile's bbox, not only its meta)
    if (P.classes) sig.append(reinterpret_cast<const char*>(P.cls.data()), P.cls.size() * sizeof(ClassArgs));
    sig.push_back(P.classes ? 'c' : 'w');
    sig.append(reinterpret_cast<const char*>(&tuning), sizeof(tuning));  // launch shapes
  }
  if (use_graphs && graph && sig == graph_sig) {
    OWM_CUDA_TRY(cudaGraphLaunch(graph, stream));
    count_launch(&launches);
  } else {
    bool capture = use_graphs;
    ProfScope no_prof(capture ? nullptr : tls_profiler());
    if (capture) OWM_CUDA_TRY(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    cudaStream_t s = stream;
    int64_t* L = &launches;
    uint32_t* k0 = (uint32_t*)at(P.o_k0);
    uint32_t* k1 = (uint32_t*)at(P.o_k1);
    uint32_t* v0 = (uint32_t*)at(P.o_v0);
    uint32_t* v1 = (uint32_t*)at(P.o_v1);
    int32_t* parent = (int32_t*)at(P.o_parent);
    int32_t* flags = (int32_t*)at(P.o_flags);
    int32_t* right_of = (int32_t*)at(P.o_right);
    int32_t* last_of = (int32_t*)at(P.o_last);
    uint32_t* cnt2 = (uint32_t*)at(P.o_cnt2);
    uint32_t* cnt3 = (uint32_t*)at(P.o_cnt3);
    uint32_t* llp_off = (uint32_t*)at(P.o_llpoff);
    uint32_t* s3_off = (uint32_t*)at(P.o_s3off);
    uint32_t* llp = (uint32_t*)at(P.o_llp);
    uint32_t* s3 = (uint32_t*)at(P.o_s3);
    int rc2 = OWM_OK;
    // side-stream schedule (stage 1 by classes): ss forks from s, prepares the
    // tables while s sorts, and finishes stages 1-2 and the LLP marks while s
    // builds the hierarchies; without classes everything runs on s
    const bool two = P.classes && side != nullptr;
    cudaStream_t ss = two ? side : s;
    bool forked = false;
    const int64_t NW = P.nwin;
    const int64_t NC = P.ncell;
    do {
      if (cudaMemsetAsync(words, 0, 256, s) != cudaSuccess) { rc2 = OWM_ECUDA; break; }
      if (two) {
        if (cudaEventRecord(ev_fork, s) != cudaSuccess || cudaStreamWaitEvent(ss, ev_fork, 0) != cudaSuccess) {
          rc2 = OWM_ECUDA;
          break;
        }
        forked = true;
      }
      // edge tables (before the gather: the class fold needs the window edges)
      if (P.ex) OWM_LAUNCH("k_b_edges", ss, k_b_edges<<<(unsigned)((P.ex + 127) / 128), 128, 0, ss>>>(0, 0, d_meta, d_exoff, ntiles, P.ex, E_wx));
      if (P.ey) OWM_LAUNCH("k_b_edges", ss, k_b_edges<<<(unsigned)((P.ey + 127) / 128), 128, 0, ss>>>(0, 1, d_meta, d_eyoff, ntiles, P.ey, E_wy));
      if (P.cx) OWM_LAUNCH("k_b_edges", ss, k_b_edges<<<(unsigned)((P.cx + 127) / 128), 128, 0, ss>>>(1, 0, d_meta, d_cxoff, ntiles, P.cx, E_cx));
      if (P.cy) OWM_LAUNCH("k_b_edges", ss, k_b_edges<<<(unsigned)((P.cy + 127) / 128), 128, 0, ss>>>(1, 1, d_meta, d_cyoff, ntiles, P.cy, E_cy));
      count_launch(L, (P.ex > 0) + (P.ey > 0) + (P.cx > 0) + (P.cy > 0));
      if (P.classes) {
        const dim3 gp((unsigned)P.cls_grid_x, (unsigned)ntiles);
        OWM_LAUNCH("k_bc_split", ss, k_bc_split<<<gp, 256, 0, ss>>>(d_cls, d_meta, E_wx, E_wy));
        OWM_LAUNCH("k_bc_prep", ss, k_bc_prep<<<gp, 256, 0, ss>>>(d_cls));
        count_launch(L, 2);
        if (cudaMemsetAsync(at(P.o_ccount), 0, (size_t)P.nsub * 4, ss) != cudaSuccess ||
            cudaMemsetAsync(at(P.o_czid), 0xFF, (size_t)P.nsub * 16, ss) != cudaSuccess) {
          rc2 = OWM_ECUDA;
          break;
        }
      }
      // stage 2/3 buffers cleared ahead of time
      if (cudaMemsetAsync(cnt2, 0, T1 * 4, ss) != cudaSuccess || cudaMemsetAsync(cnt3, 0, T1 * 4, ss) != cudaSuccess) {
        rc2 = OWM_ECUDA;
        break;
      }
      if (NW > 0 && P.s2_bitmap &&
          cudaMemsetAsync(at(P.o_bm1), 0, (size_t)(P.o_bm2 - P.o_bm1) + (size_t)P.bm_words * 4, ss) != cudaSuccess) {
        rc2 = OWM_ECUDA;
        break;
      }
      if (NC > 0 && cudaMemsetAsync(mark, 0, (size_t)NC, ss) != cudaSuccess) { rc2 = OWM_ECUDA; break; }
      if (two && cudaEventRecord(ev_cls, ss) != cudaSuccess) { rc2 = OWM_ECUDA; break; }

      const int key_bits = P.tile_bits + 2 * P.mbits;
      const RadixSortPlan sp = radix_sort_plan(N);
      if (sp.parts) {  // the Morton pass also counts the sort's first digit
        OWM_LAUNCH("k_b_morton", s, k_b_morton_counts<<<(unsigned)sp.parts, 256, 0, s>>>(
            xyz, N, d_ptoff, d_meta, ntiles, P.mbits, sp.ntiles, (1u << radix_digit_bits(key_bits, 0, radix_ranked_widths(N, key_bits))) - 1u, k0,
            (uint32_t*)at(P.o_sort)));
      } else {
        OWM_LAUNCH("k_b_morton", s, k_b_morton<<<gsz(N), 256, 0, s>>>(xyz, N, d_ptoff, d_meta, ntiles, P.mbits, k0));
      }
      count_launch(L);
      bool alt = false;
      if (radix_sort(k0, v0, k1, v1, N, key_bits, true, at(P.o_sort), radix_sort_temp_bytes(N), s, &alt, L,
                     sp.parts > 0) != cudaSuccess) { rc2 = OWM_ECUDA; break; }
      const uint32_t* mk = alt ? k1 : k0;
      const uint32_t* perm = alt ? v1 : v0;
      if (two && cudaStreamWaitEvent(s, ev_cls, 0) != cudaSuccess) { rc2 = OWM_ECUDA; break; }
      {
        // one warp per leaf: resident warps then work on neighbouring leaves
        const int gb = tuning.gather_block;
        int64_t blocks = std::min<int64_t>((P.nleaves * 32 + gb - 1) / gb, (int64_t)152 * 1024 * 256 / gb);
        OWM_LAUNCH("k_b_gather_leaves", s, k_b_gather_leaves<<<(unsigned)std::max<int64_t>(blocks, 1), gb, 0, s>>>(
            xyz, perm, d_meta, d_leafoff, ntiles, P.nleaves, xk, yk, zk, pid, nodes, words, d_cls));
        count_launch(L);
      }
      if (two && (cudaEventRecord(ev_gather, s) != cudaSuccess || cudaStreamWaitEvent(ss, ev_gather, 0) != cudaSuccess)) {
        rc2 = OWM_ECUDA;
        break;
      }
      // stage 1: window classes (rows, windows) on ss, or the persistent walk
      // (on s, after the hierarchies, below)
      if (P.classes) {
        if (P.rows_total > 0) {
          OWM_LAUNCH("k_bc_rows", ss, k_bc_rows<<<gsz(P.rows_total), 256, 0, ss>>>(d_cls, d_rowsoff, ntiles, P.rows_total));
          count_launch(L);
        }
        if (NW > 0) {
          OWM_LAUNCH("k_bc_windows", ss, k_bc_windows<<<gsz(NW), 256, 0, ss>>>(d_cls, d_meta, d_winoff, ntiles, NW, win));
          count_launch(L);
        }
      }
      // hierarchies on s
      if (P.ninternal > 0) {
        uint32_t* lk = alt ? k0 : k1;  // the sort's other key buffer is free now
        OWM_LAUNCH("k_b_leaf_keys", s, k_b_leaf_keys<<<(unsigned)((P.nleaves + 255) / 256), 256, 0, s>>>(
            mk, d_meta, d_leafoff, ntiles, P.nleaves, lk));
        OWM_LAUNCH("k_b_karras", s, k_b_karras<<<(unsigned)((P.ninternal + 255) / 256), 256, 0, s>>>(
            lk, d_meta, d_intoff, ntiles, P.ninternal, nodes, parent, right_of, last_of, flags));
        count_launch(L, 2);
      }
      OWM_LAUNCH("k_b_refit", s, k_b_refit<<<(unsigned)((P.nleaves + 255) / 256), 256, 0, s>>>(
          nodes, parent, flags, right_of, last_of, d_meta, d_leafoff, ntiles, P.nleaves));
      count_launch(L);
      if (!P.classes && launch_query_persistent(d_j1, ntiles, w1, qnext, 152 * 16, s, L, "k_query_s1_batch")) {
        rc2 = OWM_ECUDA;
        break;
      }
      // stage 2 on (tile, id) keys, on ss
      const uint32_t none = (P.idbits >= 32) ? 0xFFFFFFFFu : ((1u << P.idbits) - 1u);
      uint32_t* s2k0 = (uint32_t*)at(P.o_s2k0);
      uint32_t* s2k1 = (uint32_t*)at(P.o_s2k1);
      uint32_t* s2f = (uint32_t*)at(P.o_s2f);
      uint32_t* s2p = (uint32_t*)at(P.o_s2p);
      char* s2t = at(P.o_s2t);
      if (NW > 0 && P.s2_bitmap) {
        const int64_t BW = P.bm_words;
        uint32_t* bm1 = (uint32_t*)at(P.o_bm1);
        uint32_t* bm2 = (uint32_t*)at(P.o_bm2);
        uint32_t* bmc = (uint32_t*)at(P.o_bmc);
        uint32_t* bmp = (uint32_t*)at(P.o_bmp);
        OWM_LAUNCH("k_b_s2_mark", ss, k_b_s2_mark<<<gsz(NW), 256, 0, ss>>>(win, NW, d_winoff, ntiles, d_meta, bm1, bm2));
        OWM_LAUNCH("k_b_s2_popc", ss, k_b_s2_popc<<<gsz(BW), 256, 0, ss>>>(bm2, BW, bmc));
        count_launch(L, 2);
        if (exclusive_scan_u32(bmc, bmp, BW, words + 1, at(P.o_bmt), scan_temp_bytes(BW) + 256, ss, L) != cudaSuccess) {
          rc2 = OWM_ECUDA;
          break;
        }
        OWM_LAUNCH("k_b_s2_emit", ss, k_b_s2_emit<<<gsz(BW), 256, 0, ss>>>(bm2, bmp, BW, d_bmoff, ntiles, P.idbits, llp));
        OWM_LAUNCH("k_b_s2_tilecount", ss, k_b_s2_tilecount<<<(ntiles + 255) / 256, 256, 0, ss>>>(bmp, d_bmoff, ntiles, BW,
                                                                                               words + 1, cnt2));
        count_launch(L, 2);
      } else if (NW > 0) {
        OWM_LAUNCH("k_b_s2_keys", ss, k_b_s2_keys<<<gsz(NW), 256, 0, ss>>>(win, NW, d_winoff, ntiles, P.idbits, none, s2k0));
        count_launch(L);
        bool a2 = false;
        size_t sb = radix_sort_temp_bytes(NW);
        if (radix_sort(s2k0, nullptr, s2k1, nullptr, NW, P.tile_bits + P.idbits, false, s2t, sb, ss, &a2, L) !=
            cudaSuccess) { rc2 = OWM_ECUDA; break; }
        const uint32_t* sk = a2 ? s2k1 : s2k0;
        OWM_LAUNCH("k_b_s2_flags", ss, k_b_s2_flags<<<gsz(NW), 256, 0, ss>>>(sk, NW, P.idbits, none, d_meta, s2f, cnt2));
        count_launch(L);
        if (exclusive_scan_u32(s2f, s2p, NW, words + 1, s2t + a256(sb), scan_temp_bytes(std::max<int64_t>(NW, P.ncell)) + 256,
                               ss, L) != cudaSuccess) { rc2 = OWM_ECUDA; break; }
        OWM_LAUNCH("k_b_compact", ss, k_b_compact<<<gsz(NW), 256, 0, ss>>>(sk, s2f, s2p, NW, llp));
        count_launch(L);
      }
      if (exclusive_scan_u32(cnt2, llp_off, ntiles + 1, nullptr, s2t, scan_temp_bytes(ntiles + 1) + 256, ss, L) !=
          cudaSuccess) { rc2 = OWM_ECUDA; break; }
      // stage 3: LLP marks on ss; queries on s once both streams are done
      if (NC > 0 && NW > 0) {
        OWM_LAUNCH("k_b_s3_mark", ss, k_b_s3_mark<<<gsz(NW), 256, 0, ss>>>(xyz, llp, words + 1, NW, P.idbits, d_meta, E_cx, E_cy, mark));
        count_launch(L);
      }
      if (two) {
        if (cudaEventRecord(ev_join, ss) != cudaSuccess || cudaStreamWaitEvent(s, ev_join, 0) != cudaSuccess) {
          rc2 = OWM_ECUDA;
          break;
        }
        forked = false;
      }
      if (NC > 0) {
        if ((NC + 1) / 2 >= 0x7FFFFFFFll) { rc2 = OWM_ERANGE; break; }
        const cudaError_t e3 = tuning.cell_warps == 2   ? launch_b_query_cells<2>(d_j3, d_celloff, ntiles, NC, s)
                               : tuning.cell_warps == 8 ? launch_b_query_cells<8>(d_j3, d_celloff, ntiles, NC, s)
                                                        : launch_b_query_cells<4>(d_j3, d_celloff, ntiles, NC, s);
        if (e3 != cudaSuccess) { rc2 = OWM_ECUDA; break; }
        count_launch(L);
        uint32_t* cf = (uint32_t*)at(P.o_cf);
        uint32_t* cp = (uint32_t*)at(P.o_cp);
        OWM_LAUNCH("k_b_flag_cells", s, k_b_flag_cells<<<gsz(NC), 256, 0, s>>>(cmin, NC, d_celloff, ntiles, cf, cnt3));
        count_launch(L);
        if (exclusive_scan_u32(cf, cp, NC, words + 2, at(P.o_ct), scan_temp_bytes(NC) + 256, s, L) != cudaSuccess) {
          rc2 = OWM_ECUDA;
          break;
        }
        OWM_LAUNCH("k_b_compact", s, k_b_compact<<<gsz(NC), 256, 0, s>>>(cmin, cf, cp, NC, s3));
        count_launch(L);
      }
      if (exclusive_scan_u32(cnt3, s3_off, ntiles + 1, nullptr, at(P.o_ct), scan_temp_bytes(ntiles + 1) + 256, s, L) !=
          cudaSuccess) { rc2 = OWM_ECUDA; break; }
      OWM_LAUNCH("k_b_assemble", s, k_b_assemble<<<gsz(NW + NC + ntiles + 1), 256, 0, s>>>(s3, s3_off, llp, llp_off, P.idbits, ntiles, d_out, d_outoff));
      count_launch(L);
      if (cudaMemcpyAsync(h_off, d_outoff, T1 * 8, cudaMemcpyDeviceToHost, s) != cudaSuccess) { rc2 = OWM_ECUDA; break; }
      if (cudaMemcpyAsync(h_off + T1, words, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess) { rc2 = OWM_ECUDA; break; }
    } while (false);
    if (forked) {  // an error left the side stream forked: join it (a capture must end joined)
      cudaEventRecord(ev_join, ss);
      cudaStreamWaitEvent(s, ev_join, 0);
    }
    if (capture) {
      cudaGraph_t g = nullptr;
      cudaError_t e = cudaStreamEndCapture(stream, &g);
      if (rc2 == OWM_OK && e == cudaSuccess) {
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
        e = cudaGraphInstantiate(&graph, g, 0);
        if (e == cudaSuccess) {
          graph_sig = sig;
          e = cudaGraphLaunch(graph, stream);
          count_launch(&launches);
        }
      }
      if (g) cudaGraphDestroy(g);
      if (e != cudaSuccess) {
        set_last_cuda_error(e, "batch graph", __FILE__, __LINE__);
        return OWM_ECUDA;
      }
    }
    if (rc2) return rc2;
  }
  OWM_CUDA_TRY(cudaEventRecord(done, stream));
  return OWM_OK;
}

bool BatchRun::ready() {
  cudaError_t e = cudaEventQuery(done);
  if (e == cudaErrorNotReady) return false;
  cudaGetLastError();
  return true;
}

int BatchRun::finish(int64_t* seeds, int64_t cap, int64_t* offsets, owm_run_info* info) {
  OWM_CUDA_TRY(cudaSetDevice(device));
  OWM_CUDA_TRY(cudaEventSynchronize(done));
  const int64_t nt = (int64_t)tiles.size();
  uint32_t st = 0;
  std::memcpy(&st, h_off + nt + 1, 4);  // read back with the offsets at the end of the batch
  if (st & kStatusNonFinite) return OWM_EINVAL;
  if (st & kStatusWalkBound) return OWM_ETIMEOUT;
  total_out = h_off[nt];
  if (offsets) std::memcpy(offsets, h_off, (size_t)(nt + 1) * 8);
  if (info) {
    std::memset(info, 0, sizeof(*info));
    info->n_seeds = total_out;
  }
  if (total_out > cap) return OWM_ERANGE;
  if (total_out > 0 && seeds) {
    OWM_CUDA_TRY(cudaMemcpyAsync(seeds, d_out, (size_t)total_out * 8, cudaMemcpyDefault, stream));
    OWM_CUDA_TRY(cudaStreamSynchronize(stream));
  }
  return OWM_OK;
}

}  // namespace owm

using namespace owm;

struct owm_batch {
  owm_ctx* ctx;  // used only inside owm_batch_run (profiler, launch count)
  BatchRun run;
};

extern "C" {

int owm_batch_create(owm_ctx* ctx, owm_batch** out) {
  if (!ctx || !out) return OWM_EINVAL;
  owm_batch* b = new owm_batch();
  b->ctx = ctx;
  // own stream: the batch may outlive nothing of its context but the device
  int rc = b->run.init(ctx->device, nullptr);
  if (rc) {
    delete b;
    return rc;
  }
  *out = b;
  return OWM_OK;
}

int owm_batch_destroy(owm_batch* b) {
  if (!b) return OWM_OK;
  b->run.destroy();
  delete b;
  return OWM_OK;
}

int owm_batch_set_graphs(owm_batch* b, int enable) {
  if (!b) return OWM_EINVAL;
  b->run.use_graphs = enable != 0;
  return OWM_OK;
}

int owm_batch_set_leaf_classes(owm_batch* b, int32_t nclass, const int64_t* bounds, const int32_t* leaf) {
  if (!b || nclass < 0 || nclass > 8 || (nclass > 0 && (!bounds || !leaf))) return OWM_EINVAL;
  for (int32_t k = 0; k < nclass; ++k) {
    int m = leaf[k];
    if (m < 1 || m > 256 || (m & (m - 1))) return OWM_EINVAL;
    if (k > 0 && bounds[k] <= bounds[k - 1]) return OWM_EINVAL;
  }
  b->run.nclass = nclass;
  for (int32_t k = 0; k < nclass; ++k) {
    b->run.class_bound[k] = bounds[k];
    b->run.class_leaf[k] = leaf[k];
  }
  if (b->run.graph) {
    cudaGraphExecDestroy(b->run.graph);
    b->run.graph = nullptr;
    b->run.graph_sig.clear();
  }
  return OWM_OK;
}

int owm_batch_run(owm_batch* b, const owm_tile_desc* tiles, int32_t ntiles, int64_t* seeds, int64_t cap,
                  int64_t* offsets, owm_run_info* info) {
  if (!b || !tiles || ntiles <= 0 || !offsets || (!seeds && cap > 0)) return OWM_EINVAL;
  ProfScope prof_scope(b->ctx->active_prof());
  b->run.tuning = b->ctx->tuning;
  int64_t l0 = b->run.launches;
  int rc = b->run.launch(tiles, ntiles);
  if (rc) return rc;
  rc = b->run.finish(seeds, cap, offsets, info);
  b->ctx->launches += b->run.launches - l0;
  return rc;
}

}  // extern "C"
