// OWM stages on the device.
//
// Stage 1 / stage 3 boxes (reference: stage1, optim3_func.cpp:541-561, and
// stage3, :627-662) are answered by one traversal kernel:
//   * one thread owns one box; a warp owns a 4 x 8 patch of neighbouring
//     boxes, so its lanes walk nearly the same nodes (broadcast loads);
//   * the walk is stackless (escape links) and runs in two phases:
//       A  nodes strictly inside the box give their memoised count and
//          (z, id)-min at once (the reference's O3 memo); partial leaves are
//          left for later;
//       B  partial nodes are revisited only while they can still matter:
//          once the count reached the threshold, a node whose memoised min is
//          not below the current best is skipped (min-z pruning); a partial
//          leaf whose min point lies inside the box needs no scan for the
//          min (optim3_func.cpp:437-445);
//   * remaining leaf scans are done by the whole warp together: 32 lanes
//     test 32 points of one lane's leaf and a shuffle reduction hands the
//     count and the (z, id)-min back to the owner.
// Stage 3 of one cloud (threshold 1, few cells left after the LLP marks) is
// answered by one warp per cell instead (k_query_cells).
// All point tests are strict and run on exact int64 keys of the FP64
// coordinates; node tests run on outward-rounded float boxes and only decide
// "inside"/"outside" when that is certain.
//
// Stage 2 (owm_optim3.cpp:160,173; optim3_func.cpp:610-625): radix sort of
// the window results, then ids with run length >= 2, ascending; for one cloud
// with overlap > 0 occupancy bitmaps give the same list without the sort.
#include <cuda_runtime.h>

#include <algorithm>

#include "owm_query.cuh"
#include "owm_cellq.cuh"

namespace owm {

namespace {

constexpr int kQBlock = 128;

__device__ __forceinline__ Edge make_edge(double lo, double hi, double o) {
  Edge e;
  e.lo_k = dkey(lo);
  e.hi_k = dkey(hi);
  e.lo_dn = __double2float_rd(__dsub_rd(lo, o));
  e.lo_up = __double2float_ru(__dsub_ru(lo, o));
  e.hi_dn = __double2float_rd(__dsub_rd(hi, o));
  e.hi_up = __double2float_ru(__dsub_ru(hi, o));
  return e;
}

// Stage-1 windows (optim3_func.cpp:544-555, makeBox :318-324):
//   init = (min - (double)(Wsize/2)) + Displace;  c = init + i*Displace;
//   box  = c -/+ (double)(float)(Wsize/2)
// Stage-3 cells (optim3_func.cpp:630-651, makeBox :310-316):
//   init = min + (double)(Bsize/2);  c = init + (double)(i*Bsize);
//   box  = c -/+ (double)(float)(Bsize/2)
// Every operation is a separately rounded IEEE op (no contraction).
__global__ void k_edges(double min_x, double min_y, double step, int32_t half, int cells, int32_t ncols,
                        int32_t nrows, int32_t bsize, double ox, double oy, Edge* __restrict__ ex,
                        Edge* __restrict__ ey) {
  int32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  double r = (double)(float)half;
  if (t < ncols) {
    double c;
    if (cells) {
      double init = __dadd_rn(min_x, (double)half);
      c = __dadd_rn(init, (double)(t * bsize));
    } else {
      double init = __dadd_rn(__dsub_rn(min_x, (double)half), step);
      c = __dadd_rn(init, __dmul_rn((double)t, step));
    }
    ex[t] = make_edge(__dsub_rn(c, r), __dadd_rn(c, r), ox);
  }
  if (t < nrows) {
    double c;
    if (cells) {
      double init = __dadd_rn(min_y, (double)half);
      c = __dadd_rn(init, (double)(t * bsize));
    } else {
      double init = __dadd_rn(__dsub_rn(min_y, (double)half), step);
      c = __dadd_rn(init, __dmul_rn((double)t, step));
    }
    ey[t] = make_edge(__dsub_rn(c, r), __dadd_rn(c, r), oy);
  }
}

__device__ __forceinline__ int find_job(const QueryJob* __restrict__ jobs, int32_t njobs, int64_t warp) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(&jobs[mid].warp_begin) <= warp) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ int64_t shfl64(int64_t v, int src) { return __shfl_sync(0xffffffffu, v, src); }

// One warp answers the 4 x 8 patch `warp` of the job list (all 32 lanes call
// this together).
__device__ __forceinline__ void query_warp(const QueryJob* __restrict__ jobs, int32_t njobs, int64_t warp,
                                           int lane) {
  const QueryJob& J = jobs[njobs > 1 ? find_job(jobs, njobs, warp) : 0];
  const TreeView T = J.tree;
  const int64_t lw = warp - J.warp_begin;
  const int32_t lx = J.patch_lx;  // patch of 2^lx columns x 2^(5 - lx) rows of windows
  const int32_t gx = (J.ncols + (1 << lx) - 1) >> lx;
  const int32_t ii = (int32_t)(lw % gx) * (1 << lx) + (lane & ((1 << lx) - 1));
  const int32_t jj = (int32_t)(lw / gx) * (32 >> lx) + (lane >> lx);
  bool active = ii < J.ncols && jj < J.nrows;
  int64_t oidx = 0;
  Edge ex, ey;
  if (active) {
    oidx = J.cell_order ? (int64_t)jj * J.ncols + ii : (int64_t)ii * J.nrows + jj;
    ex = J.ex[ii];
    ey = J.ey[jj];
    if (J.skip && J.skip[oidx]) {
      J.out[oidx] = kNone;
      active = false;
    }
  } else {
    ex.lo_k = ex.hi_k = ey.lo_k = ey.hi_k = 0;
  }
  const uint32_t thr = J.thr;
  const int32_t first_leaf = T.nleaves - 1;
  int64_t bz = kZSentinel;
  uint32_t bid = 0, cnt = 0;
  int phase = 0;
  int32_t nodei = active ? T.root : kEnd;
  bool done = !active;
  int32_t scan_leaf = -1;
  // A well-formed depth-first walk visits each node at most once per phase;
  // the bound only guards against a corrupted hierarchy (then: status bit,
  // stop, no hang).
  const int64_t step_bound = T.walk_limit > 0 ? (int64_t)T.walk_limit : 4 * (int64_t)T.nleaves + 16;
  int64_t walked = 0;

  for (;;) {
    int steps = 0;
    while (!done && scan_leaf < 0 && steps < 64) {
      ++steps;
      if (++walked > step_bound) {
        atomicOr(J.status, kStatusWalkBound);
        done = true;
        break;
      }
      if (nodei == kEnd) {
        if (phase == 0) {
          phase = 1;
          nodei = T.root;
          continue;
        }
        done = true;
        break;
      }
      // 48-byte node = three aligned 16-byte words:
      //   [x0 y0 x1 y1] [zmin.lo zmin.hi min_id min_pos] [count left escape right]
      const uint4* np = reinterpret_cast<const uint4*>(T.nodes + nodei);
      const float4 b = __ldg(reinterpret_cast<const float4*>(np));
      const uint4 mw = __ldg(np + 1);
      const uint4 cw = __ldg(np + 2);
      const int64_t nz = (int64_t)(((uint64_t)mw.y << 32) | mw.x);
      const uint32_t nid = mw.z, npos = mw.w, ncount = cw.x;
      const int32_t nleft = (int32_t)cw.y, esc = (int32_t)cw.z;
      const bool out = b.z <= ex.lo_dn || b.x >= ex.hi_up || b.w <= ey.lo_dn || b.y >= ey.hi_up;
      const bool in = !out && b.x > ex.lo_up && b.z < ex.hi_dn && b.y > ey.lo_up && b.w < ey.hi_dn;
      const bool leaf = nodei >= first_leaf;
      const bool improve = zid_less(nz, nid, bz, bid);
      if (phase == 0) {
        if (in) {
          cnt += ncount;
          if (improve) {
            bz = nz;
            bid = nid;
          }
          nodei = esc;
        } else if (out || leaf || (cnt >= thr && !improve)) {
          nodei = esc;
        } else {
          nodei = nleft;
        }
      } else {
        if (in || out || (cnt >= thr && !improve)) {
          nodei = esc;
        } else if (!leaf) {
          nodei = nleft;
        } else {
          bool min_inside = false;
          if (improve) {
            int64_t mx = __ldg(T.xk + npos), my = __ldg(T.yk + npos);
            min_inside = mx > ex.lo_k && mx < ex.hi_k && my > ey.lo_k && my < ey.hi_k;
            if (min_inside) {
              bz = nz;
              bid = nid;
            }
          }
          if (cnt < thr || (improve && !min_inside)) scan_leaf = nodei;
          nodei = esc;
        }
      }
    }
    uint32_t want = __ballot_sync(0xffffffffu, scan_leaf >= 0);
    if (want == 0) {
      if (__all_sync(0xffffffffu, done)) break;
      continue;
    }
    while (want) {
      const int src = __ffs(want) - 1;
      want &= want - 1;
      const int32_t leafi = __shfl_sync(0xffffffffu, scan_leaf, src);
      const int64_t lx = shfl64(ex.lo_k, src), hx = shfl64(ex.hi_k, src);
      const int64_t ly = shfl64(ey.lo_k, src), hy = shfl64(ey.hi_k, src);
      const Node* np = T.nodes + leafi;
      const int32_t first = __ldg(&np->left);
      const uint32_t c = __ldg(&np->count);
      uint32_t in_cnt = 0;
      int64_t mz = 0x7FFFFFFFFFFFFFFFll;
      uint32_t mid = 0xFFFFFFFFu;
      for (uint32_t o = 0; o < c; o += 32) {
        bool inside = false;
        if (o + lane < c) {
          const int64_t p = (int64_t)first + o + lane;
          const int64_t x = __ldg(T.xk + p), y = __ldg(T.yk + p);
          inside = x > lx && x < hx && y > ly && y < hy;
          if (inside) {
            const int64_t z = __ldg(T.zk + p);
            const uint32_t id = __ldg(T.pid + p);
            if (zid_less(z, id, mz, mid)) {
              mz = z;
              mid = id;
            }
          }
        }
        in_cnt += __popc(__ballot_sync(0xffffffffu, inside));
      }
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) {
        int64_t z2 = shfl64(mz, lane ^ o);
        uint32_t i2 = __shfl_xor_sync(0xffffffffu, mid, o);
        if (zid_less(z2, i2, mz, mid)) {
          mz = z2;
          mid = i2;
        }
      }
      if (lane == src) {
        cnt += in_cnt;
        if (zid_less(mz, mid, bz, bid)) {
          bz = mz;
          bid = mid;
        }
        scan_leaf = -1;
      }
    }
  }
  if (active) J.out[oidx] = cnt >= thr ? bid : kNone;
}

__global__ void __launch_bounds__(kQBlock) k_query(const QueryJob* __restrict__ jobs, int32_t njobs,
                                                   int64_t total_warps) {
  const int64_t warp = ((int64_t)blockIdx.x * kQBlock + threadIdx.x) >> 5;
  if (warp >= total_warps) return;  // warp-uniform
  query_warp(jobs, njobs, warp, threadIdx.x & 31);
}

// Persistent form for many uneven jobs: a fixed grid of warps pulls patch
// indices from one counter until the list is exhausted (each pull advances
// the counter, so the loop ends after at most total_warps + grid pulls).
__global__ void __launch_bounds__(kQBlock) k_query_persistent(const QueryJob* __restrict__ jobs, int32_t njobs,
                                                              int64_t total_warps,
                                                              unsigned long long* __restrict__ next) {
  const int lane = threadIdx.x & 31;
  for (;;) {
    unsigned long long w = 0;
    if (lane == 0) w = atomicAdd(next, 1ull);
    w = __shfl_sync(0xffffffffu, w, 0);
    if ((int64_t)w >= total_warps) return;
    query_warp(jobs, njobs, (int64_t)w, lane);
  }
}

// ---- stage 3: one warp per cell (owm_cellq.cuh) ---------------------------------
template <int kW, bool kPerm>
__global__ void __launch_bounds__(kW * 32) k_query_cells(TreeView T, const Edge* __restrict__ exs,
                                                           const Edge* __restrict__ eys, int32_t ncols,
                                                           int64_t ncells, const uint8_t* __restrict__ skip,
                                                           uint32_t* __restrict__ out, uint32_t* status) {
  extern __shared__ int32_t stack_all[];  // [kW][kS3Stack]
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int64_t cell = (int64_t)blockIdx.x * kW + wib;
  if (cell >= ncells) return;  // warp-uniform
  if (skip && skip[cell]) {
    if (lane == 0) out[cell] = kNone;
    return;
  }
  const uint32_t r =
      cell_min_warp<kPerm>(T, exs[cell % ncols], eys[cell / ncols], stack_all + wib * kS3Stack, status, lane);
  if (lane == 0) out[cell] = r;
}

template <int kW, bool kPerm>
cudaError_t launch_query_cells_as(const TreeView& t, const Edge* ex, const Edge* ey, int32_t ncols, int64_t ng,
                                  const uint8_t* skip, uint32_t* out, uint32_t* status, cudaStream_t s) {
  static bool configured = false;  // per template instance
  const size_t smem = (size_t)kW * kS3Stack * sizeof(int32_t);
  if (!configured) {
    cudaError_t e =
        cudaFuncSetAttribute(k_query_cells<kW, kPerm>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  OWM_LAUNCH("k_query_s3", s, (k_query_cells<kW, kPerm><<<(unsigned)((ng + kW - 1) / kW), kW * 32, smem, s>>>(
      t, ex, ey, ncols, ng, skip, out, status)));
  return cudaGetLastError();
}
// Trees without point arrays (t.perm set) read points through the permutation.
template <int kW>
cudaError_t launch_query_cells(const TreeView& t, const Edge* ex, const Edge* ey, int32_t ncols, int64_t ng,
                               const uint8_t* skip, uint32_t* out, uint32_t* status, cudaStream_t s) {
  return t.perm ? launch_query_cells_as<kW, true>(t, ex, ey, ncols, ng, skip, out, status, s)
                : launch_query_cells_as<kW, false>(t, ex, ey, ncols, ng, skip, out, status, s);
}

// ---- stage 2 -----------------------------------------------------------------
__global__ void k_s2_keys(const uint32_t* __restrict__ win, int64_t n, uint32_t none_key, uint32_t* __restrict__ keys) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    uint32_t v = win[i];
    keys[i] = v == kNone ? none_key : v;
  }
}

// Sorted keys -> flag of the first element of every run of length >= 2
// (overlap > 0), or of every valid element (overlap == 0: the reference
// counts all valid minima there, owm_optim3.cpp:185-188, and this kernel
// compacts them; only the sentinel id 0 of empty windows can repeat).
__global__ void k_s2_flags(const uint32_t* __restrict__ keys, int64_t n, uint32_t none_key, int need_dup,
                           uint32_t* __restrict__ flags) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    uint32_t k = keys[i];
    bool f = k != none_key;
    if (need_dup) f = f && (i == 0 || keys[i - 1] != k) && (i + 1 < n && keys[i + 1] == k);
    flags[i] = f ? 1u : 0u;
  }
}

// Stage 2 with overlap > 0 by occupancy bitmaps.  Ids of one cloud lie in
// [0, npoints]: the first atomic OR of an id's bit into `once` returns the old
// word, so a second occurrence also sets the bit in `twice`.  The LLPs are
// the set bits of `twice` -- ids that are the minimum of two or more windows
// -- in ascending id order: the list that sorting the minima and keeping the
// first id of every run of length >= 2 gives (owm_optim3.cpp:160-173,
// stage2 in optim3_func.cpp:609-625).
__global__ void k_s2_mark(const uint32_t* __restrict__ win, int64_t n, uint32_t max_id,
                          uint32_t* __restrict__ once, uint32_t* __restrict__ twice) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    s2_mark_id(once, twice, max_id, win[i]);  // kNone (and nothing else: ids are <= max_id) is skipped
  }
}

// The set bits of a bitmap, in ascending order, by blocks of kS2Chunk words:
// k_s2_count sums each block's bits, a scan of those sums gives each block's
// first output slot, and k_s2_emit_chunk ranks its threads' words (thread t
// owns kS2Words consecutive words, one 16-byte load) and writes their bit
// indices.  The bitmap is padded to whole chunks (zero words).
constexpr int kS2Block = 256;
constexpr int kS2Words = 4;
constexpr int64_t kS2Chunk = (int64_t)kS2Block * kS2Words;

__device__ __forceinline__ uint32_t block_sum_excl_256(uint32_t v, uint32_t* total) {
  __shared__ uint32_t ws[kS2Block / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) ws[w] = inc;
  __syncthreads();
  uint32_t before = 0, all = 0;
#pragma unroll
  for (int q = 0; q < kS2Block / 32; ++q) {
    const uint32_t x = ws[q];
    before += q < w ? x : 0u;
    all += x;
  }
  if (total) *total = all;
  return before + inc - v;
}

__global__ void __launch_bounds__(kS2Block) k_s2_count(const uint32_t* __restrict__ bm, uint32_t* __restrict__ part) {
  const uint4 q = __ldg(reinterpret_cast<const uint4*>(bm) + (int64_t)blockIdx.x * kS2Block + threadIdx.x);
  const uint32_t c = (uint32_t)(__popc(q.x) + __popc(q.y) + __popc(q.z) + __popc(q.w));
  uint32_t tot;
  block_sum_excl_256(c, &tot);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kS2Block) k_s2_emit_chunk(const uint32_t* __restrict__ bm,
                                                            const uint32_t* __restrict__ part,
                                                            uint32_t* __restrict__ out) {
  const int64_t w0 = (int64_t)blockIdx.x * kS2Chunk + (int64_t)threadIdx.x * kS2Words;
  const uint4 q = __ldg(reinterpret_cast<const uint4*>(bm + w0));
  const uint32_t word[4] = {q.x, q.y, q.z, q.w};
  const uint32_t c = (uint32_t)(__popc(q.x) + __popc(q.y) + __popc(q.z) + __popc(q.w));
  uint32_t p = block_sum_excl_256(c, nullptr) + part[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kS2Words; ++k) {
    uint32_t b = word[k];
    while (b) {
      out[p++] = (uint32_t)((w0 + k) * 32) + (uint32_t)(__ffs(b) - 1);
      b &= b - 1;
    }
  }
}

__global__ void k_compact(const uint32_t* __restrict__ vals, const uint32_t* __restrict__ flags,
                          const uint32_t* __restrict__ pos, int64_t n, uint32_t* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (flags[i]) out[pos[i]] = vals[i];
}

__global__ void k_flag_valid(const uint32_t* __restrict__ v, int64_t n, uint32_t* __restrict__ flags) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    flags[i] = v[i] != kNone ? 1u : 0u;
}

// The valid entries (!= kNone) of v[0..n), in order, into out and their
// number into *count, by one block: thread t owns the contiguous range
// [t*per, (t+1)*per).  For small n it replaces flag + scan + compact.
constexpr int kCompactBlock = 1024;
constexpr int64_t kCompactSmallMax = (int64_t)1 << 18;
__global__ void __launch_bounds__(kCompactBlock) k_compact_small(const uint32_t* __restrict__ v, int64_t n,
                                                                uint32_t* __restrict__ out,
                                                                uint32_t* __restrict__ count) {
  __shared__ uint32_t warp_tot[kCompactBlock / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t per = (n + kCompactBlock - 1) / kCompactBlock;
  const int64_t b = (int64_t)threadIdx.x * per;
  const int64_t e = b + per < n ? b + per : n;
  uint32_t c = 0;
  for (int64_t i = b; i < e; ++i) c += v[i] != kNone ? 1u : 0u;
  uint32_t inc = c;  // inclusive warp scan
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) warp_tot[w] = inc;
  __syncthreads();
  if (w == 0) {
    const uint32_t x = warp_tot[lane];
    uint32_t y = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, y, o);
      if (lane >= o) y += t;
    }
    warp_tot[lane] = y - x;  // exclusive warp offsets
    if (lane == 31) *count = y;
  }
  __syncthreads();
  uint32_t off = warp_tot[w] + inc - c;
  for (int64_t i = b; i < e; ++i) {
    const uint32_t x = v[i];
    if (x != kNone) out[off++] = x;
  }
}

// ---- stage 3 -----------------------------------------------------------------
// LLP grid (owm_optim3.cpp:192-197 + countNeighbors, optim3_func.cpp:503-539):
// a cell is occupied when an LLP lies strictly inside its box.
__global__ void k_s3_mark(const double* __restrict__ xyz, int stride, const uint32_t* __restrict__ llp,
                          const uint32_t* __restrict__ nllp, int64_t cap, const Edge* __restrict__ ex,
                          const Edge* __restrict__ ey, int32_t ncols, int32_t nrows, double min_x, double min_y,
                          double bsize, uint8_t* __restrict__ mark) {
  const int64_t n = min((int64_t)*nllp, cap);
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    uint32_t id = llp[k];
    double x = 0.0, y = 0.0;  // id 0 is the sentinel point {0, 0, DBL_MAX}
    if (id > 0) {
      x = xyz[stride * (int64_t)(id - 1)];
      y = xyz[stride * (int64_t)(id - 1) + 1];
    }
    const int64_t xk = dkey(x), yk = dkey(y);
    // candidate cells around floor((v - min)/B); the exact test decides
    double fi = floor((x - min_x) / bsize), fj = floor((y - min_y) / bsize);
    if (!(fi > -4.0 && fi < (double)ncols + 4.0 && fj > -4.0 && fj < (double)nrows + 4.0)) continue;
    int32_t ic = (int32_t)fi, jc = (int32_t)fj;
    for (int32_t jj = max(jc - 1, 0); jj <= min(jc + 1, nrows - 1); ++jj) {
      if (!(yk > ey[jj].lo_k && yk < ey[jj].hi_k)) continue;
      for (int32_t ii = max(ic - 1, 0); ii <= min(ic + 1, ncols - 1); ++ii)
        if (xk > ex[ii].lo_k && xk < ex[ii].hi_k) mark[(int64_t)jj * ncols + ii] = 1;
    }
  }
}

__global__ void k_u32_to_i64(const uint32_t* __restrict__ in, const uint32_t* __restrict__ count, int64_t cap,
                             int64_t* __restrict__ out) {
  const int64_t n = count ? min((int64_t)*count, cap) : cap;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    uint32_t v = in[i];
    out[i] = v == kNone ? -1 : (int64_t)v;
  }
}

__global__ void k_i64_to_u32(const int64_t* __restrict__ in, int64_t n, uint32_t* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t v = in[i];
    out[i] = (v < 0 || v >= (int64_t)kNone) ? kNone : (uint32_t)v;
  }
}

int grid1d(int64_t n, int block = 256) {
  int64_t g = (n + block - 1) / block;
  if (g > 152 * 32) g = 152 * 32;
  return (int)std::max<int64_t>(g, 1);
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

int compute_edges(const owm_params& p, double ox, double oy, bool cells, Edge* d_ex, Edge* d_ey, cudaStream_t s,
                  int64_t* launches) {
  int32_t nc = cells ? (int32_t)p.ncols_grid : (int32_t)p.ncols;
  int32_t nr = cells ? (int32_t)p.nrows_grid : (int32_t)p.nrows;
  int32_t m = std::max(nc, nr);
  if (m <= 0) return OWM_OK;
  uint16_t w16 = (uint16_t)p.wsize, b16 = (uint16_t)p.bsize;
  int32_t half = cells ? b16 / 2 : w16 / 2;  // integer division of a ushort
  double step = p.displace;
  OWM_LAUNCH("k_edges", s, k_edges<<<(m + 127) / 128, 128, 0, s>>>(p.bbox.min_x, p.bbox.min_y, step, half, cells ? 1 : 0, nc, nr, (int32_t)b16,
                                         ox, oy, d_ex, d_ey));
  count_launch(launches);
  OWM_CUDA_TRY(cudaGetLastError());
  return OWM_OK;
}

int64_t job_warps(int32_t ncols, int32_t nrows, int32_t patch_lx) {
  if (ncols <= 0 || nrows <= 0) return 0;
  const int32_t px = 1 << patch_lx, py = 32 >> patch_lx;
  return (int64_t)((ncols + px - 1) / px) * ((nrows + py - 1) / py);
}

int launch_query(const QueryJob* d_jobs, int32_t njobs, int64_t total_warps, cudaStream_t s, int64_t* launches,
                 const char* name) {
  if (total_warps <= 0) return OWM_OK;
  int64_t blocks = (total_warps * 32 + kQBlock - 1) / kQBlock;
  OWM_LAUNCH(name, s, k_query<<<(unsigned)blocks, kQBlock, 0, s>>>(d_jobs, njobs, total_warps));
  count_launch(launches);
  OWM_CUDA_TRY(cudaGetLastError());
  return OWM_OK;
}

int launch_query_persistent(const QueryJob* d_jobs, int32_t njobs, int64_t total_warps, unsigned long long* d_next,
                            int blocks, cudaStream_t s, int64_t* launches, const char* name) {
  if (total_warps <= 0) return OWM_OK;
  OWM_CUDA_TRY(cudaMemsetAsync(d_next, 0, sizeof(unsigned long long), s));
  int64_t need = (total_warps * 32 + kQBlock - 1) / kQBlock;
  int g = (int)std::min<int64_t>(need, blocks);
  OWM_LAUNCH(name, s, k_query_persistent<<<g, kQBlock, 0, s>>>(d_jobs, njobs, total_warps, d_next));
  count_launch(launches);
  OWM_CUDA_TRY(cudaGetLastError());
  return OWM_OK;
}

int run_query(const QueryJob& job, QueryJob* d_job_slot, cudaStream_t s, int64_t* launches, const char* name) {
  QueryJob j = job;
  j.warp_begin = 0;
  OWM_CUDA_TRY(cudaMemcpyAsync(d_job_slot, &j, sizeof(QueryJob), cudaMemcpyHostToDevice, s));
  return launch_query(d_job_slot, 1, job_warps(j.ncols, j.nrows, j.patch_lx), s, launches, name);
}

size_t stage2_scratch_bytes(int64_t n) {
  return 4 * align256((size_t)n * 4) + align256(radix_sort_temp_bytes(n)) + align256(scan_temp_bytes(n)) + 1024;
}

int run_stage2(const uint32_t* d_win, int64_t n, int64_t npoints, double overlap, uint32_t* d_llp,
               uint32_t* d_count, void* scratch, size_t scratch_bytes, cudaStream_t s, int64_t* launches) {
  if (n <= 0) {
    OWM_CUDA_TRY(cudaMemsetAsync(d_count, 0, 4, s));
    return OWM_OK;
  }
  if (scratch_bytes < stage2_scratch_bytes(n)) return OWM_ENOMEM;
  char* sp = static_cast<char*>(scratch);
  auto take = [&](size_t b) {
    void* p = sp;
    sp += align256(b);
    return p;
  };
  uint32_t* k0 = (uint32_t*)take((size_t)n * 4);
  uint32_t* k1 = (uint32_t*)take((size_t)n * 4);
  uint32_t* flags = (uint32_t*)take((size_t)n * 4);
  uint32_t* pos = (uint32_t*)take((size_t)n * 4);
  size_t sb = radix_sort_temp_bytes(n);
  void* st = take(sb);
  size_t cb = scan_temp_bytes(n);
  void* ct = take(cb);
  // ids are <= npoints < none_key, so `bits` key bits order them with "none" last
  int bits = 1;
  while (bits < 32 && ((uint64_t)1 << bits) <= (uint64_t)npoints + 1) ++bits;
  uint32_t none_key = bits >= 32 ? 0xFFFFFFFFu : (uint32_t)(((uint64_t)1 << bits) - 1);
  OWM_LAUNCH("k_s2_keys", s, k_s2_keys<<<grid1d(n), 256, 0, s>>>(d_win, n, none_key, k0));
  count_launch(launches);
  bool alt = false;
  OWM_CUDA_TRY(radix_sort(k0, nullptr, k1, nullptr, n, bits, false, st, sb, s, &alt, launches));
  const uint32_t* sk = alt ? k1 : k0;
  OWM_LAUNCH("k_s2_flags", s, k_s2_flags<<<grid1d(n), 256, 0, s>>>(sk, n, none_key, overlap > 0.0 ? 1 : 0, flags));
  count_launch(launches);
  OWM_CUDA_TRY(exclusive_scan_u32(flags, pos, n, d_count, ct, cb, s, launches));
  OWM_LAUNCH("k_compact", s, k_compact<<<grid1d(n), 256, 0, s>>>(sk, flags, pos, n, d_llp));
  count_launch(launches);
  OWM_CUDA_TRY(cudaGetLastError());
  return OWM_OK;
}

namespace {
struct S2Bitmaps {
  uint32_t *once, *twice, *part;
  void* ct;
  size_t cb;
  int64_t nw, nblocks;
};
S2Bitmaps stage2_bitmap_layout(void* scratch, int64_t npoints) {
  S2Bitmaps B;
  B.nblocks = ((npoints + 1 + 31) / 32 + kS2Chunk - 1) / kS2Chunk;  // bits for ids 0..npoints
  B.nw = B.nblocks * kS2Chunk;                                      // whole chunks
  char* sp = static_cast<char*>(scratch);
  auto take = [&](size_t b) {
    void* p = sp;
    sp += align256(b);
    return p;
  };
  B.once = (uint32_t*)take((size_t)B.nw * 4);   // once and twice are adjacent:
  B.twice = (uint32_t*)take((size_t)B.nw * 4);  // one memset clears both
  B.part = (uint32_t*)take((size_t)B.nblocks * 4);
  B.cb = scan_temp_bytes(B.nblocks);
  B.ct = take(B.cb);
  return B;
}
}  // namespace

size_t stage2_bitmap_scratch_bytes(int64_t npoints) {
  const int64_t nb = ((npoints + 1 + 31) / 32 + kS2Chunk - 1) / kS2Chunk;
  const int64_t nw = nb * kS2Chunk;
  return 2 * align256((size_t)nw * 4) + align256((size_t)nb * 4) + align256(scan_temp_bytes(nb)) + 1024;
}

int stage2_bitmap_clear(void* scratch, size_t scratch_bytes, int64_t npoints, cudaStream_t s) {
  if (npoints < 0 || npoints >= (int64_t)kNone) return OWM_EINVAL;
  if (scratch_bytes < stage2_bitmap_scratch_bytes(npoints)) return OWM_ENOMEM;
  const S2Bitmaps B = stage2_bitmap_layout(scratch, npoints);
  OWM_CUDA_TRY(cudaMemsetAsync(B.once, 0, 2 * align256((size_t)B.nw * 4), s));  // once, then twice
  return OWM_OK;
}

void stage2_bitmap_ptrs(void* scratch, int64_t npoints, uint32_t** once, uint32_t** twice) {
  const S2Bitmaps B = stage2_bitmap_layout(scratch, npoints);
  *once = B.once;
  *twice = B.twice;
}

int run_stage2_bitmap(const uint32_t* d_win, int64_t n, int64_t npoints, double overlap, uint32_t* d_llp,
                      uint32_t* d_count, void* scratch, size_t scratch_bytes, cudaStream_t s, int64_t* launches,
                      bool cleared, bool marked) {
  if (n <= 0) {
    OWM_CUDA_TRY(cudaMemsetAsync(d_count, 0, 4, s));
    return OWM_OK;
  }
  if (npoints < 0 || npoints >= (int64_t)kNone || !(overlap > 0.0)) return OWM_EINVAL;
  if (scratch_bytes < stage2_bitmap_scratch_bytes(npoints)) return OWM_ENOMEM;
  const S2Bitmaps B = stage2_bitmap_layout(scratch, npoints);
  if (!marked) {
    if (!cleared) OWM_CUDA_TRY(cudaMemsetAsync(B.once, 0, 2 * align256((size_t)B.nw * 4), s));
    OWM_LAUNCH("k_s2_mark", s, k_s2_mark<<<grid1d(n), 256, 0, s>>>(d_win, n, (uint32_t)npoints, B.once, B.twice));
    count_launch(launches);
  }
  OWM_LAUNCH("k_s2_count", s, k_s2_count<<<(unsigned)B.nblocks, kS2Block, 0, s>>>(B.twice, B.part));
  count_launch(launches);
  OWM_CUDA_TRY(exclusive_scan_u32(B.part, B.part, B.nblocks, d_count, B.ct, B.cb, s, launches));
  OWM_LAUNCH("k_s2_emit", s, k_s2_emit_chunk<<<(unsigned)B.nblocks, kS2Block, 0, s>>>(B.twice, B.part, d_llp));
  count_launch(launches);
  OWM_CUDA_TRY(cudaGetLastError());
  return OWM_OK;
}

int run_stage2_into(const uint32_t* d_win, uint32_t* k0, uint32_t* k1, uint32_t* flags, uint32_t* pos, int64_t n,
                    int64_t npoints, double overlap, uint32_t* d_llp, uint32_t* d_count, void* temp,
                    size_t temp_bytes, cudaStream_t s, int64_t* launches) {
  if (n <= 0) {
    OWM_CUDA_TRY(cudaMemsetAsync(d_count, 0, 4, s));
    return OWM_OK;
  }
  size_t sb = radix_sort_temp_bytes(n);
  size_t cb = scan_temp_bytes(n);
  if (temp_bytes < align256(sb) + cb) return OWM_ENOMEM;
  void* st = temp;
  void* ct = static_cast<char*>(temp) + align256(sb);
  // ids are <= npoints < none_key, so `bits` key bits order them with "none" last
  int bits = 1;
  while (bits < 32 && ((uint64_t)1 << bits) <= (uint64_t)npoints + 1) ++bits;
  uint32_t none_key = bits >= 32 ? 0xFFFFFFFFu : (uint32_t)(((uint64_t)1 << bits) - 1);
  OWM_LAUNCH("k_s2_keys", s, k_s2_keys<<<grid1d(n), 256, 0, s>>>(d_win, n, none_key, k0));
  count_launch(launches);
  bool alt = false;
  OWM_CUDA_TRY(radix_sort(k0, nullptr, k1, nullptr, n, bits, false, st, sb, s, &alt, launches));
  const uint32_t* sk = alt ? k1 : k0;
  OWM_LAUNCH("k_s2_flags", s, k_s2_flags<<<grid1d(n), 256, 0, s>>>(sk, n, none_key, overlap > 0.0 ? 1 : 0, flags));
  count_launch(launches);
  OWM_CUDA_TRY(exclusive_scan_u32(flags, pos, n, d_count, ct, cb, s, launches));
  OWM_LAUNCH("k_compact", s, k_compact<<<grid1d(n), 256, 0, s>>>(sk, flags, pos, n, d_llp));
  count_launch(launches);
  OWM_CUDA_TRY(cudaGetLastError());
  return OWM_OK;
}

size_t stage3_scratch_bytes(int64_t ngrid) {
  int64_t m = std::max<int64_t>(ngrid, 1);
  return align256((size_t)m) + 3 * align256((size_t)m * 4) + 2 * align256((size_t)65536 * sizeof(Edge)) +
         align256(scan_temp_bytes(m)) + 1024;
}

namespace {
struct S3Layout {
  uint8_t* mark;
  uint32_t *cellmin, *flags, *pos;
  Edge *ex, *ey;
  void* ct;
  size_t cb;
};
S3Layout stage3_layout(void* scratch, int64_t ng) {
  char* sp = static_cast<char*>(scratch);
  auto take = [&](size_t b) {
    void* q = sp;
    sp += align256(b);
    return q;
  };
  S3Layout L;
  L.mark = (uint8_t*)take((size_t)ng);
  L.cellmin = (uint32_t*)take((size_t)ng * 4);
  L.flags = (uint32_t*)take((size_t)ng * 4);
  L.pos = (uint32_t*)take((size_t)ng * 4);
  L.ex = (Edge*)take((size_t)65536 * sizeof(Edge));
  L.ey = (Edge*)take((size_t)65536 * sizeof(Edge));
  L.cb = scan_temp_bytes(ng);
  L.ct = take(L.cb);
  return L;
}
}  // namespace

int run_stage3_prepare(double ox, double oy, const owm_params& p, void* scratch, size_t scratch_bytes,
                       cudaStream_t s, int64_t* launches) {
  const int64_t ng = p.ngrid;
  if (p.bsize == 0 || ng <= 0) return OWM_OK;
  if (scratch_bytes < stage3_scratch_bytes(ng)) return OWM_ENOMEM;
  const S3Layout L = stage3_layout(scratch, ng);
  int rc = compute_edges(p, ox, oy, true, L.ex, L.ey, s, launches);
  if (rc) return rc;
  OWM_CUDA_TRY(cudaMemsetAsync(L.mark, 0, (size_t)ng, s));
  return OWM_OK;
}

int run_stage3_mark(const double* d_xyz, int stride, const owm_params& p, const uint32_t* d_llp, const uint32_t* d_nllp,
                    int64_t llp_cap, void* scratch, size_t scratch_bytes, cudaStream_t s, int64_t* launches) {
  const int64_t ng = p.ngrid;
  if (p.bsize == 0 || ng <= 0) return OWM_OK;
  if (scratch_bytes < stage3_scratch_bytes(ng)) return OWM_ENOMEM;
  const S3Layout L = stage3_layout(scratch, ng);
  if (llp_cap > 0) {
    OWM_LAUNCH("k_s3_mark", s, k_s3_mark<<<grid1d(llp_cap), 256, 0, s>>>(d_xyz, stride, d_llp, d_nllp, llp_cap, L.ex, L.ey,
                                                                       (int32_t)p.ncols_grid, (int32_t)p.nrows_grid,
                                                                       p.bbox.min_x, p.bbox.min_y, (double)p.bsize,
                                                                       L.mark));
    count_launch(launches);
  }
  OWM_CUDA_TRY(cudaGetLastError());
  return OWM_OK;
}

int run_stage3_query(const TreeView& t, const owm_params& p, uint32_t* d_out, uint32_t* d_count, void* scratch,
                     size_t scratch_bytes, uint32_t* status, cudaStream_t s, int64_t* launches) {
  const int64_t ng = p.ngrid;
  if (p.bsize == 0 || ng <= 0) {
    OWM_CUDA_TRY(cudaMemsetAsync(d_count, 0, 4, s));
    return OWM_OK;
  }
  if (scratch_bytes < stage3_scratch_bytes(ng)) return OWM_ENOMEM;
  const S3Layout L = stage3_layout(scratch, ng);
  if ((ng + 1) / 2 >= 0x7FFFFFFFll) return OWM_ERANGE;
  OWM_CUDA_TRY(t.cell_warps == 2   ? launch_query_cells<2>(t, L.ex, L.ey, (int32_t)p.ncols_grid, ng, L.mark, L.cellmin, status, s)
               : t.cell_warps == 8 ? launch_query_cells<8>(t, L.ex, L.ey, (int32_t)p.ncols_grid, ng, L.mark, L.cellmin, status, s)
                                   : launch_query_cells<4>(t, L.ex, L.ey, (int32_t)p.ncols_grid, ng, L.mark, L.cellmin, status, s));
  count_launch(launches);
  if (ng <= kCompactSmallMax) {
    OWM_LAUNCH("k_compact_small", s, k_compact_small<<<1, kCompactBlock, 0, s>>>(L.cellmin, ng, d_out, d_count));
    count_launch(launches);
  } else {
    OWM_LAUNCH("k_flag_valid", s, k_flag_valid<<<grid1d(ng), 256, 0, s>>>(L.cellmin, ng, L.flags));
    count_launch(launches);
    OWM_CUDA_TRY(exclusive_scan_u32(L.flags, L.pos, ng, d_count, L.ct, L.cb, s, launches));
    OWM_LAUNCH("k_compact", s, k_compact<<<grid1d(ng), 256, 0, s>>>(L.cellmin, L.flags, L.pos, ng, d_out));
    count_launch(launches);
  }
  OWM_CUDA_TRY(cudaGetLastError());
  return OWM_OK;
}

int run_stage3(const TreeView& t, const double* d_xyz, int stride, const owm_params& p, const uint32_t* d_llp,
               const uint32_t* d_nllp, int64_t llp_cap, uint32_t* d_out, uint32_t* d_count, void* scratch,
               size_t scratch_bytes, QueryJob* d_job_slot, uint32_t* status, cudaStream_t s, int64_t* launches) {
  (void)d_job_slot;
  int rc = run_stage3_prepare(t.ox, t.oy, p, scratch, scratch_bytes, s, launches);
  if (!rc) rc = run_stage3_mark(d_xyz, stride, p, d_llp, d_nllp, llp_cap, scratch, scratch_bytes, s, launches);
  if (rc) return rc;
  return run_stage3_query(t, p, d_out, d_count, scratch, scratch_bytes, status, s, launches);
}

int u32_to_i64_ids(const uint32_t* in, const uint32_t* d_count, int64_t cap, int64_t* out, cudaStream_t s,
                   int64_t* launches) {
  if (cap <= 0) return OWM_OK;
  OWM_LAUNCH("k_u32_to_i64", s, k_u32_to_i64<<<grid1d(cap), 256, 0, s>>>(in, d_count, cap, out));
  count_launch(launches);
  OWM_CUDA_TRY(cudaGetLastError());
  return OWM_OK;
}

int i64_to_u32_ids(const int64_t* in, int64_t n, uint32_t* out, cudaStream_t s, int64_t* launches) {
  if (n <= 0) return OWM_OK;
  OWM_LAUNCH("k_i64_to_u32", s, k_i64_to_u32<<<grid1d(n), 256, 0, s>>>(in, n, out));
  count_launch(launches);
  OWM_CUDA_TRY(cudaGetLastError());
  return OWM_OK;
}

}  // namespace owm
