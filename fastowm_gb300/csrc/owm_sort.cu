// Device-wide primitives: exclusive scan and an on-chip-staged LSD radix sort
// (the fewest passes of digits of at most 8 bits, or 7 bits for large sorts,
// their widths balanced: radix_digit_bits; reduce-then-scan).
//
// Radix pass over tiles of 4096 keys.  Large sorts split the tiles into one
// contiguous chunk per persistent block:
//   upsweep    digit histogram of each chunk (vectorised 16-byte key loads)
//   scan       exclusive scan of the digit-major [256 x chunks] count table
//              (small sorts: per tile, [256 x tiles])
//   downsweep  stable ranking inside the tile, keys/values staged in shared
//              memory in digit order, then written out so that each digit's
//              run is a contiguous, coalesced stretch of the output.
// Digits of at most 7 bits are ranked by k_rs_downsweep_rank: every thread
// counts its 16 consecutive keys in its own byte counters (shared-memory
// atomics, no warp vote), a word-parallel scan turns the counters into
// ranks, and tiles arrive by TMA (cp.async.bulk.tensor, 128-byte swizzle,
// mbarrier completion).  Large sorts whose buffers no tensor map can view
// (a base not 16-byte aligned, no driver entry point) fall back to the
// ballot-multisplit kernel (k_rs_downsweep_pipe).
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "owm_internal.cuh"

namespace owm {

namespace {

constexpr int kBlock = 256;
constexpr int kItems = 16;
constexpr int kTile = kBlock * kItems;  // 4096 keys
static_assert(kTile == kSortTile, "the count-table layout is shared with key producers");
constexpr int kWarps = kBlock / 32;
constexpr int kRadix = 256;
constexpr int kSubChunks = 4;     // upsweep blocks per downsweep chunk (sort_part_range)
constexpr int64_t kMaxChunks = 1024;  // persistent downsweep blocks, at most

// Count-table entries a sort of ntiles tiles may use: per tile (small
// sorts) or per upsweep part (large sorts).
int64_t hist_entries(int64_t ntiles) {
  return std::max<int64_t>(ntiles, kSubChunks * std::min<int64_t>(ntiles, kMaxChunks)) * kRadix;
}

constexpr int kScanBlock = 1024;
constexpr int kScanItems = 8;
constexpr int kScanChunk = kScanBlock * kScanItems;  // 8192 values per block

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Lanes of the warp whose 8-bit digit equals this lane's, among the lanes
// with valid set: one ballot per digit bit, the mask narrowed by each
// (warp-level multisplit by ballots, Ashkiani et al., 2016).  Cheaper than
// the general 32-bit match instruction when the label has few bits.
__device__ __forceinline__ uint32_t match_digit8(uint32_t d, bool valid) {
  uint32_t m = __ballot_sync(0xffffffffu, valid);
#pragma unroll
  for (int b = 0; b < 8; ++b) {
    const uint32_t bit = (d >> b) & 1u;
    const uint32_t v = __ballot_sync(0xffffffffu, bit);
    m &= bit ? v : ~v;
  }
  return m;
}

// The same for a digit of dbits < 8 bits (d < 2^dbits): one ballot per live
// bit.  dbits is uniform over the grid.
__device__ __forceinline__ uint32_t match_digit_n(uint32_t d, bool valid, int dbits) {
  uint32_t m = __ballot_sync(0xffffffffu, valid);
#pragma unroll
  for (int b = 0; b < 7; ++b) {
    if (b < dbits) {
      const uint32_t bit = (d >> b) & 1u;
      const uint32_t v = __ballot_sync(0xffffffffu, bit);
      m &= bit ? v : ~v;
    }
  }
  return m;
}

// Inclusive warp scan.
__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
  int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Exclusive block scan of one value per thread; returns the block total in
// *total.  blockDim.x must be a multiple of 32 and <= 1024.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* total) {
  __shared__ uint32_t warp_sums[32];
  __shared__ uint32_t block_total;
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  uint32_t inc = warp_incl_scan(v);
  if (lane == 31) warp_sums[w] = inc;
  __syncthreads();
  if (w == 0) {
    uint32_t s = lane < nw ? warp_sums[lane] : 0u;
    uint32_t si = warp_incl_scan(s);
    if (lane < nw) warp_sums[lane] = si - s;
    if (lane == nw - 1) block_total = si;
  }
  __syncthreads();
  uint32_t r = inc - v + warp_sums[w];
  if (total) *total = block_total;
  __syncthreads();
  return r;
}

// ---- scan ------------------------------------------------------------------
__global__ void k_scan_reduce(const uint32_t* __restrict__ in, int64_t n, uint32_t* __restrict__ part) {
  int64_t base = (int64_t)blockIdx.x * kScanChunk;
  uint32_t s = 0;
  for (int i = threadIdx.x; i < kScanChunk; i += kScanBlock) {
    int64_t p = base + i;
    if (p < n) s += in[p];
  }
  uint32_t tot;
  block_excl_scan(s, &tot);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

// Single block: exclusive scan of <= kScanChunk values (the partial sums of a
// large scan, or a whole small one); in == out allowed.
__global__ void k_scan_parts(const uint32_t* in, uint32_t* out, int64_t nparts, uint32_t* total) {
  uint32_t v[kScanItems];
  uint32_t s = 0;
  for (int k = 0; k < kScanItems; ++k) {
    int64_t p = (int64_t)threadIdx.x * kScanItems + k;
    v[k] = p < nparts ? in[p] : 0u;
    s += v[k];
  }
  uint32_t tot;
  uint32_t off = block_excl_scan(s, &tot);
  for (int k = 0; k < kScanItems; ++k) {
    int64_t p = (int64_t)threadIdx.x * kScanItems + k;
    if (p < nparts) out[p] = off;
    off += v[k];
  }
  if (threadIdx.x == 0 && total) *total = tot;
}

// Down-sweep of block b from an already scanned chunk offset part[b].
__global__ void k_scan_down_scanned(const uint32_t* in, uint32_t* out, int64_t n, const uint32_t* __restrict__ part) {
  int64_t base = (int64_t)blockIdx.x * kScanChunk + (int64_t)threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t s = 0;
  for (int k = 0; k < kScanItems; ++k) {
    int64_t p = base + k;
    v[k] = p < n ? in[p] : 0u;
    s += v[k];
  }
  uint32_t off = block_excl_scan(s, nullptr) + part[blockIdx.x];
  for (int k = 0; k < kScanItems; ++k) {
    int64_t p = base + k;
    if (p < n) out[p] = off;
    off += v[k];
  }
}

// Block b scans its chunk from the sum of the chunk totals before it, which
// it adds up itself (at most kScanChunk of them, in L2), so no separate scan
// of the totals is needed; the last block writes the grand total.
__global__ void k_scan_down(const uint32_t* in, uint32_t* out, int64_t n, const uint32_t* __restrict__ part,
                            uint32_t* __restrict__ total) {
  uint32_t before = 0;
  for (int64_t i = threadIdx.x; i < (int64_t)blockIdx.x; i += kScanBlock) before += part[i];
  uint32_t base_off;
  block_excl_scan(before, &base_off);
  if (total && threadIdx.x == 0 && blockIdx.x == gridDim.x - 1) *total = base_off + part[blockIdx.x];
  int64_t base = (int64_t)blockIdx.x * kScanChunk + (int64_t)threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t s = 0;
  for (int k = 0; k < kScanItems; ++k) {
    int64_t p = base + k;
    v[k] = p < n ? in[p] : 0u;
    s += v[k];
  }
  uint32_t off = block_excl_scan(s, nullptr) + base_off;
  for (int k = 0; k < kScanItems; ++k) {
    int64_t p = base + k;
    if (p < n) out[p] = off;
    off += v[k];
  }
}

// ---- radix sort --------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_rs_upsweep(const uint32_t* __restrict__ keys, int64_t n,
                                                       int shift, uint32_t dmask, uint32_t* __restrict__ hist,
                                                       int64_t ntiles) {
  __shared__ uint32_t h[kWarps][kRadix];
  for (int i = threadIdx.x; i < kWarps * kRadix; i += kBlock) (&h[0][0])[i] = 0;
  __syncthreads();
  int w = threadIdx.x >> 5;
  int64_t base = (int64_t)blockIdx.x * kTile;
  if (base + kTile <= n) {
    const uint4* k4 = reinterpret_cast<const uint4*>(keys + base);
#pragma unroll
    for (int it = 0; it < kTile / 4 / kBlock; ++it) {
      uint4 q = __ldg(k4 + it * kBlock + threadIdx.x);
      atomicAdd(&h[w][(q.x >> shift) & dmask], 1u);
      atomicAdd(&h[w][(q.y >> shift) & dmask], 1u);
      atomicAdd(&h[w][(q.z >> shift) & dmask], 1u);
      atomicAdd(&h[w][(q.w >> shift) & dmask], 1u);
    }
  } else {
    for (int i = threadIdx.x; i < kTile; i += kBlock) {
      int64_t p = base + i;
      if (p < n) atomicAdd(&h[w][(keys[p] >> shift) & dmask], 1u);
    }
  }
  __syncthreads();
  for (int d = threadIdx.x; d < kRadix; d += kBlock) {
    uint32_t s = 0;
#pragma unroll
    for (int q = 0; q < kWarps; ++q) s += h[q][d];
    hist[(int64_t)d * ntiles + blockIdx.x] = s;
  }
}

// Digit histogram of sub-chunk blockIdx.x: part blockIdx.x % kSubChunks of
// chunk blockIdx.x / kSubChunks (gridDim.x / kSubChunks chunks), into
// hist[d * gridDim.x + blockIdx.x].  The scanned entry of a chunk's first
// part is then that chunk's output base.  Keys are 16-byte aligned.
// At most 32 registers a thread (8 bytes spill): 8 blocks per SM, so the
// 4 x 304 parts run in one wave (36 registers: 7 blocks, 1.14 waves).
__global__ void __maxnreg__(32) k_rs_upsweep_chunk(const uint32_t* __restrict__ keys, int64_t n,
                                                             int shift, uint32_t dmask, uint32_t* __restrict__ hist,
                                                             int64_t ntiles) {
  __shared__ uint32_t h[kWarps][kRadix];
  for (int i = threadIdx.x; i < kWarps * kRadix; i += kBlock) (&h[0][0])[i] = 0;
  __syncthreads();
  const int w = threadIdx.x >> 5;
  int64_t b, e;  // an empty part reads nothing
  sort_part_range(n, ntiles, gridDim.x, blockIdx.x, &b, &e);
  const int64_t e4 = b + ((e - b) & ~(int64_t)3);  // 16-byte loads up to here
  const uint4* k4 = reinterpret_cast<const uint4*>(keys + b);
  for (int64_t i = threadIdx.x; i < (e4 - b) / 4; i += kBlock) {
    const uint4 q = __ldg(k4 + i);
    atomicAdd(&h[w][(q.x >> shift) & dmask], 1u);
    atomicAdd(&h[w][(q.y >> shift) & dmask], 1u);
    atomicAdd(&h[w][(q.z >> shift) & dmask], 1u);
    atomicAdd(&h[w][(q.w >> shift) & dmask], 1u);
  }
  for (int64_t p = e4 + threadIdx.x; p < e; p += kBlock) atomicAdd(&h[w][(__ldg(keys + p) >> shift) & dmask], 1u);
  __syncthreads();
  for (int d = threadIdx.x; d < kRadix; d += kBlock) {
    uint32_t s = 0;
#pragma unroll
    for (int q = 0; q < kWarps; ++q) s += h[q][d];
    hist[(int64_t)d * gridDim.x + blockIdx.x] = s;
  }
}

template <bool kHasVals, bool kIota>
__global__ void __launch_bounds__(kBlock, 3) k_rs_downsweep(const uint32_t* __restrict__ kin,
                                                            const uint32_t* __restrict__ vin,
                                                            uint32_t* __restrict__ kout,
                                                            uint32_t* __restrict__ vout, int64_t n, int shift,
                                                            uint32_t dmask, const uint32_t* __restrict__ hist,
                                                            int64_t ntiles) {
  __shared__ uint32_t s_keys[kTile];
  __shared__ uint32_t s_vals[kHasVals ? kTile : 1];
  __shared__ uint32_t s_wcnt[kWarps][kRadix];
  __shared__ uint32_t s_start[kRadix];
  __shared__ uint32_t s_glob[kRadix];

  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t tile_base = (int64_t)blockIdx.x * kTile;
  const int64_t warp_base = tile_base + (int64_t)w * 32 * kItems;
  for (int i = threadIdx.x; i < kWarps * kRadix; i += kBlock) (&s_wcnt[0][0])[i] = 0;
  for (int d = threadIdx.x; d < kRadix; d += kBlock) s_glob[d] = hist[(int64_t)d * ntiles + blockIdx.x];
  __syncthreads();

  // keys only during ranking; values are fetched at the scatter (shorter
  // live ranges -> 3 resident blocks per SM)
  uint32_t k[kItems];
  uint32_t rank[kItems / 2];  // two 16-bit ranks per word
  const uint32_t lt = lanemask_lt();
  const bool full = warp_base + 32 * kItems <= n;
#pragma unroll
  for (int i = 0; i < kItems; ++i) {
    int64_t p = warp_base + i * 32 + lane;
    k[i] = (full || p < n) ? __ldg(kin + p) : 0u;
  }
#pragma unroll
  for (int i = 0; i < kItems; ++i) {
    int64_t p = warp_base + i * 32 + lane;
    bool valid = full || p < n;
    uint32_t d = (k[i] >> shift) & dmask;
    uint32_t peers = match_digit8(d, valid);
    uint32_t before = valid ? s_wcnt[w][d] : 0u;
    __syncwarp();
    uint32_t r = __popc(peers & lt);
    if (valid && r == 0) s_wcnt[w][d] = before + __popc(peers);
    __syncwarp();
    uint32_t rk = before + r;
    if (i & 1)
      rank[i >> 1] |= rk << 16;
    else
      rank[i >> 1] = rk;
  }
  __syncthreads();
  // exclusive prefix over warps per digit, then over digits (one per thread)
  uint32_t tot = 0;
  {
    int d = threadIdx.x;  // kBlock == kRadix
#pragma unroll
    for (int q = 0; q < kWarps; ++q) {
      uint32_t c = s_wcnt[q][d];
      s_wcnt[q][d] = tot;
      tot += c;
    }
  }
  uint32_t start = block_excl_scan(tot, nullptr);
  s_start[threadIdx.x] = start;
  __syncthreads();
#pragma unroll
  for (int i = 0; i < kItems; ++i) {
    int64_t p = warp_base + i * 32 + lane;
    if (full || p < n) {
      uint32_t d = (k[i] >> shift) & dmask;
      uint32_t rk = (rank[i >> 1] >> ((i & 1) * 16)) & 0xFFFFu;
      uint32_t pos = s_start[d] + s_wcnt[w][d] + rk;
      s_keys[pos] = k[i];
      if (kHasVals) s_vals[pos] = kIota ? (uint32_t)p : __ldg(vin + p);
    }
  }
  __syncthreads();
  int64_t tile_n = n - tile_base < kTile ? n - tile_base : kTile;
  for (int j = threadIdx.x; j < tile_n; j += kBlock) {
    uint32_t key = s_keys[j];
    uint32_t d = (key >> shift) & dmask;
    uint32_t gp = s_glob[d] + (uint32_t)j - s_start[d];
    kout[gp] = key;
    if (kHasVals) vout[gp] = s_vals[j];
  }
}

// ---- pipelined downsweep ------------------------------------------------------
// Persistent form of the downsweep: each block walks tiles blockIdx.x,
// blockIdx.x + grid, ...  While one tile is ranked and scattered, the next
// tile's keys, values and digit offsets are already being copied into shared
// memory with cp.async (double buffer), so global latency is off the critical
// path.  cp.async.wait_group is a hardware wait on this thread's own copies.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  unsigned a = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(a), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  unsigned a = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(a), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

// Copies tile t (keys [t*kTile, ...)) into shared memory.  Element i of the
// tile goes to slot i + (base & 3), so global and shared addresses agree
// modulo 16 bytes and the bulk of the tile moves with 16-byte cp.async
// whatever the tile's start.  Slots outside the tile may receive neighbouring
// keys; they are never read.  Stage buffers hold kTile + 4 slots.
template <bool kLoadVals>
__device__ __forceinline__ void rs_issue(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                                         int64_t t, int64_t n, uint32_t* sk, uint32_t* sv) {
  const int64_t base = t * kTile;
  const int32_t tn = (int32_t)(n - base < kTile ? n - base : kTile);
  const int r = (int)(base & 3);
  const int64_t a0 = base - r;                       // 16-byte aligned
  const int64_t a1 = base + tn;                      // one past the tile
  const int64_t full_end = a1 & ~(int64_t)3;         // last full 16-byte chunk inside the tile
  const int nfull = (int)((full_end - a0) >> 2);     // chunks [a0, full_end)
  for (int c = threadIdx.x; c < nfull; c += kBlock) {
    cp_async16(sk + 4 * c, kin + a0 + 4 * c);
    if (kLoadVals) cp_async16(sv + 4 * c, vin + a0 + 4 * c);
  }
  for (int64_t g = full_end + threadIdx.x; g < a1 && g < n; g += kBlock) {  // ragged tail
    cp_async4(sk + (g - a0), kin + g);
    if (kLoadVals) cp_async4(sv + (g - a0), vin + g);
  }
}

// Persistent downsweep over chunk blockIdx.x of the tiles (the same chunks as
// k_rs_upsweep_chunk).  The block walks its tiles in order and carries each
// digit's running output offset in a register (thread d owns digit d): it
// starts at the scanned chunk count hist[d * gridDim.x + blockIdx.x] and grows
// by the digit's count in every tile.  While one tile is ranked and
// scattered, the next two are already being copied into shared memory with
// cp.async (double buffer); cp.async.wait_group is a hardware wait on this
// thread's own copies.
// kFull: 8-bit digit; otherwise a digit of dbits < 8 bits.
template <bool kHasVals, bool kIota, bool kFull>
__global__ void __launch_bounds__(kBlock, 2) k_rs_downsweep_pipe(const uint32_t* __restrict__ kin,
                                                                 const uint32_t* __restrict__ vin,
                                                                 uint32_t* __restrict__ kout,
                                                                 uint32_t* __restrict__ vout, int shift, int dbits,
                                                                 int64_t ntiles, const uint32_t* __restrict__ hist,
                                                                 int64_t n) {
  constexpr bool kLoadVals = kHasVals && !kIota;
  extern __shared__ __align__(16) uint32_t dsm[];
  constexpr int kStage = kTile + 4;                       // slots per stage (alignment shift)
  uint32_t* in_k = dsm;                                   // [2][kStage]
  uint32_t* in_v = in_k + 2 * kStage;                     // [2][kStage] when kLoadVals
  uint32_t* out_k = in_v + (kLoadVals ? 2 * kStage : 0);  // [kTile]
  uint32_t* out_v = out_k + kTile;                        // [kTile] when kHasVals
  uint32_t* wcnt = out_v + (kHasVals ? kTile : 0);        // [kWarps][kRadix]
  uint32_t* st_ = wcnt + kWarps * kRadix;                 // [kRadix] tile-local digit starts
  uint32_t* adj = st_ + kRadix;                           // [kRadix] output offset minus tile-local start

  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t lt = lanemask_lt();
  const uint32_t dmask = kFull ? 255u : (1u << dbits) - 1u;
  int64_t t0, t1;
  chunk_tiles(ntiles, gridDim.x, blockIdx.x, &t0, &t1);
  // kBlock == kRadix; the upsweep ran kSubChunks parts per chunk
  uint32_t run = hist[(int64_t)threadIdx.x * gridDim.x * kSubChunks + (int64_t)blockIdx.x * kSubChunks];
  if (t0 < t1) rs_issue<kLoadVals>(kin, vin, t0, n, in_k, in_v);
  cp_async_commit();
  if (t0 + 1 < t1) rs_issue<kLoadVals>(kin, vin, t0 + 1, n, in_k + kStage, in_v + kStage);
  cp_async_commit();
  for (int i = threadIdx.x; i < kWarps * kRadix; i += kBlock) wcnt[i] = 0;

  for (int64_t t = t0; t < t1; ++t) {
    const int stg = (int)((t - t0) & 1);
    const int64_t tile_base = t * kTile;
    const int32_t tn = (int32_t)(n - tile_base < kTile ? n - tile_base : kTile);
    const int sh = (int)(tile_base & 3);  // alignment shift of this tile's slots
    const uint32_t* sk = in_k + stg * kStage + sh;
    const uint32_t* sv = in_v + stg * kStage + sh;
    cp_async_wait1();  // this thread's copies of tile t have landed
    __syncthreads();   // ... and everybody else's

    uint32_t k[kItems];
    uint32_t rank[kItems / 2];
    uint32_t peers[kItems];
    const bool full = tn == kTile;
#pragma unroll
    for (int i = 0; i < kItems; ++i) k[i] = sk[w * 32 * kItems + i * 32 + lane];
    // all items' peer masks first: their ballots are independent and pipeline
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      const int32_t lp = w * 32 * kItems + i * 32 + lane;
      const uint32_t d = (k[i] >> shift) & dmask;
      peers[i] = kFull ? match_digit8(d, full || lp < tn) : match_digit_n(d, full || lp < tn, dbits);
    }
    // then the per-warp digit counters, item by item (stable order)
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      const int32_t lp = w * 32 * kItems + i * 32 + lane;
      const bool valid = full || lp < tn;
      const uint32_t d = (k[i] >> shift) & dmask;
      const uint32_t before = valid ? wcnt[w * kRadix + d] : 0u;
      __syncwarp();
      const uint32_t r = __popc(peers[i] & lt);
      if (valid && r == 0) wcnt[w * kRadix + d] = before + __popc(peers[i]);
      __syncwarp();
      const uint32_t rk = before + r;
      if (i & 1)
        rank[i >> 1] |= rk << 16;
      else
        rank[i >> 1] = rk;
    }
    __syncthreads();
    uint32_t tot = 0;
    {
      const int d = threadIdx.x;  // kBlock == kRadix
#pragma unroll
      for (int q = 0; q < kWarps; ++q) {
        const uint32_t c = wcnt[q * kRadix + d];
        wcnt[q * kRadix + d] = tot;
        tot += c;
      }
    }
    const uint32_t start = block_excl_scan(tot, nullptr);
    st_[threadIdx.x] = start;
    adj[threadIdx.x] = run - start;  // output slot j of digit d -> adj[d] + j
    run += tot;
    __syncthreads();
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      const int32_t lp = w * 32 * kItems + i * 32 + lane;
      if (full || lp < tn) {
        const uint32_t d = (k[i] >> shift) & dmask;
        const uint32_t rk = (rank[i >> 1] >> ((i & 1) * 16)) & 0xFFFFu;
        const uint32_t pos = st_[d] + wcnt[w * kRadix + d] + rk;
        out_k[pos] = k[i];
        if (kHasVals) out_v[pos] = kIota ? (uint32_t)(tile_base + lp) : sv[lp];
      }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kWarps * kRadix; i += kBlock) wcnt[i] = 0;  // for the next tile
    for (int j = threadIdx.x; j < tn; j += kBlock) {
      const uint32_t key = out_k[j];
      const uint32_t gp = adj[(key >> shift) & dmask] + (uint32_t)j;
      kout[gp] = key;
      if (kHasVals) vout[gp] = out_v[j];
    }
    __syncthreads();  // stage stg and the staging buffers are free again
    if (t + 2 < t1) rs_issue<kLoadVals>(kin, vin, t + 2, n, in_k + stg * kStage, in_v + stg * kStage);
    cp_async_commit();
  }
}

// ---- ranked downsweep (digits of at most 7 bits) ------------------------------
// Tile t = keys [4096 t, 4096 t + 4096), seen through a 2-D tensor map as 128
// rows of 32 uint32 (rows of 128 bytes; the map covers the n / 32 full rows,
// so rows past it -- the ragged end of the last tile -- arrive as zeros and
// are fixed up by plain loads).  The TMA box {32, 128} lands in shared
// memory with the 128-byte swizzle: the 16-byte chunk c of row r is stored
// at chunk c ^ (r & 7).  Thread t owns the 16 consecutive keys 16t..16t+15
// (row t/2, chunks 4(t&1)..4(t&1)+3), so its four 16-byte reads, taken by a
// quarter warp at a time, hit eight different chunks of four rows: no bank
// conflicts.
constexpr int kRkMaxBits = 7;
constexpr int kRkDigits = 1 << kRkMaxBits;  // 128
constexpr int kRkQuads = kRkDigits / 4;     // byte-counter words per thread
constexpr int kRkGroups = kBlock / 16;      // 16 groups of 16 threads
// gt[g][d] (uint16) at g * kRkGtRow + d: word 65g + d/2, bank (g + d/2) % 32, so
// the scan's writes (one group per lane, one digit) and the rank's reads (2
// groups per warp, any digits) spread over the banks
constexpr int kRkGtRow = kRkDigits + 2;
constexpr uint32_t kRkTileBytes = kTile * 4;  // one array's tile: 16 KB
constexpr uint32_t kStatusWaitExpired = 2u;   // the status bit of a bounded wait that ran out
constexpr unsigned long long kRkWaitNs = 2000000000ull;  // 2 s: a TMA tile arrives in microseconds

struct RkSmem {  // byte offsets into the (1024-aligned) dynamic shared memory
  uint32_t stage[2];  // per stage: keys tile, then the values tile when present
  uint32_t cnt, gt, S, dtot, adj, mbar, total;
};
__host__ __device__ constexpr RkSmem rk_layout(bool has_vals) {
  const uint32_t stage_bytes = kRkTileBytes * (has_vals ? 2u : 1u);
  RkSmem L{};
  L.stage[0] = 0;
  L.stage[1] = stage_bytes;
  L.cnt = 2 * stage_bytes;                               // [kRkQuads][kBlock] u32: 4 byte counters
  L.gt = L.cnt + kRkQuads * kBlock * 4;                  // [kRkGroups][kRkGtRow] u16
  L.S = L.gt + kRkGroups * kRkGtRow * 2;                 // [kRkDigits] u32 digit start in the tile
  L.dtot = L.S + kRkDigits * 4;                          // [kRkDigits] u32 digit count in the tile
  L.adj = L.dtot + kRkDigits * 4;                        // [kRkDigits] u32 output offset - start
  L.mbar = L.adj + kRkDigits * 4;                        // 2 x u64
  L.total = L.mbar + 16;
  return L;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// Waits for the phase with the given parity, at most kRkWaitNs; false when
// the limit ran out.
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity) {
  if (mbar_try(bar, parity)) return true;  // the usual case: the tile is there; no timer read
  const unsigned long long t0 = global_ns();
  for (uint32_t it = 1;; ++it) {
    if (mbar_try(bar, parity)) return true;
    if ((it & 255u) == 0 && global_ns() - t0 > kRkWaitNs) return false;
  }
}
// Tile box {32 columns, 128 rows} at row `row` into shared memory dst.
__device__ __forceinline__ void tma_tile(uint32_t dst, const CUtensorMap* map, int32_t row, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
      "[%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(row), "r"(bar)
      : "memory");
}

// The issuing thread: refills stage stg with tile t (keys, and values when
// kLoadVals); returns the stage's pending bit.
template <bool kLoadVals>
__device__ __forceinline__ uint32_t rk_issue(const CUtensorMap* tm_k, const CUtensorMap* tm_v, uint32_t stage_sm,
                                             uint32_t stage_stride, uint32_t bar0, int64_t t, int stg) {
  const uint32_t bar = bar0 + 8u * stg;
  const uint32_t dst = stage_sm + stage_stride * stg;
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // generic accesses to the stage come first
  mbar_expect_tx(bar, kRkTileBytes * (kLoadVals ? 2u : 1u));
  tma_tile(dst, tm_k, (int32_t)(t * (kTile / 32)), bar);
  if (kLoadVals) tma_tile(dst + kRkTileBytes, tm_v, (int32_t)(t * (kTile / 32)), bar);
  return 1u << stg;
}

// Persistent downsweep of one pass with a digit of dbits <= 7 bits over the
// chunks of k_rs_upsweep_chunk (same count table as k_rs_downsweep_pipe).
// Per tile:
//   count  thread t adds each of its keys to its own byte counter of the
//          key's digit (word (d / 4, t), byte d % 4) with a shared-memory
//          atomic add, whose returned old value is the key's rank among the
//          thread's earlier keys of that digit (at most 15: one byte);
//   scan   per word of four digits, each half warp's lane g takes the 16
//          words of threads 16g..16g+15 (two words at once per warp): an
//          exclusive running sum of the words (byte-wise, at most 240
//          before the last word, so no carries) gives each thread's offset
//          inside its group, written back in place; the group totals, as
//          two words of 16-bit halves, take one 16-lane scan for the 16
//          groups (group offsets gt, digit totals);
//   starts warp 0 scans the digit totals (S = digit starts) and moves every
//          digit's running output offset, while every thread adds up the
//          rest of each key's position: gt[group][d] + in-group offset + own
//          rank (its loads overlap warp 0's scan);
//   rank   key position = S[d] + that sum: stable, since the order (digit,
//          thread, item) is the tile order within a digit; each key and its
//          value are stored there, in the tile's own stage buffer (the
//          thread holds them in registers);
//   write  each digit's run goes to its contiguous stretch of the output.
// Two stages: tile t+1 is in flight while tile t is ranked.  The stage of
// tile t - 1, written out at the end of the last iteration, is refilled with
// tile t + 1 during tile t's starts phase, by a lane of warp 1, which has
// slack there (warp 0 scans the digit starts).  A TMA wait is bounded
// (kRkWaitNs): if one ever runs out, the block sets kStatusWaitExpired in
// *status, waits (bounded again) for its copies still in flight, and ends.
template <bool kHasVals, bool kIota>
__global__ void __launch_bounds__(kBlock, 2) k_rs_downsweep_rank(const __grid_constant__ CUtensorMap tm_k,
                                                                 const __grid_constant__ CUtensorMap tm_v,
                                                                 const uint32_t* __restrict__ kin,
                                                                 const uint32_t* __restrict__ vin,
                                                                 uint32_t* __restrict__ kout,
                                                                 uint32_t* __restrict__ vout, int shift, int dbits,
                                                                 int64_t ntiles, const uint32_t* __restrict__ hist,
                                                                 int64_t n, uint32_t* __restrict__ status) {
  constexpr bool kLoadVals = kHasVals && !kIota;
  constexpr RkSmem L = rk_layout(kHasVals);
  constexpr uint32_t kStageBytes = kRkTileBytes * (kHasVals ? 2u : 1u);
  static_assert(L.stage[0] == 0 && L.stage[1] == kStageBytes, "stage s starts at s * kStageBytes");
  extern __shared__ unsigned char rk_raw[];
  unsigned char* base = rk_raw + ((1024u - (smem_u32(rk_raw) & 1023u)) & 1023u);
  uint32_t* cnt = reinterpret_cast<uint32_t*>(base + L.cnt);
  uint16_t* gt = reinterpret_cast<uint16_t*>(base + L.gt);
  uint32_t* S = reinterpret_cast<uint32_t*>(base + L.S);
  uint32_t* dtot = reinterpret_cast<uint32_t*>(base + L.dtot);
  uint32_t* adj = reinterpret_cast<uint32_t*>(base + L.adj);
  const uint32_t bar0 = smem_u32(base + L.mbar);

  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const uint32_t dmask = (1u << dbits) - 1u;
  const int nquads = ((1 << dbits) + 3) >> 2;
  int64_t t0, t1;
  chunk_tiles(ntiles, gridDim.x, blockIdx.x, &t0, &t1);
  const int64_t full_end = (n >> 5) << 5;  // keys covered by the tensor maps

  // warp 0, lane l: running output offsets of digits 4l..4l+3 (the scanned
  // count of this chunk's first upsweep part)
  uint32_t run[4] = {0, 0, 0, 0};
  if (w == 0) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int d = 4 * lane + k;
      if (d <= (int)dmask) run[k] = hist[(int64_t)d * gridDim.x * kSubChunks + (int64_t)blockIdx.x * kSubChunks];
    }
  }
  for (int i = tid; i < nquads * (kBlock / 4); i += kBlock) reinterpret_cast<uint4*>(cnt)[i] = make_uint4(0, 0, 0, 0);
  // Thread kIssuer (warp 1, lane 0) issues the tile copies, during the digit-
  // start phase, where warp 1 has slack; its bit s of pending: a copy into
  // stage s is in flight.
  constexpr int kIssuer = 32;
  uint32_t pending = 0;
  const uint32_t stage_sm = smem_u32(base);  // stage s at s * kStageBytes
  const uint32_t stage_stride = kStageBytes;
  if (tid == 0) {
    mbar_init(bar0, 1);
    mbar_init(bar0 + 8, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (tid == kIssuer && t0 < t1) pending |= rk_issue<kLoadVals>(&tm_k, &tm_v, stage_sm, stage_stride, bar0, t0, 0);

  for (int64_t t = t0; t < t1; ++t) {
    const int stg = (int)((t - t0) & 1);
    const bool arrived = mbar_wait_bounded(bar0 + 8u * stg, (uint32_t)(((t - t0) >> 1) & 1));
    if (tid == kIssuer && arrived) pending &= ~(1u << stg);
    uint32_t* sk = reinterpret_cast<uint32_t*>(base + (uint32_t)stg * kStageBytes);
    uint32_t* sv = reinterpret_cast<uint32_t*>(base + (uint32_t)stg * kStageBytes + kRkTileBytes);
    const int64_t tile_base = t * kTile;
    const int64_t my0 = tile_base + 16 * tid;
    uint32_t k[16], v[16];
    {
      const int r = tid >> 1;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int word = r * 32 + ((((tid & 1) * 4 + j) ^ (r & 7)) << 2);
        const uint4 q = *reinterpret_cast<const uint4*>(sk + word);
        k[4 * j] = q.x;
        k[4 * j + 1] = q.y;
        k[4 * j + 2] = q.z;
        k[4 * j + 3] = q.w;
        if (kLoadVals) {
          const uint4 u = *reinterpret_cast<const uint4*>(sv + word);
          v[4 * j] = u.x;
          v[4 * j + 1] = u.y;
          v[4 * j + 2] = u.z;
          v[4 * j + 3] = u.w;
        }
      }
    }
    if (my0 + 16 > full_end) {  // the last tile's ragged end: past the maps, or past n
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const int64_t p = my0 + i;
        if (p >= n) {
          k[i] = 0xFFFFFFFFu;  // after every key: the top digit, and later in tile order
        } else if (p >= full_end) {
          k[i] = __ldg(kin + p);
          if (kLoadVals) v[i] = __ldg(vin + p);
        }
      }
    }
    if (kIota) {
#pragma unroll
      for (int i = 0; i < 16; ++i) v[i] = (uint32_t)(my0 + i);
    }
    // count: own rank of every key among this thread's keys of its digit
    uint32_t own[2] = {0u, 0u};  // 16 nibbles
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const uint32_t d = (k[i] >> shift) & dmask;
      const uint32_t sh = (d & 3u) * 8u;
      const uint32_t old = atomicAdd(cnt + (d >> 2) * kBlock + tid, 1u << sh);
      own[i >> 3] |= ((old >> sh) & 0xFFu) << ((i & 7) * 4);
    }
    if (__syncthreads_or(!arrived)) {  // a tile never arrived: stop the block
      if (tid == kIssuer) {
        atomicOr(status, kStatusWaitExpired);
#pragma unroll
        for (int s2 = 0; s2 < 2; ++s2)
          if (pending & (1u << s2))
            mbar_wait_bounded(bar0 + 8u * s2, (uint32_t)((((t - t0) + (s2 != stg ? 1 : 0)) >> 1) & 1));
      }
      return;
    }
    // scan: in-group offsets in place, group offsets gt, digit totals.
    // Groups of 16 threads: lanes 0-15 take quad q, lanes 16-31 quad q + 8,
    // lane g of a half the 16 words of threads 16g..16g+15.  Lane g takes its
    // four 16-byte chunks starting at chunk r = (g >> 1) & 3, so that each
    // quarter warp's 16-byte accesses cover the 32 banks once.
    {
      const int g = lane & 15, hw = lane >> 4, r = (g >> 1) & 3;
      for (int q0 = w; q0 < nquads; q0 += 2 * kWarps) {
        const int q = q0 + kWarps * hw;
        const bool live = q < nquads;
        uint32_t* gw = cnt + q * kBlock + 16 * g;
        uint4 L[4], T[4], W[4];
#pragma unroll
        for (int j = 0; j < 4; ++j)
          L[j] = live ? *reinterpret_cast<const uint4*>(gw + 4 * ((j + r) & 3)) : make_uint4(0, 0, 0, 0);
#pragma unroll
        for (int c = 0; c < 4; ++c) T[c] = (r & 1) ? L[(c + 3) & 3] : L[c];
#pragma unroll
        for (int c = 0; c < 4; ++c) W[c] = (r & 2) ? T[(c + 2) & 3] : T[c];  // W[c] = chunk c
        // exclusive byte-wise running sum of the 16 words: at most 15 * 16 =
        // 240 per byte before the last word, so no carries; the group totals
        // (up to 256) are formed in 16-bit halves
        uint32_t acc = 0, e;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          e = acc; acc += W[c].x; W[c].x = e;
          e = acc; acc += W[c].y; W[c].y = e;
          e = acc; acc += W[c].z; W[c].z = e;
          if (c < 3) {
            e = acc; acc += W[c].w; W[c].w = e;
          }
        }
        const uint32_t last = W[3].w;
        W[3].w = acc;
        const uint32_t g02 = (acc & 0x00FF00FFu) + (last & 0x00FF00FFu);  // digits 4q+{0,2}
        const uint32_t g13 = ((acc >> 8) & 0x00FF00FFu) + ((last >> 8) & 0x00FF00FFu);  // digits 4q+{1,3}
#pragma unroll
        for (int c = 0; c < 4; ++c) T[c] = (r & 1) ? W[(c + 1) & 3] : W[c];
#pragma unroll
        for (int c = 0; c < 4; ++c) L[c] = (r & 2) ? T[(c + 2) & 3] : T[c];  // L[j] = chunk (j + r) & 3
        if (live) {
#pragma unroll
          for (int j = 0; j < 4; ++j) *reinterpret_cast<uint4*>(gw + 4 * ((j + r) & 3)) = L[j];
        }
        uint32_t i02 = g02, i13 = g13;
#pragma unroll
        for (int o = 1; o < 16; o <<= 1) {
          const uint32_t x = __shfl_up_sync(0xffffffffu, i02, o, 16), y = __shfl_up_sync(0xffffffffu, i13, o, 16);
          if (g >= o) {
            i02 += x;
            i13 += y;
          }
        }
        if (live) {
          const uint32_t e02 = i02 - g02, e13 = i13 - g13;
          uint16_t* gl = gt + g * kRkGtRow + 4 * q;
          gl[0] = (uint16_t)(e02 & 0xFFFFu);
          gl[1] = (uint16_t)(e13 & 0xFFFFu);
          gl[2] = (uint16_t)(e02 >> 16);
          gl[3] = (uint16_t)(e13 >> 16);
          if (g == 15) {
            dtot[4 * q + 0] = i02 & 0xFFFFu;
            dtot[4 * q + 1] = i13 & 0xFFFFu;
            dtot[4 * q + 2] = i02 >> 16;
            dtot[4 * q + 3] = i13 >> 16;
          }
        }
      }
    }
    __syncthreads();
    // the other stage's tile (t - 1) was written out in the last iteration:
    // refill it with tile t + 1
    if (tid == kIssuer && t + 1 < t1)
      pending |= rk_issue<kLoadVals>(&tm_k, &tm_v, stage_sm, stage_stride, bar0, t + 1, stg ^ 1);
    if (w == 0) {  // digit starts and output offsets, lane l: digits 4l..4l+3
      // entries of digits above dmask in the last word are zero counts (the
      // scan wrote them) and are never read back
      const uint4 c = lane < nquads ? *reinterpret_cast<const uint4*>(dtot + 4 * lane) : make_uint4(0, 0, 0, 0);
      const uint32_t sum = c.x + c.y + c.z + c.w;
      const uint32_t pre = warp_incl_scan(sum) - sum;
      if (lane < nquads) {
        const uint4 st = make_uint4(pre, pre + c.x, pre + c.x + c.y, pre + c.x + c.y + c.z);
        *reinterpret_cast<uint4*>(S + 4 * lane) = st;
        // output slot of tile position j of digit d: adj[d] + j
        *reinterpret_cast<uint4*>(adj + 4 * lane) = make_uint4(run[0] - st.x, run[1] - st.y, run[2] - st.z, run[3] - st.w);
        run[0] += c.x;
        run[1] += c.y;
        run[2] += c.z;
        run[3] += c.w;
      }
    }
    // partial positions (all but the digit start): their loads overlap warp
    // 0's digit starts
    uint32_t part[16];
    {
      const uint16_t* gg = gt + (tid >> 4) * kRkGtRow;
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const uint32_t d = (k[i] >> shift) & dmask;
        const uint32_t sh = (d & 3u) * 8u;
        const uint32_t in_group = (cnt[(d >> 2) * kBlock + tid] >> sh) & 0xFFu;
        part[i] = gg[d] + in_group + ((own[i >> 3] >> ((i & 7) * 4)) & 15u);
      }
    }
    __syncthreads();
    // rank and place into the stage buffer, now in digit order
    {
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const uint32_t d = (k[i] >> shift) & dmask;
        const uint32_t pos = S[d] + part[i];
        if (kHasVals)
          reinterpret_cast<uint2*>(sk)[pos] = make_uint2(k[i], v[i]);  // key and value as one word
        else
          sk[pos] = k[i];
      }
    }
    __syncthreads();
    for (int i = tid; i < nquads * (kBlock / 4); i += kBlock)  // for the next tile
      reinterpret_cast<uint4*>(cnt)[i] = make_uint4(0, 0, 0, 0);
    {
      const int tn = (int)(n - tile_base < kTile ? n - tile_base : kTile);
      auto put = [&](int j) {
        if (kHasVals) {
          const uint2 kv = reinterpret_cast<const uint2*>(sk)[j];
          const uint32_t gp = adj[(kv.x >> shift) & dmask] + (uint32_t)j;
          kout[gp] = kv.x;
          vout[gp] = kv.y;
        } else {
          const uint32_t key = sk[j];
          kout[adj[(key >> shift) & dmask] + (uint32_t)j] = key;
        }
      };
      if (tn == kTile) {
#pragma unroll 4
        for (int i = 0; i < kItems; ++i) put(tid + i * kBlock);
      } else {
        for (int j = tid; j < tn; j += kBlock) put(j);
      }
    }
    __syncthreads();  // stage stg is free again
  }
}

size_t rank_smem_bytes(bool has_vals) { return rk_layout(has_vals).total + 1024; }

// cuTensorMapEncodeTiled, looked up once through the runtime (no link-time
// dependence on the driver library).
using EncodeTiledFn = CUresult(CUDAAPI*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                         const cuuint64_t*, const cuuint32_t*, const cuuint32_t*,
                                         CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                         CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
  static std::once_flag once;
  static EncodeTiledFn fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
    cudaGetLastError();
  });
  return fn;
}

// Tensor map of a uint32 array of n keys as rows of 32 (the n / 32 full
// rows), boxes of 128 rows, 128-byte swizzle.  False when it cannot be made
// (n < 32, a base that is not 16-byte aligned, no entry point).
bool tile_map(CUtensorMap* m, const uint32_t* base, int64_t n) {
  EncodeTiledFn fn = encode_tiled();
  const int64_t rows = n >> 5;
  if (!fn || rows <= 0 || rows > ((int64_t)1 << 31) || (reinterpret_cast<uintptr_t>(base) & 15u)) return false;
  const cuuint64_t dims[2] = {32, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {128};
  const cuuint32_t box[2] = {32, (cuuint32_t)(kTile / 32)};
  const cuuint32_t estr[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, const_cast<uint32_t*>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <bool kHasVals, bool kIota>
cudaError_t launch_rank(const CUtensorMap& mk, const CUtensorMap& mv, const uint32_t* kin, const uint32_t* vin,
                        uint32_t* kout, uint32_t* vout, int shift, int dbits, int64_t ntiles, int64_t chunks,
                        const uint32_t* hist, int64_t n, uint32_t* status, cudaStream_t s) {
  static bool configured = false;  // per template instance
  const size_t smem = rank_smem_bytes(kHasVals);
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(k_rs_downsweep_rank<kHasVals, kIota>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  OWM_LAUNCH("k_rs_downsweep", s, (k_rs_downsweep_rank<kHasVals, kIota><<<(unsigned)chunks, kBlock, smem, s>>>(
      mk, mv, kin, vin, kout, vout, shift, dbits, ntiles, hist, n, status)));
  return cudaGetLastError();
}

template <bool kHasVals, bool kIota>
size_t pipe_smem_bytes() {
  constexpr bool kLoadVals = kHasVals && !kIota;
  return sizeof(uint32_t) * (2 * (kTile + 4) + (kLoadVals ? 2 * (kTile + 4) : 0) + kTile + (kHasVals ? kTile : 0) +
                             kWarps * kRadix + 2 * kRadix);
}

template <bool kHasVals, bool kIota, bool kFull>
cudaError_t launch_pipe_t(const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout, int shift,
                          int dbits, int64_t ntiles, int64_t chunks, const uint32_t* hist, int64_t n, cudaStream_t s) {
  static bool configured = false;  // per template instance
  const size_t smem = pipe_smem_bytes<kHasVals, kIota>();
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(k_rs_downsweep_pipe<kHasVals, kIota, kFull>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  OWM_LAUNCH("k_rs_downsweep", s, (k_rs_downsweep_pipe<kHasVals, kIota, kFull><<<(unsigned)chunks, kBlock, smem, s>>>(
      kin, vin, kout, vout, shift, dbits, ntiles, hist, n)));
  return cudaGetLastError();
}

template <bool kHasVals, bool kIota>
cudaError_t launch_pipe(const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout, int shift,
                        int dbits, int64_t ntiles, int64_t chunks, const uint32_t* hist, int64_t n, cudaStream_t s) {
  return dbits == 8 ? launch_pipe_t<kHasVals, kIota, true>(kin, vin, kout, vout, shift, dbits, ntiles, chunks, hist, n, s)
                    : launch_pipe_t<kHasVals, kIota, false>(kin, vin, kout, vout, shift, dbits, ntiles, chunks, hist, n, s);
}

}  // namespace

size_t scan_temp_bytes(int64_t n) {
  const int64_t parts = (n + kScanChunk - 1) / kScanChunk;
  size_t b = ((size_t)(parts + 64) * sizeof(uint32_t) + 255) & ~(size_t)255;
  if (parts > (int64_t)kScanChunk) b += scan_temp_bytes(parts);  // the partial sums are scanned the same way
  return b;
}

namespace {
int64_t sort_chunks(int64_t ntiles) {
  if (ntiles < 64) return 0;  // small sorts: one block per tile
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return std::min<int64_t>(std::min<int64_t>(ntiles, (int64_t)sms * 2), kMaxChunks);
}
}  // namespace

RadixSortPlan radix_sort_plan(int64_t n) {
  RadixSortPlan p;
  p.ntiles = (n + kTile - 1) / kTile;
  p.parts = sort_chunks(p.ntiles) * kSubChunks;
  return p;
}

size_t radix_sort_temp_bytes(int64_t n) {
  int64_t ntiles = (n + kTile - 1) / kTile;
  int64_t hn = hist_entries(ntiles);
  size_t hbytes = ((size_t)hn * sizeof(uint32_t) + 255) & ~(size_t)255;
  return hbytes + scan_temp_bytes(hn) + 256;
}

cudaError_t exclusive_scan_u32(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* total,
                               void* temp, size_t temp_bytes, cudaStream_t s, int64_t* launches) {
  if (n <= 0) {
    if (total) return cudaMemsetAsync(total, 0, sizeof(uint32_t), s);
    return cudaSuccess;
  }
  const int64_t parts = (n + kScanChunk - 1) / kScanChunk;
  if (temp_bytes < scan_temp_bytes(n) || n >= ((int64_t)1 << 40)) return cudaErrorInvalidValue;
  if (parts == 1) {  // one block does it all
    OWM_LAUNCH("k_scan_parts", s, k_scan_parts<<<1, kScanBlock, 0, s>>>(in, out, n, total));
    count_launch(launches);
    return cudaGetLastError();
  }
  uint32_t* part = static_cast<uint32_t*>(temp);
  OWM_LAUNCH("k_scan_reduce", s, k_scan_reduce<<<(unsigned)parts, kScanBlock, 0, s>>>(in, n, part));
  count_launch(launches, 2);
  if (parts <= (int64_t)kScanChunk) {  // each down-sweep block adds up the chunk totals before it
    OWM_LAUNCH("k_scan_down", s, k_scan_down<<<(unsigned)parts, kScanBlock, 0, s>>>(in, out, n, part, total));
    return cudaGetLastError();
  }
  // more than 2^26 values: scan the chunk totals in place, recursively; each
  // down-sweep block then reads its scanned offset
  const size_t pb = ((size_t)(parts + 64) * sizeof(uint32_t) + 255) & ~(size_t)255;
  cudaError_t e = exclusive_scan_u32(part, part, parts, total, static_cast<char*>(temp) + pb, temp_bytes - pb, s,
                                     launches);
  if (e != cudaSuccess) return e;
  OWM_LAUNCH("k_scan_down_scanned", s, k_scan_down_scanned<<<(unsigned)parts, kScanBlock, 0, s>>>(in, out, n, part));
  return cudaGetLastError();
}

cudaError_t radix_sort(uint32_t* k0, uint32_t* v0, uint32_t* k1, uint32_t* v1, int64_t n, int end_bit,
                       bool iota_vals, void* temp, size_t temp_bytes, cudaStream_t s, bool* in_alt,
                       int64_t* launches, bool first_counts_given, uint32_t* status) {
  *in_alt = false;
  if (n <= 0) return cudaSuccess;
  if (temp_bytes < radix_sort_temp_bytes(n) || end_bit <= 0 || end_bit > 32) return cudaErrorInvalidValue;
  const bool has_vals = v0 != nullptr;
  int64_t ntiles = (n + kTile - 1) / kTile;
  uint32_t* hist = static_cast<uint32_t*>(temp);
  size_t hbytes = ((size_t)hist_entries(ntiles) * sizeof(uint32_t) + 255) & ~(size_t)255;
  void* stemp = static_cast<char*>(temp) + hbytes;
  size_t sbytes = temp_bytes - hbytes;
  uint32_t *ka = k0, *va = v0, *kb = k1, *vb = v1;
  bool alt = false;
  bool first = true;
  // large sorts: one contiguous chunk of tiles per persistent block (two per SM)
  const int64_t chunks = sort_chunks(ntiles);
  if (first_counts_given && !chunks) return cudaErrorInvalidValue;
  // TMA views of the four buffers for the ranked downsweep (digits <= 7 bits)
  CUtensorMap maps[4];  // k0, k1, v0, v1
  bool maps_ok = chunks > 0 && tile_map(&maps[0], k0, n) && tile_map(&maps[1], k1, n);
  if (maps_ok && has_vals) maps_ok = tile_map(&maps[2], v0, n) && tile_map(&maps[3], v1, n);
  if (!maps_ok) maps[2] = maps[3] = maps[1] = maps[0];  // unused (pipe kernel); keeps them initialised
  if (maps_ok && !has_vals) maps[2] = maps[3] = maps[0];
  // where a bounded wait that runs out is recorded when the caller gives no status word
  uint32_t* st = status ? status : reinterpret_cast<uint32_t*>(static_cast<char*>(temp) + temp_bytes - 256);
  int pass = 0;
  const bool ranked = chunks > 0 && radix_ranked_widths(n, end_bit);  // digits of at most 7 bits
  for (int shift = 0; shift < end_bit; shift += radix_digit_bits(end_bit, pass++, ranked)) {
    // a pass sorts on bits [shift, shift + dbits); higher key bits are ignored
    const int dbits = radix_digit_bits(end_bit, pass, ranked);
    const uint32_t dmask = (1u << dbits) - 1u;
    if (chunks) {
      if (!(first && first_counts_given))
        OWM_LAUNCH("k_rs_upsweep", s, k_rs_upsweep_chunk<<<(unsigned)(chunks * kSubChunks), kBlock, 0, s>>>(
            ka, n, shift, dmask, hist, ntiles));
      // digit-major table: the live digits' counts come first, and only they
      // need offsets (no key has a digit >= 2^dbits)
      cudaError_t e = exclusive_scan_u32(hist, hist, (chunks * kSubChunks) << dbits, nullptr, stemp, sbytes, s, launches);
      if (e != cudaSuccess) return e;
      cudaError_t e2;
      if (maps_ok && dbits <= kRkMaxBits) {
        const CUtensorMap& mk = maps[alt ? 1 : 0];
        const CUtensorMap& mv = maps[alt ? 3 : 2];
        if (has_vals)
          e2 = (first && iota_vals)
                   ? launch_rank<true, true>(mk, mv, ka, va, kb, vb, shift, dbits, ntiles, chunks, hist, n, st, s)
                   : launch_rank<true, false>(mk, mv, ka, va, kb, vb, shift, dbits, ntiles, chunks, hist, n, st, s);
        else
          e2 = launch_rank<false, false>(mk, mv, ka, nullptr, kb, nullptr, shift, dbits, ntiles, chunks, hist, n, st,
                                         s);
      } else if (has_vals) {
        e2 = (first && iota_vals) ? launch_pipe<true, true>(ka, va, kb, vb, shift, dbits, ntiles, chunks, hist, n, s)
                                  : launch_pipe<true, false>(ka, va, kb, vb, shift, dbits, ntiles, chunks, hist, n, s);
      } else {
        e2 = launch_pipe<false, false>(ka, nullptr, kb, nullptr, shift, dbits, ntiles, chunks, hist, n, s);
      }
      if (e2 != cudaSuccess) return e2;
    } else {  // small sorts: one block per tile, per-tile counts
      OWM_LAUNCH("k_rs_upsweep", s, k_rs_upsweep<<<(unsigned)ntiles, kBlock, 0, s>>>(ka, n, shift, dmask, hist, ntiles));
      cudaError_t e = exclusive_scan_u32(hist, hist, ntiles << dbits, nullptr, stemp, sbytes, s, launches);
      if (e != cudaSuccess) return e;
      if (has_vals && first && iota_vals)
        OWM_LAUNCH("k_rs_downsweep", s, k_rs_downsweep<true, true><<<(unsigned)ntiles, kBlock, 0, s>>>(ka, va, kb, vb, n, shift, dmask, hist, ntiles));
      else if (has_vals)
        OWM_LAUNCH("k_rs_downsweep", s, k_rs_downsweep<true, false><<<(unsigned)ntiles, kBlock, 0, s>>>(ka, va, kb, vb, n, shift, dmask, hist, ntiles));
      else
        OWM_LAUNCH("k_rs_downsweep", s, k_rs_downsweep<false, false><<<(unsigned)ntiles, kBlock, 0, s>>>(ka, nullptr, kb, nullptr, n, shift, dmask, hist, ntiles));
    }
    count_launch(launches, (chunks && first && first_counts_given) ? 1 : 2);
    first = false;
    std::swap(ka, kb);
    std::swap(va, vb);
    alt = !alt;
  }
  *in_alt = alt;
  return cudaGetLastError();
}

}  // namespace owm
