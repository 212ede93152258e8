// Device-wide primitives: exclusive scan and an on-chip-staged LSD radix sort
// (8-bit digits, reduce-then-scan).
//
// Radix pass over a tile of 4096 keys per 256-thread block:
//   upsweep    digit histogram of the tile (vectorised 16-byte key loads)
//   scan       exclusive scan of the digit-major [256 x tiles] count table
//   downsweep  stable ranking inside the tile with __match_any_sync warp
//              multisplit, keys/values staged in shared memory in digit order,
//              then written out so that each digit's run is a contiguous,
//              coalesced stretch of the output.
#include <cuda_runtime.h>

#include <algorithm>

#include "owm_internal.cuh"

namespace owm {

namespace {

constexpr int kBlock = 256;
constexpr int kItems = 16;
constexpr int kTile = kBlock * kItems;  // 4096 keys
constexpr int kWarps = kBlock / 32;
constexpr int kRadix = 256;

constexpr int kScanBlock = 1024;
constexpr int kScanItems = 8;
constexpr int kScanChunk = kScanBlock * kScanItems;  // 8192 values per block

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
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

// Single block: exclusive scan of the partial sums (<= kScanChunk of them).
__global__ void k_scan_parts(uint32_t* part, int64_t nparts, uint32_t* total) {
  uint32_t v[kScanItems];
  uint32_t s = 0;
  for (int k = 0; k < kScanItems; ++k) {
    int64_t p = (int64_t)threadIdx.x * kScanItems + k;
    v[k] = p < nparts ? part[p] : 0u;
    s += v[k];
  }
  uint32_t tot;
  uint32_t off = block_excl_scan(s, &tot);
  for (int k = 0; k < kScanItems; ++k) {
    int64_t p = (int64_t)threadIdx.x * kScanItems + k;
    if (p < nparts) part[p] = off;
    off += v[k];
  }
  if (threadIdx.x == 0 && total) *total = tot;
}

__global__ void k_scan_down(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, int64_t n,
                            const uint32_t* __restrict__ part) {
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

// ---- radix sort --------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_rs_upsweep(const uint32_t* __restrict__ keys, int64_t n,
                                                       int shift, uint32_t* __restrict__ hist,
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
      atomicAdd(&h[w][(q.x >> shift) & 255u], 1u);
      atomicAdd(&h[w][(q.y >> shift) & 255u], 1u);
      atomicAdd(&h[w][(q.z >> shift) & 255u], 1u);
      atomicAdd(&h[w][(q.w >> shift) & 255u], 1u);
    }
  } else {
    for (int i = threadIdx.x; i < kTile; i += kBlock) {
      int64_t p = base + i;
      if (p < n) atomicAdd(&h[w][(keys[p] >> shift) & 255u], 1u);
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

template <bool kHasVals, bool kIota>
__global__ void __launch_bounds__(kBlock, 3) k_rs_downsweep(const uint32_t* __restrict__ kin,
                                                            const uint32_t* __restrict__ vin,
                                                            uint32_t* __restrict__ kout,
                                                            uint32_t* __restrict__ vout, int64_t n, int shift,
                                                            const uint32_t* __restrict__ hist, int64_t ntiles) {
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
    uint32_t d = valid ? ((k[i] >> shift) & 255u) : 256u;
    uint32_t peers = __match_any_sync(0xffffffffu, d);
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
      uint32_t d = (k[i] >> shift) & 255u;
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
    uint32_t d = (key >> shift) & 255u;
    uint32_t gp = s_glob[d] + (uint32_t)j - s_start[d];
    kout[gp] = key;
    if (kHasVals) vout[gp] = s_vals[j];
  }
}

}  // namespace

size_t scan_temp_bytes(int64_t n) {
  int64_t parts = (n + kScanChunk - 1) / kScanChunk;
  return (size_t)(parts + 64) * sizeof(uint32_t);
}

size_t radix_sort_temp_bytes(int64_t n) {
  int64_t ntiles = (n + kTile - 1) / kTile;
  int64_t hn = ntiles * kRadix;
  size_t hbytes = ((size_t)hn * sizeof(uint32_t) + 255) & ~(size_t)255;
  return hbytes + scan_temp_bytes(hn) + 256;
}

cudaError_t exclusive_scan_u32(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* total,
                               void* temp, size_t temp_bytes, cudaStream_t s, int64_t* launches) {
  if (n <= 0) {
    if (total) return cudaMemsetAsync(total, 0, sizeof(uint32_t), s);
    return cudaSuccess;
  }
  int64_t parts = (n + kScanChunk - 1) / kScanChunk;
  if (parts > (int64_t)kScanChunk || temp_bytes < scan_temp_bytes(n)) return cudaErrorInvalidValue;
  uint32_t* part = static_cast<uint32_t*>(temp);
  OWM_LAUNCH("k_scan_reduce", s, k_scan_reduce<<<(unsigned)parts, kScanBlock, 0, s>>>(in, n, part));
  OWM_LAUNCH("k_scan_parts", s, k_scan_parts<<<1, kScanBlock, 0, s>>>(part, parts, total));
  OWM_LAUNCH("k_scan_down", s, k_scan_down<<<(unsigned)parts, kScanBlock, 0, s>>>(in, out, n, part));
  count_launch(launches, 3);
  return cudaGetLastError();
}

cudaError_t radix_sort(uint32_t* k0, uint32_t* v0, uint32_t* k1, uint32_t* v1, int64_t n, int end_bit,
                       bool iota_vals, void* temp, size_t temp_bytes, cudaStream_t s, bool* in_alt,
                       int64_t* launches) {
  *in_alt = false;
  if (n <= 0) return cudaSuccess;
  if (temp_bytes < radix_sort_temp_bytes(n) || end_bit <= 0 || end_bit > 32) return cudaErrorInvalidValue;
  const bool has_vals = v0 != nullptr;
  int64_t ntiles = (n + kTile - 1) / kTile;
  int64_t hn = ntiles * kRadix;
  uint32_t* hist = static_cast<uint32_t*>(temp);
  size_t hbytes = ((size_t)hn * sizeof(uint32_t) + 255) & ~(size_t)255;
  void* stemp = static_cast<char*>(temp) + hbytes;
  size_t sbytes = temp_bytes - hbytes;
  uint32_t *ka = k0, *va = v0, *kb = k1, *vb = v1;
  bool alt = false;
  bool first = true;
  for (int shift = 0; shift < end_bit; shift += 8) {
    OWM_LAUNCH("k_rs_upsweep", s, k_rs_upsweep<<<(unsigned)ntiles, kBlock, 0, s>>>(ka, n, shift, hist, ntiles));
    cudaError_t e = exclusive_scan_u32(hist, hist, hn, nullptr, stemp, sbytes, s, launches);
    if (e != cudaSuccess) return e;
    if (has_vals) {
      if (first && iota_vals)
        OWM_LAUNCH("k_rs_downsweep", s, k_rs_downsweep<true, true><<<(unsigned)ntiles, kBlock, 0, s>>>(ka, va, kb, vb, n, shift, hist, ntiles));
      else
        OWM_LAUNCH("k_rs_downsweep", s, k_rs_downsweep<true, false><<<(unsigned)ntiles, kBlock, 0, s>>>(ka, va, kb, vb, n, shift, hist, ntiles));
    } else {
      OWM_LAUNCH("k_rs_downsweep", s, k_rs_downsweep<false, false><<<(unsigned)ntiles, kBlock, 0, s>>>(ka, nullptr, kb, nullptr, n, shift, hist, ntiles));
    }
    count_launch(launches, 2);
    first = false;
    std::swap(ka, kb);
    std::swap(va, vb);
    alt = !alt;
  }
  *in_alt = alt;
  return cudaGetLastError();
}

}  // namespace owm
