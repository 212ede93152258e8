// Internal device/host definitions shared by the OWM CUDA translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <cstdio>

#include "owm_gb300.h"

namespace owm {

// ---------------------------------------------------------------------------
// Order-preserving integer keys for IEEE doubles.
//
// For finite doubles a, b (with -0.0 folded to +0.0):  a < b  <=>
// key(a) < key(b) as signed int64.  Every containment and minimum test of the
// path is done on these keys, so the decisions equal the reference's FP64
// comparisons bit for bit while running on the integer pipes (GB300's FP64
// rate is low).
__host__ __device__ __forceinline__ int64_t dkey(double d) {
  int64_t b;
#ifdef __CUDA_ARCH__
  b = __double_as_longlong(d);
#else
  __builtin_memcpy(&b, &d, 8);
#endif
  if (b == (int64_t)0x8000000000000000ull) b = 0;  // -0.0 -> +0.0
  return b ^ ((b >> 63) & 0x7FFFFFFFFFFFFFFFll);
}
__host__ __device__ __forceinline__ double dkey_inv(int64_t k) {
  int64_t b = k ^ ((k >> 63) & 0x7FFFFFFFFFFFFFFFll);
  double d;
#ifdef __CUDA_ARCH__
  d = __longlong_as_double(b);
#else
  __builtin_memcpy(&d, &b, 8);
#endif
  return d;
}

// key(DBL_MAX): z of the reference's sentinel point 0 (optim3_func.cpp:708).
constexpr int64_t kZSentinel = 0x7FEFFFFFFFFFFFFFll;
constexpr int32_t kEnd = -1;  // end of a stackless walk

// (z, id) lexicographic "less": the reference's strict `<` on z plus a
// deterministic tie rule on the point id.
__host__ __device__ __forceinline__ bool zid_less(int64_t za, uint32_t ia, int64_t zb, uint32_t ib) {
  return za < zb || (za == zb && ia < ib);
}

// ---------------------------------------------------------------------------
// Hierarchy node (48 B = three 16-byte words, loaded as such by queries).
// Boxes are float offsets from the tree origin, rounded outward, so "fully
// inside" / "disjoint" decisions taken on them are always right and anything
// unsure falls to an exact per-point test.
struct __align__(16) Node {
  float x0, y0, x1, y1;  // outward-rounded box, relative to origin
  int64_t zmin;          // dkey of the minimum z under the node
  uint32_t min_id;       // 1-based id of that point
  uint32_t min_pos;      // its position in the sorted point arrays
  uint32_t count;        // points under the node
  int32_t left;          // internal: left child node; leaf: first point
  int32_t escape;        // next node of a depth-first walk after this subtree
  int32_t right;         // internal: right child; leaf: -1
};
static_assert(sizeof(Node) == 48, "Node must stay 48 bytes");

// Window / cell edge along one axis: exact keys for point tests, and the
// float offsets rounded down / up for node tests.
struct __align__(16) Edge {
  int64_t lo_k, hi_k;
  float lo_dn, lo_up, hi_dn, hi_up;
};
static_assert(sizeof(Edge) == 32, "Edge must stay 32 bytes");

// Device view of one tree (also one tile of a batch).
struct TreeView {
  const int64_t* xk;  // sorted point keys
  const int64_t* yk;
  const int64_t* zk;
  const uint32_t* pid;  // 1-based ids
  const Node* nodes;    // [2*nleaves-1]: internal 0..nl-2, leaves nl-1..
  int32_t nleaves;
  int32_t root;
  double ox, oy;        // origin of the float boxes
  // > 0: step limit of the bounded tree walks (stage-1 walk steps, stage-3
  // cell-walk rounds) in place of their structural bounds; lets a test make
  // a walk give up on a well-formed tree (owm_ctx_set_walk_limit)
  int32_t walk_limit = 0;
  int32_t cell_warps = 4;  // stage-3 cell walk: cells (warps) per block, 2, 4 or 8
  // Set when the build kept no sorted point arrays (xk, yk, zk and pid then
  // hold nothing): point p of the sorted order is record perm[p] of `rec`
  // (records of rec_stride doubles, x y z first), with id perm[p] + 1.  Only
  // the stage-3 cell walk reads points this way; builds for anything else
  // keep the arrays.
  const uint32_t* perm = nullptr;
  const double* rec = nullptr;
  int32_t rec_stride = 0;
};

// ---------------------------------------------------------------------------
// Error plumbing.
#define OWM_CUDA_TRY(expr)                                                          \
  do {                                                                              \
    cudaError_t _e = (expr);                                                        \
    if (_e != cudaSuccess) {                                                        \
      owm::set_last_cuda_error(_e, #expr, __FILE__, __LINE__);                      \
      return OWM_ECUDA;                                                             \
    }                                                                               \
  } while (0)

// Bytes the single-cloud point buffers keep readable past the last point, so
// that the build's gather may read whole 16-byte words (load_point16).
constexpr size_t kXyzSlack = 16;

void set_last_cuda_error(cudaError_t e, const char* what, const char* file, int line);
void set_last_error_text(const char* what);
const char* last_cuda_error();

// Library-wide kernel launch counter (every launch of this library's kernels
// goes through count_launch) and the per-context one.
void count_launch(int64_t* ctx_counter, int64_t k = 1);

// Per-kernel CUDA-event timing.  Every launch site is wrapped in OWM_LAUNCH;
// when the calling thread has an active profiler (set for the duration of an
// API call on a context with profiling on), an event pair is recorded on the
// launch stream around the kernel.
struct Profiler;
Profiler*& tls_profiler();
void prof_begin(const char* name, cudaStream_t s);
void prof_end(cudaStream_t s);
#define OWM_LAUNCH(name, stream, ...)      \
  do {                                     \
    if (owm::tls_profiler()) owm::prof_begin(name, stream); \
    __VA_ARGS__;                           \
    if (owm::tls_profiler()) owm::prof_end(stream);         \
  } while (0)

// ---------------------------------------------------------------------------
// Primitives (owm_sort.cu).
struct SortTemp {
  void* ptr = nullptr;
  size_t bytes = 0;
};
inline size_t align256ul(size_t b) { return (b + 255) & ~(size_t)255; }

// Temp bytes for sorting n keys (pairs or keys-only) and for scanning n ints.
size_t radix_sort_temp_bytes(int64_t n);
size_t scan_temp_bytes(int64_t n);

// LSD radix sort of uint32 keys (and optional uint32 values) on bits
// [0, end_bit); higher key bits are ignored.  Data ping-pongs between (k0,v0) and (k1,v1); *in_alt tells
// where the result is.  If iota_vals, the values of the first pass are the
// positions 0..n-1 (v0 is not read).  Stable.  With first_counts_given the
// caller has already written the first pass's digit counts (see
// RadixSortPlan) at the start of temp.
cudaError_t radix_sort(uint32_t* k0, uint32_t* v0, uint32_t* k1, uint32_t* v1, int64_t n, int end_bit,
                       bool iota_vals, void* temp, size_t temp_bytes, cudaStream_t s, bool* in_alt,
                       int64_t* launches, bool first_counts_given = false, uint32_t* status = nullptr);

// Digit width of pass `pass` of a sort on end_bit key bits: the fewest passes
// of at most 8 bits, or (ranked) of at most 7 bits, which the ranked
// downsweep handles; widths balanced (differing by at most one bit, wider
// first): 20 bits -> 7, 7, 6 either way; 23 -> 8, 8, 7 or 6, 6, 6, 5.
__host__ __device__ __forceinline__ int radix_digit_bits(int end_bit, int pass, bool ranked = false) {
  const int np = ranked ? (end_bit + 6) / 7 : (end_bit + 7) / 8;
  return end_bit / np + (pass < end_bit % np ? 1 : 0);
}
// Whether a large (chunked) sort of n keys on end_bit bits takes the ranked
// widths: when they need no more passes than 8-bit digits, or from 4 M keys
// (a ranked pass costs about 0.39 ms per 100 M keys and an 8-bit ballot-
// multisplit pass 0.69, each with about 12 us of upsweep, scan and launches:
// the extra pass pays from about 2.3 M keys for 23-24 bits, 5 M for 16).
// Producers that count the first digit (RadixSortPlan) use the same rule.
inline bool radix_ranked_widths(int64_t n, int end_bit) {
  return (end_bit + 6) / 7 == (end_bit + 7) / 8 || n >= ((int64_t)4 << 20);
}

// Layout of a large sort's count table, for producers of keys that also count
// the first pass's digits (bits 0..radix_digit_bits(end_bit, 0, radix_ranked_widths(n, end_bit))-1) on the fly.  The keys are split into
// `parts` contiguous ranges (sort_part_range); count[d * parts + p] is the
// number of keys of part p whose low byte is d, at the start of the sort's
// temp.  parts == 0: the sort takes its small-sort path (counts not given).
constexpr int64_t kSortTile = 4096;
struct RadixSortPlan {
  int64_t ntiles = 0, parts = 0;
};
RadixSortPlan radix_sort_plan(int64_t n);

// Tiles [*t0, *t1) of chunk b when ntiles tiles are split into g chunks.
__host__ __device__ __forceinline__ void chunk_tiles(int64_t ntiles, int64_t g, int64_t b, int64_t* t0, int64_t* t1) {
  const int64_t q = ntiles / g, r = ntiles % g;
  *t0 = b * q + (b < r ? b : r);
  *t1 = *t0 + q + (b < r ? 1 : 0);
}

// Keys [*b, *e) of part p of a plan for n keys (4 parts per downsweep chunk;
// a part may be empty).
__host__ __device__ __forceinline__ void sort_part_range(int64_t n, int64_t ntiles, int64_t parts, int64_t p,
                                                         int64_t* b, int64_t* e) {
  int64_t c0, c1, t0, t1;
  chunk_tiles(ntiles, parts / 4, p / 4, &c0, &c1);
  chunk_tiles(c1 - c0, 4, p % 4, &t0, &t1);
  t0 = (t0 + c0) * kSortTile;
  t1 = (t1 + c0) * kSortTile;
  *b = t0 < n ? t0 : n;
  *e = t1 < n ? t1 : n;
}

// Exclusive scan of n uint32 (in place allowed); *total (device) gets the sum
// when non-null.
cudaError_t exclusive_scan_u32(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* total,
                               void* temp, size_t temp_bytes, cudaStream_t s, int64_t* launches);

}  // namespace owm
