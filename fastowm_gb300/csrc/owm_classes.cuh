// Stage 1 by exact window classes (see owm_classes.cu for the method).
//
// Along one axis let L[j] < R[j] be the window edges (order keys, both
// non-decreasing in j).  For a point key p
//     s(p) = #{j : L[j] < p} + #{j : R[j] <= p}
// is non-decreasing in p, and window i contains p (L[i] < p < R[i]) exactly
// when s(L[i] + 1) <= s(p) <= s(R[i] - 1).  Every point therefore falls in
// one (s_x, s_y) sub-cell, and each window is a rectangle of sub-cells.
#pragma once

#include "owm_query.cuh"

namespace owm {

// Everything the per-point classification needs (device pointers).
// Class-table cell of one axis: the left and right edges below its start
// (a = #{L < start}, b = #{R < start}) and the first of each at or after it
// (INT64_MAX when none).  A cell spans at most half a window step, so it
// holds at most one edge of each kind, and a point's sub-cell index is one
// 32-byte read away: a + b + (l < key) + (r <= key).
struct __align__(32) ClsCell {
  int64_t l, r;
  int32_t a, b;
  int32_t pad0, pad1;
};

struct ClassArgs {
  const int64_t *Lx, *Rx, *Ly, *Ry;  // edge keys per axis
  int32_t nx, ny;                     // window columns / rows
  const ClsCell *tabx, *taby;         // class tables (q* == 0: none)
  int64_t kx0, ky0;
  int32_t shx, shy, qx, qy;
  int32_t tx, ty;                     // sub-cell grid: 2*nx+1 by 2*ny+1
  uint32_t* count;                    // [tx*ty] points per sub-cell
  ulonglong2* zid;                    // [tx*ty] (z order key sign-flipped, id): the (z, id)-min
  int32_t *sxl, *sxh, *syl, *syh;     // s-range of every window column / row
  uint32_t *rc, *ri;                  // row reduction buffers [ty][nx]: sub-cell row t, window column ii
  unsigned long long* rz;
};

// Lower-bound style search of v in a[lo, hi) (non-decreasing a): first index
// whose element is >= v (le == false) or > v (le == true).
__device__ __forceinline__ int32_t cls_bsearch(const int64_t* a, int32_t lo, int32_t hi, int64_t v, bool le) {
  while (lo < hi) {
    int32_t mid = (lo + hi) >> 1;
    int64_t m = a[mid];
    if (le ? (m <= v) : (m < v)) lo = mid + 1; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ int64_t cls_wmin64(int64_t v) {
  for (int o = 16; o >= 1; o >>= 1) v = min(v, (int64_t)__shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ int64_t cls_wmax64(int64_t v) {
  for (int o = 16; o >= 1; o >>= 1) v = max(v, (int64_t)__shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// 128-bit compare-and-swap on global memory (sm_90+): *addr = {new_lo,
// new_hi} if it equals {cmp_lo, cmp_hi}; returns the value found.
__device__ __forceinline__ void cls_cas128(ulonglong2* addr, unsigned long long cmp_lo, unsigned long long cmp_hi,
                                           unsigned long long new_lo, unsigned long long new_hi,
                                           unsigned long long* old_lo, unsigned long long* old_hi) {
  asm volatile(
      "{\n\t.reg .b128 d, b, c;\n\t"
      "mov.b128 b, {%2, %3};\n\t"
      "mov.b128 c, {%4, %5};\n\t"
      "atom.global.cas.b128 d, [%6], b, c;\n\t"
      "mov.b128 {%0, %1}, d;\n\t}"
      : "=l"(*old_lo), "=l"(*old_hi)
      : "l"(cmp_lo), "l"(cmp_hi), "l"(new_lo), "l"(new_hi), "l"(addr)
      : "memory");
}

// Lexicographic atomic min of (z, id) in one 16-byte word.  Lock-free: a
// failed swap means another thread stored a smaller pair, and the stored pair
// only decreases, so the loop ends.  A stale first read is never below the
// stored pair, so returning early on it is safe.
__device__ __forceinline__ void cls_zid_min(ulonglong2* p, unsigned long long z, unsigned long long id) {
  ulonglong2 cur = __ldcg(p);
  while (z < cur.x || (z == cur.x && id < cur.y)) {
    unsigned long long lo, hi;
    cls_cas128(p, cur.x, cur.y, z, id, &lo, &hi);
    if (lo == cur.x && hi == cur.y) break;
    cur.x = lo;
    cur.y = hi;
  }
}

// Sub-cell index along one axis of a key that lies in table cell *e (below
// INT64_MAX, as every key inside a table does).
__device__ __forceinline__ int32_t cls_cell_index(const ClsCell* e, int64_t k) {
  int64_t l, r, ab;
  asm("ld.global.nc.v4.b64 {%0, %1, %2, _}, [%3];" : "=l"(l), "=l"(r), "=l"(ab) : "l"(e));
  return (int32_t)(uint32_t)ab + (int32_t)(ab >> 32) + (l < k) + (r <= k);
}

// All 32 lanes call this together, each with one point (valid or not).
// Folds the warp's points into their sub-cells: per group of lanes in one
// sub-cell, one atomic add of the count and one (z, id) atomic min.
__device__ __forceinline__ void cls_aggregate_warp(const ClassArgs& A, bool valid, int64_t px, int64_t py,
                                                   int64_t pz, uint32_t id, int lane) {
  int32_t sx = -1, sy = -1;
  if (A.qx > 0) {  // table: one read
    const int64_t q = (px - A.kx0) >> A.shx;
    if (q >= 0 && q < A.qx) sx = cls_cell_index(A.tabx + q, px);
  }
  if (A.qy > 0) {
    const int64_t q = (py - A.ky0) >> A.shy;
    if (q >= 0 && q < A.qy) sy = cls_cell_index(A.taby + q, py);
  }
  if (__any_sync(0xffffffffu, valid && (sx < 0 || sy < 0))) {
    // search: the warp's keys lie in [x0, x1] x [y0, y1], so every lane's
    // answer lies between those for the range ends; lanes 0..7 find the eight
    // bounds at once, then each lane searches its narrowed interval.
    const int64_t x0 = cls_wmin64(px), x1 = cls_wmax64(px), y0 = cls_wmin64(py), y1 = cls_wmax64(py);
    const int qq = lane & 7;
    const int64_t* arr = (qq < 2) ? A.Lx : (qq < 4) ? A.Rx : (qq < 6) ? A.Ly : A.Ry;
    const int32_t na = qq < 4 ? A.nx : A.ny;
    const int64_t v = (qq == 0) ? x0 : (qq == 1) ? x1 : (qq == 2) ? x0 - 1 : (qq == 3) ? x1
                    : (qq == 4) ? y0 : (qq == 5) ? y1 : (qq == 6) ? y0 - 1 : y1;
    const int32_t bnd = cls_bsearch(arr, 0, na, v, (qq & 3) != 0);  // '<' for qq = 0, 4
    const int32_t lx0 = __shfl_sync(0xffffffffu, bnd, 0), lx1 = __shfl_sync(0xffffffffu, bnd, 1);
    const int32_t rx0 = __shfl_sync(0xffffffffu, bnd, 2), rx1 = __shfl_sync(0xffffffffu, bnd, 3);
    const int32_t ly0 = __shfl_sync(0xffffffffu, bnd, 4), ly1 = __shfl_sync(0xffffffffu, bnd, 5);
    const int32_t ry0 = __shfl_sync(0xffffffffu, bnd, 6), ry1 = __shfl_sync(0xffffffffu, bnd, 7);
    if (sx < 0) sx = cls_bsearch(A.Lx, lx0, lx1, px, false) + cls_bsearch(A.Rx, rx0, rx1, px, true);
    if (sy < 0) sy = cls_bsearch(A.Ly, ly0, ly1, py, false) + cls_bsearch(A.Ry, ry0, ry1, py, true);
  }
  const uint32_t c = (uint32_t)sy * (uint32_t)A.tx + (uint32_t)sx;
  const unsigned long long zu = valid ? ((unsigned long long)pz ^ 0x8000000000000000ull) : ~0ull;
  const uint32_t peers = __match_any_sync(0xffffffffu, valid ? c : 0xFFFFFFFFu);
  if (valid) {
    const uint32_t hi = (uint32_t)(zu >> 32), lo = (uint32_t)zu;
    const uint32_t mh = __reduce_min_sync(peers, hi);
    const uint32_t ml = __reduce_min_sync(peers, hi == mh ? lo : 0xFFFFFFFFu);
    const uint32_t mid = __reduce_min_sync(peers, (hi == mh && lo == ml) ? id : 0xFFFFFFFFu);
    if (lane == __ffs(peers) - 1) {
      atomicAdd(A.count + c, (uint32_t)__popc(peers));
      cls_zid_min(A.zid + c, ((unsigned long long)mh << 32) | ml, mid);
    }
  }
}

// ---- per-element bodies, shared by the single-cloud and the batched kernels ----
constexpr int32_t kClsMaxTable = 1 << 16;  // class-table cells per axis, at most

__device__ __forceinline__ int32_t cls_count_less(const int64_t* a, int32_t n, int64_t v) {
  return cls_bsearch(a, 0, n, v, false);
}
__device__ __forceinline__ int32_t cls_count_le(const int64_t* a, int32_t n, int64_t v) {
  return cls_bsearch(a, 0, n, v, true);
}

// s-range [lo, hi] of window i along one axis (empty when lo > hi).
__device__ __forceinline__ void cls_range_one(const int64_t* L, const int64_t* R, int32_t n, int32_t i, int32_t* lo,
                                              int32_t* hi) {
  const int64_t a = L[i] + 1, b = R[i] - 1;
  *lo = cls_count_less(L, n, a) + cls_count_le(R, n, a);
  *hi = a <= b ? cls_count_less(L, n, b) + cls_count_le(R, n, b) : -1;
}

// Class-table cell q: (#{L < cell start}, #{R < cell start}) for cells of
// 2^sh keys from k0.
__device__ __forceinline__ ClsCell cls_table_one(const int64_t* L, const int64_t* R, int32_t n, int64_t k0, int sh,
                                              int32_t q) {
  const int64_t qs = k0 + ((int64_t)q << sh);
  ClsCell c;
  c.a = cls_count_less(L, n, qs);
  c.b = cls_count_less(R, n, qs);
  c.l = c.a < n ? L[c.a] : INT64_MAX;
  c.r = c.b < n ? R[c.b] : INT64_MAX;
  c.pad0 = c.pad1 = 0;
  return c;
}

__device__ __forceinline__ bool cls_zu_less(unsigned long long za, uint32_t ia, unsigned long long zb, uint32_t ib) {
  return za < zb || (za == zb && ia < ib);
}

// Row reduction k = ii * ty + t: sub-cells s of window column ii in sub-cell row t.
__device__ __forceinline__ void cls_row_one(const ClassArgs& A, int64_t k) {
  // k = t * nx + ii: neighbouring threads take neighbouring window columns of
  // one sub-cell row, so their sub-cell reads and row writes coalesce
  const int32_t t = (int32_t)(k / A.nx), ii = (int32_t)(k % A.nx);
  uint32_t c = 0, bi = 0xFFFFFFFFu;
  unsigned long long bz = ~0ull;
  const int64_t base = (int64_t)t * A.tx;
  for (int32_t s = A.sxl[ii]; s <= A.sxh[ii]; ++s) {
    c += A.count[base + s];
    const ulonglong2 e = A.zid[base + s];
    const unsigned long long z = e.x;
    const uint32_t id = (uint32_t)e.y;
    if (cls_zu_less(z, id, bz, bi)) {
      bz = z;
      bi = id;
    }
  }
  A.rc[k] = c;
  A.rz[k] = bz;
  A.ri[k] = bi;
}

// Window number w = jj * nx + ii (neighbouring threads take neighbouring
// window columns, so the row reads coalesce): reduce its rows, apply
// minNumPoints.  The search starts from the reference's sentinel point 0
// {0, 0, DBL_MAX}.  The result belongs at cls_window_slot(A, w).
__device__ __forceinline__ uint32_t cls_window_one(const ClassArgs& A, int64_t w, uint32_t thr) {
  const unsigned long long sentinel = (unsigned long long)kZSentinel ^ 0x8000000000000000ull;
  const int32_t jj = (int32_t)(w / A.nx), ii = (int32_t)(w % A.nx);
  uint32_t c = 0, bi = 0;
  unsigned long long bz = sentinel;
  for (int32_t t = A.syl[jj]; t <= A.syh[jj]; ++t) {
    const int64_t r = (int64_t)t * A.nx + ii;
    c += A.rc[r];
    if (cls_zu_less(A.rz[r], A.ri[r], bz, bi)) {
      bz = A.rz[r];
      bi = A.ri[r];
    }
  }
  return c >= thr ? bi : kNone;
}

// Output slot of window number w: the reference's order, ii * nrows + jj
// (stage1's step, optim3_func.cpp:541-561).
__device__ __forceinline__ int64_t cls_window_slot(const ClassArgs& A, int64_t w) {
  return (w % A.nx) * A.ny + w / A.nx;
}

// Class-table geometry over [lo, hi]: cells of 2^sh key units no wider than
// half the window step (keys are linear there when lo and hi share sign and
// exponent); false when no table applies (the per-point search then runs).
bool cls_table_geometry(double lo, double hi, double step, int64_t* k0, int* sh, int32_t* Q);

size_t classes_scratch_bytes(int64_t n, int32_t ncols, int32_t nrows);
// Carves the buffers from scratch and enqueues the edge split, s-ranges,
// class tables and counter resets for the windows of p (edge tables ex/ey).
int classes_prepare(const owm_params& p, const Edge* ex, const Edge* ey, void* scratch, size_t scratch_bytes,
                    int64_t n, ClassArgs* A, cudaStream_t s, int64_t* launches);
// Aggregation as its own pass over sorted points (when it is not fused into
// the build's gather).
int classes_aggregate(const ClassArgs& A, const TreeView& t, int64_t n, cudaStream_t s, int64_t* launches);
// Tie ids, row and window reductions: stage-1 results into d_win.
int classes_finish(const ClassArgs& A, const TreeView& t, int64_t n, const owm_params& p, uint32_t* d_win,
                   cudaStream_t s, int64_t* launches);
// The same, marking stage 2's occupancy bitmaps (zeroed) as each window
// result is produced (s2_mark_id); stage 2 then only emits the LLPs.
int classes_finish_marked(const ClassArgs& A, const owm_params& p, uint32_t* d_win, uint32_t* once, uint32_t* twice,
                          uint32_t max_id, cudaStream_t s, int64_t* launches);
// prepare + aggregate + finish.
int run_stage1_classes(const TreeView& t, int64_t n, const owm_params& p, const Edge* ex, const Edge* ey,
                       uint32_t* d_win, void* scratch, size_t scratch_bytes, cudaStream_t s, int64_t* launches);

}  // namespace owm
