// Stage 1 by exact window classes: the reference's stage-1 result
// (stage1, CPP-TBB-CPU/src/optim3_func.cpp:541-561: per window the (z, id)-min
// of the points strictly inside and their count, kept when the count reaches
// minNumPoints) computed in O(N + windows) over the tree's sorted points.
//
// The window-class identity is in owm_classes.cuh.  Pipeline:
//   classes_prepare   edge keys per axis, s-range of every window column/row,
//                     class tables (cells of at most half a window step, so a
//                     point's class is one table read and two compares),
//                     counter resets
//   aggregation       per sorted point: its sub-cell; warp match + reduce of
//                     (count, (z, id)-min), then per group one atomic add and
//                     one 128-bit atomic min of the (z, id) pair (ties break
//                     on (z, id)) -- fused into the build's gather for
//                     owm_run, or k_cls_aggregate
//   k_cls_rows        per (window column, sub-cell row): reduce along x
//   k_cls_windows     per window: reduce along y, apply minNumPoints
// All integer: containment is exact by construction, and the search starts
// from the sentinel (z = DBL_MAX, id 0) like the reference, so an empty window
// with minNumPoints == 0 yields id 0.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "owm_classes.cuh"

namespace owm {

namespace {

constexpr int kClsBlock = 256;
constexpr int32_t kMaxTable = kClsMaxTable;

__global__ void k_cls_split(const Edge* __restrict__ e, int32_t n, int64_t* __restrict__ L, int64_t* __restrict__ R) {
  int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    L[i] = e[i].lo_k;
    R[i] = e[i].hi_k;
  }
}

__global__ void k_cls_table(const int64_t* __restrict__ L, const int64_t* __restrict__ R, int32_t n, int64_t k0,
                            int sh, int32_t Q, ClsCell* __restrict__ tab) {
  int32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < Q) tab[q] = cls_table_one(L, R, n, k0, sh, q);
}

__global__ void k_cls_ranges(const int64_t* __restrict__ L, const int64_t* __restrict__ R, int32_t n,
                             int32_t* __restrict__ s_lo, int32_t* __restrict__ s_hi) {
  int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) cls_range_one(L, R, n, i, s_lo + i, s_hi + i);
}

__global__ void __launch_bounds__(kClsBlock) k_cls_aggregate(ClassArgs A, const int64_t* __restrict__ xk,
                                                             const int64_t* __restrict__ yk,
                                                             const int64_t* __restrict__ zk,
                                                             const uint32_t* __restrict__ pid, int64_t n) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * kClsBlock) >> 5;
  for (int64_t wb = (((int64_t)blockIdx.x * kClsBlock + threadIdx.x) >> 5) * 32; wb < n; wb += nwarps * 32) {
    const int64_t pos = wb + lane;
    const bool valid = pos < n;
    const int64_t q = valid ? pos : wb;
    cls_aggregate_warp(A, valid, __ldg(xk + q), __ldg(yk + q), __ldg(zk + q), __ldg(pid + q), lane);
  }
}

__global__ void k_cls_rows(ClassArgs A) {
  const int64_t total = (int64_t)A.nx * A.ty;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (int64_t)gridDim.x * blockDim.x)
    cls_row_one(A, k);
}

__global__ void k_cls_windows(ClassArgs A, uint32_t thr, uint32_t* __restrict__ out) {
  const int64_t total = (int64_t)A.nx * A.ny;
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < total; w += (int64_t)gridDim.x * blockDim.x)
    out[cls_window_slot(A, w)] = cls_window_one(A, w, thr);
}

// The same, and each result also marks stage 2's occupancy bitmaps.
__global__ void k_cls_windows_marked(ClassArgs A, uint32_t thr, uint32_t* __restrict__ out, uint32_t* __restrict__ once,
                                     uint32_t* __restrict__ twice, uint32_t max_id) {
  const int64_t total = (int64_t)A.nx * A.ny;
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < total; w += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t v = cls_window_one(A, w, thr);
    out[cls_window_slot(A, w)] = v;
    s2_mark_id(once, twice, max_id, v);
  }
}

int grid(int64_t n, int block = 256) {
  int64_t g = (n + block - 1) / block;
  return (int)std::max<int64_t>(1, std::min<int64_t>(g, 152 * 32));
}

size_t a256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

bool cls_table_geometry(double lo, double hi, double step, int64_t* k0, int* sh, int32_t* Q) {
  if (!(lo > 0.0) || !(hi >= lo) || !(step > 0.0)) return false;
  int64_t blo, bhi;
  std::memcpy(&blo, &lo, 8);
  std::memcpy(&bhi, &hi, 8);
  if ((blo >> 52) != (bhi >> 52)) return false;
  int e = (int)((blo >> 52) & 0x7FF) - 1023;  // value = 1.m * 2^e, ulp = 2^(e-52)
  double cells = (step * 0.5) / std::ldexp(1.0, e - 52);  // key units in half a step
  if (!(cells >= 2.0)) return false;
  int s = 0;
  while (s < 62 && std::ldexp(1.0, s + 1) <= cells) ++s;
  int64_t q = ((dkey(hi) - dkey(lo)) >> s) + 1;
  if (q > kMaxTable) return false;
  *k0 = dkey(lo);
  *sh = s;
  *Q = (int32_t)q;
  return true;
}

size_t classes_scratch_bytes(int64_t n, int32_t ncols, int32_t nrows) {
  const int64_t tx = 2 * (int64_t)ncols + 1, ty = 2 * (int64_t)nrows + 1;
  (void)n;  // nothing per point: the sub-cell counters are the whole state
  return 2 * a256((size_t)kMaxTable * sizeof(ClsCell)) + 2 * a256((size_t)ncols * 8) +
         2 * a256((size_t)nrows * 8) + 2 * a256((size_t)ncols * 4) + 2 * a256((size_t)nrows * 4) +
         a256((size_t)(tx * ty) * 4) + a256((size_t)(tx * ty) * 16) +
         2 * a256((size_t)(ncols * ty) * 4) + a256((size_t)(ncols * ty) * 8) + 1024;
}

int classes_prepare(const owm_params& p, const Edge* ex, const Edge* ey, void* scratch, size_t scratch_bytes,
                    int64_t n, ClassArgs* A, cudaStream_t s, int64_t* launches) {
  const int32_t nc = (int32_t)p.ncols, nr = (int32_t)p.nrows;
  if (nc <= 0 || nr <= 0) return OWM_EINVAL;
  if (scratch_bytes < classes_scratch_bytes(n, nc, nr)) return OWM_ENOMEM;
  const int64_t tx = 2 * (int64_t)nc + 1, ty = 2 * (int64_t)nr + 1;
  if (tx * ty >= 0xFFFFFFFFll) return OWM_ERANGE;
  char* sp = static_cast<char*>(scratch);
  auto take = [&](size_t b) {
    void* q = sp;
    sp += a256(b);
    return q;
  };
  std::memset(A, 0, sizeof(*A));
  ClsCell* tabx = (ClsCell*)take((size_t)kMaxTable * sizeof(ClsCell));
  ClsCell* taby = (ClsCell*)take((size_t)kMaxTable * sizeof(ClsCell));
  int64_t* Lx = (int64_t*)take((size_t)nc * 8);
  int64_t* Rx = (int64_t*)take((size_t)nc * 8);
  int64_t* Ly = (int64_t*)take((size_t)nr * 8);
  int64_t* Ry = (int64_t*)take((size_t)nr * 8);
  A->sxl = (int32_t*)take((size_t)nc * 4);
  A->sxh = (int32_t*)take((size_t)nc * 4);
  A->syl = (int32_t*)take((size_t)nr * 4);
  A->syh = (int32_t*)take((size_t)nr * 4);
  A->count = (uint32_t*)take((size_t)(tx * ty) * 4);
  A->zid = (ulonglong2*)take((size_t)(tx * ty) * 16);
  A->rc = (uint32_t*)take((size_t)(nc * ty) * 4);
  A->rz = (unsigned long long*)take((size_t)(nc * ty) * 8);
  A->ri = (uint32_t*)take((size_t)(nc * ty) * 4);
  A->Lx = Lx;
  A->Rx = Rx;
  A->Ly = Ly;
  A->Ry = Ry;
  A->nx = nc;
  A->ny = nr;
  A->tx = (int32_t)tx;
  A->ty = (int32_t)ty;
  A->tabx = tabx;
  A->taby = taby;
  if (!cls_table_geometry(p.bbox.min_x, p.bbox.max_x, p.displace, &A->kx0, &A->shx, &A->qx)) A->qx = 0;
  if (!cls_table_geometry(p.bbox.min_y, p.bbox.max_y, p.displace, &A->ky0, &A->shy, &A->qy)) A->qy = 0;
  OWM_LAUNCH("k_cls_split", s, k_cls_split<<<(nc + 255) / 256, 256, 0, s>>>(ex, nc, Lx, Rx));
  OWM_LAUNCH("k_cls_split", s, k_cls_split<<<(nr + 255) / 256, 256, 0, s>>>(ey, nr, Ly, Ry));
  OWM_LAUNCH("k_cls_ranges", s, k_cls_ranges<<<(nc + 255) / 256, 256, 0, s>>>(Lx, Rx, nc, A->sxl, A->sxh));
  OWM_LAUNCH("k_cls_ranges", s, k_cls_ranges<<<(nr + 255) / 256, 256, 0, s>>>(Ly, Ry, nr, A->syl, A->syh));
  count_launch(launches, 4);
  if (A->qx) OWM_LAUNCH("k_cls_table", s, k_cls_table<<<(A->qx + 255) / 256, 256, 0, s>>>(Lx, Rx, nc, A->kx0, A->shx, A->qx, tabx));
  if (A->qy) OWM_LAUNCH("k_cls_table", s, k_cls_table<<<(A->qy + 255) / 256, 256, 0, s>>>(Ly, Ry, nr, A->ky0, A->shy, A->qy, taby));
  count_launch(launches, (A->qx > 0) + (A->qy > 0));
  OWM_CUDA_TRY(cudaMemsetAsync(A->count, 0, (size_t)(tx * ty) * 4, s));
  OWM_CUDA_TRY(cudaMemsetAsync(A->zid, 0xFF, (size_t)(tx * ty) * 16, s));
  OWM_CUDA_TRY(cudaGetLastError());
  return OWM_OK;
}

int classes_aggregate(const ClassArgs& A, const TreeView& t, int64_t n, cudaStream_t s, int64_t* launches) {
  int64_t blocks = std::min<int64_t>(((n + 31) / 32 * 32 + kClsBlock - 1) / kClsBlock, 152 * 8);
  OWM_LAUNCH("k_cls_aggregate", s, k_cls_aggregate<<<(unsigned)std::max<int64_t>(blocks, 1), kClsBlock, 0, s>>>(
      A, t.xk, t.yk, t.zk, t.pid, n));
  count_launch(launches);
  OWM_CUDA_TRY(cudaGetLastError());
  return OWM_OK;
}

int classes_finish(const ClassArgs& A, const TreeView& t, int64_t n, const owm_params& p, uint32_t* d_win,
                   cudaStream_t s, int64_t* launches) {
  (void)t;
  (void)n;
  OWM_LAUNCH("k_cls_rows", s, k_cls_rows<<<grid((int64_t)A.nx * A.ty), 256, 0, s>>>(A));
  OWM_LAUNCH("k_cls_windows", s, k_cls_windows<<<grid((int64_t)A.nx * A.ny), 256, 0, s>>>(A, p.min_num_points, d_win));
  count_launch(launches, 2);
  OWM_CUDA_TRY(cudaGetLastError());
  return OWM_OK;
}

int classes_finish_marked(const ClassArgs& A, const owm_params& p, uint32_t* d_win, uint32_t* once, uint32_t* twice,
                          uint32_t max_id, cudaStream_t s, int64_t* launches) {
  OWM_LAUNCH("k_cls_rows", s, k_cls_rows<<<grid((int64_t)A.nx * A.ty), 256, 0, s>>>(A));
  OWM_LAUNCH("k_cls_windows", s, k_cls_windows_marked<<<grid((int64_t)A.nx * A.ny), 256, 0, s>>>(
      A, p.min_num_points, d_win, once, twice, max_id));
  count_launch(launches, 2);
  OWM_CUDA_TRY(cudaGetLastError());
  return OWM_OK;
}

int run_stage1_classes(const TreeView& t, int64_t n, const owm_params& p, const Edge* ex, const Edge* ey,
                       uint32_t* d_win, void* scratch, size_t scratch_bytes, cudaStream_t s, int64_t* launches) {
  ClassArgs A;
  int rc = classes_prepare(p, ex, ey, scratch, scratch_bytes, n, &A, s, launches);
  if (!rc) rc = classes_aggregate(A, t, n, s, launches);
  if (!rc) rc = classes_finish(A, t, n, p, d_win, s, launches);
  return rc;
}

}  // namespace owm
