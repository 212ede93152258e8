// Query-side entry points (stages 1-3) shared by the API, batch and server.
#pragma once

#include "owm_build.cuh"

namespace owm {

constexpr uint32_t kNone = 0xFFFFFFFFu;  // "no minimum" (-1) in uint32 outputs

// One grid of query boxes (stage-1 windows or stage-3 cells) over one tree.
struct QueryJob {
  TreeView tree;
  const Edge* ex;       // [ncols]
  const Edge* ey;       // [nrows]
  int32_t ncols, nrows;
  uint32_t thr;         // minimum number of points strictly inside
  int32_t cell_order;   // 0: out[ii*nrows + jj] (stage 1); 1: out[jj*ncols + ii]
  int32_t patch_lx;     // a warp takes 2^patch_lx x 2^(5 - patch_lx) boxes (columns x rows)
  const uint8_t* skip;  // optional [ncols*nrows] in out order: box not queried
  uint32_t* out;        // id of the (z,id)-min point, or kNone
  uint32_t* status;     // device status word: kStatusWalkBound set if a walk overran
  int64_t warp_begin;   // first warp index of this job in a multi-job launch
};

// Status bits of the context's device status word.
constexpr uint32_t kStatusNonFinite = 1u;  // non-finite input coordinate
constexpr uint32_t kStatusWalkBound = 2u;  // a tree walk exceeded its step bound, or a bounded wait ran out

// Edge tables of the stage-1 windows (cells == false) or of the stage-3 cells
// (cells == true) of params p, float offsets relative to (ox, oy).
int compute_edges(const owm_params& p, double ox, double oy, bool cells, Edge* d_ex, Edge* d_ey, cudaStream_t s,
                  int64_t* launches);

// Number of warps a job needs (2^patch_lx x 2^(5 - patch_lx) boxes per warp).
int64_t job_warps(int32_t ncols, int32_t nrows, int32_t patch_lx);
// log2 of a power-of-two walk patch width (1..32).
inline int32_t patch_log2(int32_t patch_x) {
  int32_t l = 0;
  while ((1 << l) < patch_x && l < 5) ++l;
  return l;
}

// Runs jobs[0..njobs) (device array) whose warp ranges tile [0, total_warps).
// `name` labels the launch for the per-kernel profiler.
int launch_query(const QueryJob* d_jobs, int32_t njobs, int64_t total_warps, cudaStream_t s, int64_t* launches,
                 const char* name);
// Persistent variant: `blocks` resident blocks pull window patches from the
// device counter *d_next (reset here) -- load balance for uneven jobs.
int launch_query_persistent(const QueryJob* d_jobs, int32_t njobs, int64_t total_warps, unsigned long long* d_next,
                            int blocks, cudaStream_t s, int64_t* launches, const char* name);
// Single job convenience (job staged through a small device buffer).
int run_query(const QueryJob& job, QueryJob* d_job_slot, cudaStream_t s, int64_t* launches, const char* name);

// Stage 2 on n uint32 window results (kNone = no min): LLPs ascending into
// llp, their number into *d_count (device).  keys/alt/temp are scratch.
size_t stage2_scratch_bytes(int64_t n);
int run_stage2(const uint32_t* d_win, int64_t n, int64_t npoints, double overlap, uint32_t* d_llp,
               uint32_t* d_count, void* scratch, size_t scratch_bytes, cudaStream_t s, int64_t* launches);
// Same result, for overlap > 0 and ids known to lie in [0, npoints] (window
// minima of one cloud of npoints points), by occupancy bitmaps instead of a
// sort: one marking read of the window list, then work per 32 ids.  With
// cleared, the two bitmaps at the start of scratch were already zeroed by
// stage2_bitmap_clear (which may run early, on another stream).
size_t stage2_bitmap_scratch_bytes(int64_t npoints);
int stage2_bitmap_clear(void* scratch, size_t scratch_bytes, int64_t npoints, cudaStream_t s);
// With marked, the bitmaps were also marked already (by the stage-1 window
// kernel, s2_mark_id) and only the ascending emit remains.
int run_stage2_bitmap(const uint32_t* d_win, int64_t n, int64_t npoints, double overlap, uint32_t* d_llp,
                      uint32_t* d_count, void* scratch, size_t scratch_bytes, cudaStream_t s, int64_t* launches,
                      bool cleared = false, bool marked = false);
void stage2_bitmap_ptrs(void* scratch, int64_t npoints, uint32_t** once, uint32_t** twice);

// Stage 2's occupancy marks of one window result v (ids 0..max_id; kNone is
// skipped): the first occurrence sets `once`, a later one `twice`.
__device__ __forceinline__ void s2_mark_id(uint32_t* __restrict__ once, uint32_t* __restrict__ twice, uint32_t max_id,
                                           uint32_t v) {
  if (v > max_id) return;
  const uint32_t bit = 1u << (v & 31u);
  if (atomicOr(once + (v >> 5), bit) & bit) atomicOr(twice + (v >> 5), bit);
}
// Same with explicit working arrays (n uint32 each; d_llp must not alias
// them) and a temp block of radix_sort_temp_bytes(n) (256-aligned) +
// scan_temp_bytes(n).  d_win may equal k0.
int run_stage2_into(const uint32_t* d_win, uint32_t* k0, uint32_t* k1, uint32_t* flags, uint32_t* pos, int64_t n,
                    int64_t npoints, double overlap, uint32_t* d_llp, uint32_t* d_count, void* temp,
                    size_t temp_bytes, cudaStream_t s, int64_t* launches);

// Stage 3: mark cells holding an LLP (x, y read from the input points: AoS
// records of `stride` doubles, 3 or 4), query the rest, compact in cell
// order.  d_out gets the ids, *d_count their number.
size_t stage3_scratch_bytes(int64_t ngrid);
int run_stage3(const TreeView& t, const double* d_xyz, int stride, const owm_params& p, const uint32_t* d_llp,
               const uint32_t* d_nllp, int64_t llp_cap, uint32_t* d_out, uint32_t* d_count, void* scratch,
               size_t scratch_bytes, QueryJob* d_job_slot, uint32_t* status, cudaStream_t s, int64_t* launches);
// The same in three parts on one scratch layout: the cell edge tables (float
// offsets from (ox, oy), the tree's origin) and cleared marks (need nothing
// else), the LLP marks (need stage 2's list), then the queries and the
// compaction (need the tree hierarchy).
int run_stage3_prepare(double ox, double oy, const owm_params& p, void* scratch, size_t scratch_bytes,
                       cudaStream_t s, int64_t* launches);
int run_stage3_mark(const double* d_xyz, int stride, const owm_params& p, const uint32_t* d_llp, const uint32_t* d_nllp,
                    int64_t llp_cap, void* scratch, size_t scratch_bytes, cudaStream_t s, int64_t* launches);
int run_stage3_query(const TreeView& t, const owm_params& p, uint32_t* d_out, uint32_t* d_count, void* scratch,
                     size_t scratch_bytes, uint32_t* status, cudaStream_t s, int64_t* launches);

// Device kernels used by the API's conversions.
int u32_to_i64_ids(const uint32_t* in, const uint32_t* d_count, int64_t cap, int64_t* out, cudaStream_t s,
                   int64_t* launches);
int i64_to_u32_ids(const int64_t* in, int64_t n, uint32_t* out, cudaStream_t s, int64_t* launches);

}  // namespace owm
