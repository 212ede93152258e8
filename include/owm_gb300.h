/*
 * owm_gb300 -- C ABI of the GB300-native OWM ground-seed path.
 *
 * Drop-in boundary for the OWM path of PPMC-DAC/FastOWM.  The reference has
 * no FFI; its boundary is the set of free functions in
 * CPP-TBB-CPU/include/optim3_func.hpp:73-93 called by the driver
 * CPP-TBB-CPU/application/owm_optim3.cpp.  Each entry point below names the
 * reference function (file:line) it replaces.
 *
 * Conventions (all entry points):
 *   - return 0 (OWM_OK) or a negative OWM_E* status; owm_status_string()
 *     gives text.  Nothing calls exit() (the reference's mallocWrap does).
 *   - point ids are 1-based positions in the caller's input order, exactly
 *     the reference's cloud[] index (cloud[0] is the reference's sentinel
 *     {0, 0, DBL_MAX}); -1 means "no minimum" as in the reference's minIDs.
 *   - outputs are caller-allocated; sizes come from owm_params_compute().
 *     Output and input arrays may be host or device pointers (the library
 *     copies with cudaMemcpyDefault); host inputs should be pinned for speed.
 *   - every owm_ctx owns one CUDA stream; calls on one context are
 *     serialised by the caller; different contexts are independent.
 *   - there is no CPU fallback: without a CUDA device every compute entry
 *     point returns OWM_ECUDA.
 */
#ifndef OWM_GB300_H
#define OWM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OWM_OK 0
#define OWM_EINVAL (-1)   /* bad argument (also non-finite coordinates) */
#define OWM_ENOMEM (-2)   /* device or host allocation failed / over budget */
#define OWM_ECUDA (-3)    /* CUDA runtime error or no device */
#define OWM_ETIMEOUT (-4) /* bounded device wait expired (status word set) */
#define OWM_EIO (-5)      /* file could not be read / parsed */
#define OWM_ERANGE (-6)   /* caller's output capacity too small */
#define OWM_EAGAIN (-7)   /* result not ready yet (poll) */

/* Axis-aligned box of the cloud.  The reference takes it from the file
 * header, not from the data (optim3_func.cpp:665-700). */
typedef struct {
  double min_x, min_y, max_x, max_y;
} owm_bbox;

/* Derived OWM parameters, computed with the reference application's arithmetic
 * and integer types (owm_optim3.cpp:92-132): Width/Height = round2d(extent),
 * Density = N/(W*H), minNumPoints = (uint32)(0.5*Density*Wsize^2) passed on
 * as ushort, Displace = round2d(Wsize*(1-Overlap)), nCols/nRows as ushort,
 * nColsg = floor(Width/Bsize)+1. */
typedef struct {
  int64_t npoints;
  uint32_t wsize, bsize;
  double overlap;
  owm_bbox bbox;
  double width, height, density, displace;
  uint32_t min_num_points; /* value stage 1 compares against (ushort) */
  uint32_t ncols, nrows;   /* stage-1 windows along x / y */
  uint32_t ncols_grid, nrows_grid; /* stage-3 cells (0 when bsize == 0) */
  int64_t ncells;          /* ncols * nrows: stage-1 output length */
  int64_t ngrid;           /* ncols_grid * nrows_grid: max stage-3 output */
} owm_params;

/* Replaces the parameter block of owm_optim3.cpp:92-132 (+ round2d,
 * optim3_func.cpp:1-3).  overlap in [0,1), wsize >= 1, bsize >= 0
 * (0 disables stage 3 as in owm_optim3.cpp:192). */
int owm_params_compute(const owm_bbox* bbox, int64_t npoints, uint32_t wsize, double overlap,
                       uint32_t bsize, owm_params* out);

/* Exact min/max of x and y over n AoS points (host pointer). */
int owm_bbox_of(const double* xyz, int64_t n, owm_bbox* out);

/* ---- host cloud I/O ---------------------------------------------------- */

/* Replaces readXYZfile (optim3_func.cpp:665-722) for files that carry the
 * reference's header ("N\nminx\nmaxx\nminy\nmaxy\n", then one "x y z ..."
 * line per point; the rest of each line is skipped).  If the first line has
 * three or more numbers the file has no header: all lines are points and
 * the bbox is the data's min/max.  *xyz is malloc'd (free with
 * owm_host_free); it holds n points without the sentinel (id k+1 = row k). */
int owm_xyz_read(const char* path, double** xyz, int64_t* n, owm_bbox* bbox);
/* Writes "x y z" lines with %.2f like the reference's output dump
 * (owm_optim3.cpp:243-262) for the given 1-based ids. */
int owm_xyz_write_ids(const char* path, const double* xyz, int64_t n, const int64_t* ids,
                      int64_t n_ids);
void owm_host_free(void* p);

/* Tolerant correctness score of check_results (optim3_func.cpp:725-794):
 * the number of output points (ids into xyz) that find a gold point strictly
 * inside their displace/2 box with |dz| < 0.01, as a percentage of n_gold.
 * Id 0 is the reference's sentinel point {0, 0, DBL_MAX}, as in the
 * reference; ids above n are skipped.  Host-only helper for real-cloud runs. */
double owm_check_results(const double* gold_xyz, int64_t n_gold, const double* xyz, int64_t n,
                         const int64_t* ids, int64_t n_ids, float displace);

/* ---- synthetic clouds (seeded, bit-identical on x86-64 and aarch64) ---- */
typedef struct {
  int64_t n;
  double x0, y0, x1, y1;  /* area */
  double amplitude;       /* fBm terrain amplitude (m) */
  double wavelength;      /* base wavelength (m), 6 octaves */
  double noise_sigma;     /* ground noise sigma (m) */
  double lifted_frac;     /* fraction of points lifted */
  double lift_lo, lift_hi;/* lift height U(lo, hi) */
  double z_quantum;       /* >0: z rounded to this step (ties); 0: none */
  int32_t tie_free;       /* 1: z made unique by construction */
  int32_t strips;         /* 1: density in 60 m strips along y, U(5,60)/m2 */
  int32_t holes;          /* number of empty circular holes r~U(30,120) */
  int32_t _pad;
} owm_synth_spec;

/* Workload configs of the project (1..5) and tile index -> spec and OWM
 * knobs.  Config 1: 1 M pts uniform 200x250 m; 2: 100 M pts 2x2 km;
 * 3: 20 M pts strips + holes + 1 cm z; 4: batched tiles log-U[50k,2M];
 * 5: served tiles log-U[10k,5M]. seed = config*1000 + tile. */
int owm_synth_config(int config, int64_t tile, owm_synth_spec* spec, uint32_t* wsize,
                     double* overlap, uint32_t* bsize, int32_t* max_number, uint64_t* seed);
/* Fills xyz[3*n] and the exact data bbox.  nthreads <= 0: all cores. */
int owm_synth_cloud(const owm_synth_spec* spec, uint64_t seed, double* xyz, owm_bbox* bbox,
                    int nthreads);

/* ---- device context --------------------------------------------------- */
typedef struct owm_ctx owm_ctx;
int owm_ctx_create(int device, owm_ctx** out);
/* Destroy every tree and cloud made on a context before the context. */
int owm_ctx_destroy(owm_ctx* ctx);
int owm_ctx_sync(owm_ctx* ctx);
void* owm_ctx_stream(owm_ctx* ctx); /* the context's cudaStream_t */
/* Number of this library's kernel launches issued on the context so far. */
int64_t owm_ctx_launches(const owm_ctx* ctx);
/* Device status word: bit 0 non-finite input, bit 1 a bounded tree walk or
 * bounded device wait ran out (the call returned OWM_ETIMEOUT). */
int owm_ctx_device_status(owm_ctx* ctx, int32_t* status);
/* Step limit of this context's bounded tree walks: the stage-1 walk
 * (owm_stage1, stage1_walk = 1) stops after `limit` node steps per window and
 * the stage-3 cell walk after `limit` rounds per cell, instead of their
 * structural bounds (which only a corrupt hierarchy can reach).  A walk that
 * stops sets bit 1 of the device status word and its call returns
 * OWM_ETIMEOUT; the context stays usable.  0 restores the structural bounds.
 * For testing the failure path on a well-formed tree; no counterpart in the
 * reference, which has no bounded walk (it prints CUDA errors and goes on,
 * SYCL-CUDA-GPU/ordered/cuda/ordered_builder.inl:330-333). */
int owm_ctx_set_walk_limit(owm_ctx* ctx, int32_t limit);
/* Launch shapes of this context's kernels (owm_run, owm_tree_build,
 * owm_stage1, owm_stage3 and the batches made from the context).  Every
 * choice gives the same results; fastowm_gb300.autotune picks them by timing.
 * A field of 0 keeps its default.  No counterpart in the reference, whose
 * launch knobs are the leaf size (-s, owm_optim3.cpp:27) and the -DAUTOGRID
 * grid (SYCL-CUDA-GPU/ordered/cuda/ordered_builder.inl:306-313). */
typedef struct {
  int32_t walk_patch_x; /* stage-1 tree walk: each warp takes patch_x x (32 / patch_x)
                           windows; a power of two in 1..32 (default 4) */
  int32_t cell_warps;   /* stage-3 cell walk: cells (one warp each) per block: 2, 4 or 8
                           (default 4) */
  int32_t gather_block; /* build gather (one warp per leaf unit): threads per block:
                           128, 256 or 512 (default 256) */
  int32_t _pad;
} owm_tuning;
int owm_ctx_set_tuning(owm_ctx* ctx, const owm_tuning* tuning);
int owm_ctx_get_tuning(owm_ctx* ctx, owm_tuning* tuning);
/* Per-kernel CUDA-event timing of this context's launches (1 = on). */
int owm_ctx_set_profiling(owm_ctx* ctx, int on);
/* Sums the recorded kernel times by kernel name since the last call (and
 * clears them): names[k] (NUL-terminated), total ms and launch count;
 * *n = number of distinct kernels (OWM_ERANGE if more than cap). */
int owm_ctx_kernel_times(owm_ctx* ctx, int32_t cap, char (*names)[64], double* ms, int64_t* calls,
                         int32_t* n);

/* ---- device cloud ------------------------------------------------------ */
typedef struct owm_cloud owm_cloud;
/* Copies n AoS points (x, y, z doubles; host or device pointer) to the
 * device, where the cloud keeps each point as a 32-byte record (x, y, z,
 * pad), so that each random point read of the build's gather is one aligned
 * DRAM sector (a 24-byte point straddles two sectors half the time), and in a
 * compact x, y array for the passes that need no z: 48 bytes a point.  bbox
 * NULL = exact data min/max.  Replaces the cloud array built by readXYZfile. */
int owm_cloud_create(owm_ctx* ctx, const double* xyz, int64_t n, const owm_bbox* bbox,
                     owm_cloud** out);
int owm_cloud_destroy(owm_cloud* cloud);
int64_t owm_cloud_size(const owm_cloud* cloud);
/* The cloud's bbox (the header's or the data's, as the cloud was made). */
int owm_cloud_bbox(const owm_cloud* cloud, owm_bbox* out);
/* Copies the cloud's first n points (AoS x, y, z) to host memory. */
int owm_cloud_copy_out(const owm_cloud* cloud, double* xyz, int64_t n);
/* Cloud ingest on the GPU, replacing readXYZfile (optim3_func.cpp:665-722)
 * and map_file_atof_tbb_th (SYCL-CUDA-GPU/basic/utils.h:338-395).  Parses
 * the text of an .xyz file on the device with owm_xyz_read's rules (optional
 * header "N", "minx", "maxx", "miny", "maxy" on five lines; then one line
 * per point read as sscanf("%lf %lf %lf"); blank lines skipped; other short
 * lines, non-finite values and a short file are OWM_EIO; with a header the
 * lines after the declared count are not read).  Values are the correctly
 * rounded doubles of the C library's conversion, bit for bit.  bbox = the
 * header's, else the data's min/max.  `text` is host or device memory. */
int owm_cloud_parse_xyz(owm_ctx* ctx, const char* text, int64_t nbytes, owm_cloud** out);
/* Same for a file: read through pinned memory in 64 MB chunks, each chunk's
 * copy to the device overlapping the read of the next. */
int owm_cloud_load_xyz(owm_ctx* ctx, const char* path, owm_cloud** out);

/* ---- spatial index ----------------------------------------------------- */
#define OWM_TREE_MAX_NUMBER 1 /* leaves of <= max_number points (o4maxnum) */
#define OWM_TREE_MIN_RADIUS 0 /* leaves = quadtree cells of half-side <= min_radius */

typedef struct {
  int32_t policy;     /* OWM_TREE_MAX_NUMBER or OWM_TREE_MIN_RADIUS */
  int32_t max_number; /* leaf capacity, any value >= 1 (reference -s, default 32); leaves
                         hold at most this many points: the largest power of two not
                         above it, up to 256 (the seeds do not depend on it) */
  float min_radius;   /* reference -r, default 0.1 */
  int32_t level;      /* reference -L (CPU task split level); accepted, unused */
} owm_tree_cfg;

typedef struct {
  int64_t npoints, nleaves, nnodes;
  int64_t root_count;   /* points under the root (checkNumPoints analogue) */
  int64_t root_min_id;  /* id of the (z, id)-minimum of the whole cloud */
  int32_t max_leaf;     /* largest leaf */
  int32_t key_bits;     /* Morton key bits used by the sort */
} owm_tree_info;

typedef struct owm_tree owm_tree;
/* Replaces parallel_qtree + storeMinAndNumPoints (optim3_func.cpp:220-307):
 * Morton sort, leaves, Karras hierarchy, bottom-up (count, AABB, (z,id)-min)
 * refit, all on the device. */
int owm_tree_build(owm_ctx* ctx, const owm_cloud* cloud, const owm_tree_cfg* cfg,
                   owm_tree** out);
int owm_tree_get_info(owm_ctx* ctx, const owm_tree* tree, owm_tree_info* info);
/* Verifies that every internal node's count equals the sum of its children
 * (checkNumPoints, optim3_func.cpp:270-283); returns OWM_OK or OWM_EINVAL. */
int owm_tree_check(owm_ctx* ctx, const owm_tree* tree);
int owm_tree_destroy(owm_tree* tree);

/* ---- OWM stages -------------------------------------------------------- */
/* Replaces stage1 (optim3_func.cpp:541-561): win_min[ii*nrows + jj] = id of
 * the (z, id)-minimum point strictly inside window (ii, jj) if at least
 * min_num_points points are strictly inside, else -1.  [ncells] entries. */
int owm_stage1(owm_ctx* ctx, const owm_tree* tree, const owm_params* params, int64_t* win_min);

/* Replaces std::sort + stage2 (owm_optim3.cpp:160-188, optim3_func.cpp:
 * 610-625): sorts win_min in place and compacts every id that occurs at
 * least twice (overlap > 0) -- or every valid id (overlap == 0) -- to the
 * front in ascending order; *n_llp receives their number. */
int owm_stage2(owm_ctx* ctx, int64_t* win_min, int64_t ncells, double overlap, int64_t* n_llp);

/* Replaces the LLP grid + stage3 (owm_optim3.cpp:192-205, optim3_func.cpp:
 * 627-662): for every Bsize cell with no LLP strictly inside and at least
 * one point, the (z, id)-min point of the cell, in cell order (row jj
 * outer, column ii inner).  out needs cap >= ngrid entries. */
int owm_stage3(owm_ctx* ctx, const owm_tree* tree, const owm_params* params, const int64_t* llp,
               int64_t n_llp, int64_t* out, int64_t cap, int64_t* n_out);

/* Stage 2 without any device allocation.  No counterpart in the reference:
 * it exists for callers of this library that cannot allocate device memory
 * (a host that owns all GPU memory through its own pool, a plugin whose host
 * forbids allocation on the streams it lends, a real-time loop where an
 * allocation and its implicit synchronisation are not allowed).  Same
 * result as owm_stage2 (LLPs ascending), but d_win_min (int64, negative =
 * none) and d_llp (room for ncells ids) are caller-owned DEVICE memory, and
 * every id must lie in [0, npoints]: a larger id makes the call return
 * OWM_EINVAL (d_llp is then undefined).  The work runs on `stream` (a
 * cudaStream_t; NULL = the legacy default stream of the current device), on
 * the device that owns it (made current for the call, the caller's device
 * restored after), and the stream is synchronised before *n_llp is set.
 * Working memory is one static device array of about 21.5 MB that every
 * GPU loading this library holds until exit; at most 1,048,576 windows per
 * call (OWM_ERANGE above that).  The first call in each CUDA context of a
 * device looks up the array's address (cudaGetSymbolAddress).  All calls
 * share the array: calls that overlap on the GPU race, so serialise them. */
int owm_stage2_noalloc(void* stream, const int64_t* d_win_min, int64_t ncells, double overlap,
                       int64_t npoints, int64_t* d_llp, int64_t* n_llp);

/* ---- whole path -------------------------------------------------------- */
typedef struct {
  uint32_t wsize, bsize;
  double overlap;
  owm_tree_cfg tree;
  /* Stage-1 algorithm of owm_run (same result either way):
   *  0  exact window classes over the tree's sorted points: every point is
   *     assigned once to the sub-cell of windows that contain it, O(N);
   *  1  warp-cooperative stackless tree walk per window with min-z pruning
   *     (what owm_stage1 runs). */
  int32_t stage1_walk;
  int32_t _pad;
} owm_run_cfg;

/* Device time of the run (ms_total) and of its phases.  owm_run overlaps
 * them: with stage 1 by window classes, stages 1-2 run on a second stream
 * while the tree's hierarchy is built, so ms_stage1 counts from the end of
 * the build's gather, ms_stage3 from the end of both streams' work, and the
 * phases may add up to more than ms_total. */
typedef struct {
  double ms_tree, ms_stage1, ms_stage2, ms_stage3, ms_total;
  int64_t n_llp, n_stage3, n_seeds;
  owm_params params;
} owm_run_info;

/* Tree build + stages 1-3 on a device cloud; seeds = stage-3 ids followed
 * by the LLPs (owm_optim3.cpp:229-230).  cap >= ngrid + ncells is always
 * enough.  info may be NULL. */
int owm_run(owm_ctx* ctx, const owm_cloud* cloud, const owm_run_cfg* cfg, int64_t* seeds,
            int64_t cap, int64_t* n_seeds, owm_run_info* info);

/* Same from host points: host->device copy, build, stages, device->host
 * copy of the seeds, all on the context's stream. */
int owm_run_host(owm_ctx* ctx, const double* xyz, int64_t n, const owm_bbox* bbox,
                 const owm_run_cfg* cfg, int64_t* seeds, int64_t cap, int64_t* n_seeds,
                 owm_run_info* info);

/* Asynchronous form of owm_run_host, for streams of clouds: submit queues
 * the host->device copy of xyz (on a copy stream of the context), the run
 * and the device->host copy of the seeds, and returns a ticket at once; wait
 * blocks until that run is done and writes its seeds and counts.  Two runs
 * may be in flight per context, so the copy of one cloud overlaps the
 * compute of the other.  Tickets alternate between two slots: submit returns
 * OWM_EAGAIN while the run two tickets back has not been waited for.  xyz
 * (pinned for the copy to overlap) and seeds must stay valid until wait
 * returns.  Results are exactly those of owm_run_host.  No counterpart in
 * the reference, whose driver runs one cloud at a time synchronously. */
int owm_run_host_submit(owm_ctx* ctx, const double* xyz, int64_t n, const owm_bbox* bbox,
                        const owm_run_cfg* cfg, int64_t* seeds, int64_t cap, int64_t* ticket);
int owm_run_host_wait(owm_ctx* ctx, int64_t ticket, int64_t* n_seeds, owm_run_info* info);

/* Asynchronous form of owm_run on a device cloud: submit queues the run and
 * the device->host copy of the seeds and returns a ticket at once, so the
 * host work of the next submit (parameters, launches) overlaps this run on
 * the GPU; wait (owm_run_host_wait takes the same tickets) blocks until the
 * run is done and writes its seeds and counts.  Same two slots, OWM_EAGAIN
 * rule and results as owm_run_host_submit; the cloud and seeds must stay
 * valid until wait returns.  info's timings are left zero.  No counterpart
 * in the reference. */
int owm_run_submit(owm_ctx* ctx, const owm_cloud* cloud, const owm_run_cfg* cfg, int64_t* seeds,
                   int64_t cap, int64_t* ticket);
int owm_run_wait(owm_ctx* ctx, int64_t ticket, int64_t* n_seeds, owm_run_info* info);

/* ---- batched tiles ----------------------------------------------------- */
/* Many independent tiles (own bbox, Wsize, overlap, Bsize, leaf size) built
 * and queried together: one sort over all tiles, one launch per stage, with
 * per-tile work queues.  No reference counterpart (the reference runs one
 * cloud per process); results equal owm_run on each tile alone. */
typedef struct owm_batch owm_batch;
typedef struct {
  const double* xyz; /* host or device, n*3 doubles */
  int64_t n;
  owm_bbox bbox;     /* min_x > max_x: compute from data */
  owm_run_cfg cfg;
} owm_tile_desc;

int owm_batch_create(owm_ctx* ctx, owm_batch** out);
int owm_batch_destroy(owm_batch* b);
/* Runs ntiles tiles; seeds of tile t are seeds[offsets[t] .. offsets[t+1])
 * (offsets has ntiles+1 entries).  cap = total room in seeds.  Tiles whose
 * points already lie back to back in one device buffer (tile t+1 starting
 * right after tile t) are used in place; anything else is copied in. */
int owm_batch_run(owm_batch* b, const owm_tile_desc* tiles, int32_t ntiles, int64_t* seeds,
                  int64_t cap, int64_t* offsets, owm_run_info* total_info);
/* Capture the batch's device work into a CUDA graph keyed by the tile
 * shapes, and replay it when the same shapes come back (1 = on). */
int owm_batch_set_graphs(owm_batch* b, int enable);
/* Leaf size per size class: classes by point count, bounds[k] is the upper
 * bound of class k; leaf[k] in {16,32,64,128}.  nclass <= 8. */
int owm_batch_set_leaf_classes(owm_batch* b, int32_t nclass, const int64_t* bounds,
                               const int32_t* leaf);

/* ---- serving ----------------------------------------------------------- */
typedef struct owm_server owm_server;
typedef struct {
  int64_t hbm_budget_bytes; /* device bytes the server may hold */
  int32_t max_tiles_per_batch;
  int32_t max_inflight_batches; /* batches overlapping on the device */
  int64_t max_points_per_batch;
  int32_t use_graphs;
  /* 1: copy each tile's points into pinned staging at submit (the caller may
   * reuse its buffer at once); 0: borrow the caller's buffer until the ticket
   * is polled/waited (pinned host or device memory is fastest). */
  int32_t copy_on_submit;
} owm_server_cfg;

int owm_server_create(int device, const owm_server_cfg* cfg, owm_server** out);
int owm_server_destroy(owm_server* s);
/* Enqueue a tile; *ticket identifies it.  OWM_ENOMEM if the tile alone
 * exceeds the budget. */
int owm_server_submit(owm_server* s, const owm_tile_desc* tile, int64_t* ticket);
/* OWM_EAGAIN until done; then copies up to cap seeds, sets *n_seeds and
 * the tile's latency (submit -> result ready, ms) and releases it. */
int owm_server_poll(owm_server* s, int64_t ticket, int64_t* seeds, int64_t cap, int64_t* n_seeds,
                    double* latency_ms);
/* Blocking variant of poll with a timeout (ms); OWM_ETIMEOUT on expiry. */
int owm_server_wait(owm_server* s, int64_t ticket, int64_t* seeds, int64_t cap, int64_t* n_seeds,
                    double* latency_ms, double timeout_ms);
typedef struct {
  int64_t submitted, completed, batches, points_done;
  int64_t bytes_in_use, peak_bytes;
  double busy_ms;
} owm_server_stats;
int owm_server_get_stats(owm_server* s, owm_server_stats* st);

/* ---- misc -------------------------------------------------------------- */
const char* owm_status_string(int status);
/* Detail of the last CUDA failure behind an OWM_ECUDA on the calling thread:
 * the CUDA error text, the failing call and its source location ("" when
 * none).  No counterpart in the reference, which exits on errors. */
const char* owm_last_error(void);
int owm_version(void);

#ifdef __cplusplus
}
#endif
#endif /* OWM_GB300_H */
