// Batched tiles: many independent clouds built and queried together.
#pragma once

#include <string>
#include <vector>

#include "owm_ctx.cuh"

namespace owm {

// Per-tile record read by the batched kernels (all offsets are global).
struct TileMeta {
  int64_t pt_off;   // first point in the concatenated point arrays
  int32_t n;        // points
  int32_t leaf;     // leaf size L (power of two <= 256)
  int32_t leaf_off; // first global leaf
  int32_t nleaves;
  int32_t node_off; // first global node: internal [0, nl-1), leaves [nl-1, 2nl-1)
  int32_t int_off;  // first global internal-node slot
  double mox, moy, mscale;  // Morton domain (square) of the tile
  int64_t mkx0, mky0;       // integer Morton form (mint): cell = (key(v) - k0) >> sh
  int32_t mshx, mshy, mint, mpad;
  double ox, oy;            // float-box origin (bbox corner)
  double min_x, min_y, displace;
  int32_t ncols, nrows, ncg, nrg;
  int32_t whalf, bhalf, bsize;
  uint32_t thr;     // minNumPoints as stage 1 compares it
  int32_t need_dup; // overlap > 0: LLPs are ids occurring >= 2 times
  int32_t pad;
  int64_t win_off, cell_off;
  int32_t ex_off, ey_off, cx_off, cy_off;
  int64_t bm_word;  // first 32-bit word of the tile's stage-2 bitmaps (ids 0..n)
};

// Host-side shape of one tile (what a batch signature is made of).
struct TileHost {
  const double* xyz;
  owm_params p;
  owm_tree_cfg tree;
};

// One batch in flight on one stream: device buffers sized for the largest
// batch seen (kept, so trees stay resident until the next batch reuses them),
// pinned host words for the per-tile output offsets, an optional CUDA graph.
struct BatchRun {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  DeviceBuffer mem;
  int64_t* h_off = nullptr;  // pinned [cap_tiles+1] per-tile output offsets, then the status word
  int64_t cap_tiles = 0;
  char* h_stage = nullptr;   // pinned staging of the per-batch tables (copies from it never block)
  size_t stage_cap = 0;
  int64_t launches = 0;
  bool use_graphs = false;
  cudaGraphExec_t graph = nullptr;
  std::string graph_sig;
  int32_t nclass = 0;
  int64_t class_bound[8] = {};
  int32_t class_leaf[8] = {};
  owm_tuning tuning = {4, 4, 256, 0};  // launch shapes (a batch takes its context's)
  // results of the last launch
  std::vector<TileHost> tiles;
  int64_t total_out = 0;
  int64_t* d_out = nullptr;
  int64_t* d_out_off = nullptr;
  uint32_t* d_status = nullptr;
  size_t bytes_needed = 0;
  cudaEvent_t done = nullptr;
  // With stage 1 by window classes, a side stream prepares the edge and class
  // tables and clears the stage-2/3 buffers while the keys are sorted, then
  // runs stages 1-2 and stage 3's LLP marks while `stream` builds the
  // hierarchies (fork, tables ready, gather done, join).
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_cls = nullptr, ev_gather = nullptr, ev_join = nullptr;

  int init(int device, cudaStream_t s);
  void destroy();
  int leaf_for(int64_t n, int32_t requested) const;
  // Estimated device bytes for these tiles (admission control).
  static size_t estimate_bytes(const owm_tile_desc* t, int32_t ntiles);
  // Enqueue everything (copies in, build, stages, offsets out) on `stream`.
  int launch(const owm_tile_desc* t, int32_t ntiles);
  // Wait for the launch and copy the seeds / offsets out.
  int finish(int64_t* seeds, int64_t cap, int64_t* offsets, owm_run_info* info);
  bool ready();
};

}  // namespace owm
