// Tree storage and build entry points shared by the API, batch and server.
#pragma once

#include "owm_internal.cuh"

namespace owm {

// Device storage of one tree.  Point arrays hold `point_cap` entries, nodes
// `node_cap` (>= 2*nleaves-1).
struct TreeStore {
  int64_t* xk = nullptr;
  int64_t* yk = nullptr;
  int64_t* zk = nullptr;
  uint32_t* pid = nullptr;
  Node* nodes = nullptr;
  int64_t point_cap = 0, node_cap = 0;
  int64_t n = 0;
  int32_t nleaves = 0, root = 0, key_bits = 0, max_leaf = 0;
  int32_t gather_block = 256;  // threads per block of the build's gather (128, 256 or 512)
  double ox = 0, oy = 0;
  // points through the sort's permutation instead of the arrays (TreeView)
  const uint32_t* perm = nullptr;
  const double* rec = nullptr;
  int32_t rec_stride = 0;

  TreeView view(int32_t walk_limit = 0, int32_t cell_warps = 4) const {
    TreeView v;
    v.walk_limit = walk_limit;
    v.cell_warps = cell_warps;
    v.xk = xk;
    v.yk = yk;
    v.zk = zk;
    v.pid = pid;
    v.nodes = nodes;
    v.nleaves = nleaves;
    v.root = root;
    v.ox = ox;
    v.oy = oy;
    v.perm = perm;
    v.rec = rec;
    v.rec_stride = rec_stride;
    return v;
  }
};

// Leaf size of the max-number policy: the largest power of two not above
// max_number (nor above 256, the largest leaf the gather is built for), so
// every leaf holds at most max_number points.  The seeds do not depend on it;
// the reference's maxNumber takes any value.
constexpr int32_t kMaxLeaf = 256;
inline int32_t leaf_size(int32_t max_number) {
  int32_t L = 1;
  while (L * 2 <= max_number && L * 2 <= kMaxLeaf) L *= 2;
  return L;
}

// Node slots needed for n points under a tree configuration.
inline int64_t tree_node_cap(int64_t n, const owm_tree_cfg& cfg) {
  const int64_t L = leaf_size(cfg.max_number);
  int64_t nl = cfg.policy == OWM_TREE_MAX_NUMBER ? (n + L - 1) / L : n;
  return 2 * nl - 1;
}

size_t tree_scratch_bytes(int64_t n);
// Integer Morton quantisation of [lo, hi]: true (and the key origin and
// shift) when lo, hi > 0 share their exponent, so order keys are linear.
bool morton_int_shifts(double lo, double hi, int bits, int64_t* klo, int* shift);
int choose_key_bits(int64_t n, int policy, double side, float min_radius, int32_t leaf);

// Device points as the kernels read them: `rec`, AoS records of rec_stride
// doubles for the random reads of the gather (4: a cloud's 32-byte records
// x, y, z, pad, 32-byte aligned; 3: plain x, y, z, 16-byte aligned with
// kXyzSlack readable bytes after the last point), and `xy`, x and y of point i
// at xy[xy_stride * i] and the next double, for the streaming reads that need
// no z (the Morton pass, a bbox, stage 3's LLP marks): 2 for a cloud's x, y
// array, 3 for plain points (then xy == rec).
struct PointsView {
  const double* rec;
  int rec_stride;
  const double* xy;
  int xy_stride;
};
inline PointsView plain_points(const double* xyz) { return PointsView{xyz, 3, xyz, 3}; }

// Builds the tree of n device points into t (whose arrays must be allocated
// with enough capacity).  Scratch is caller-provided.
// Non-finite input coordinates set bit 0 of *status (device word).  With cls,
// the fixed-leaf gather also folds every point into the stage-1 window
// classes (*fused says whether it did; the min-radius build does not); when
// cls_ready is given, s waits on it right before that gather, so the class
// tables may be prepared on another stream while the keys are sorted, and
// gather_done (if given) is recorded on s right after that gather, so the
// classes may be finished on another stream while the hierarchy is built.
struct ClassArgs;
int build_tree(const PointsView& pts, int64_t n, const owm_bbox& bbox, const owm_tree_cfg& cfg, TreeStore* t,
               void* scratch, size_t scratch_bytes, uint32_t* status, cudaStream_t s, int64_t* launches,
               const ClassArgs* cls = nullptr, bool* fused = nullptr, cudaEvent_t cls_ready = nullptr,
               cudaEvent_t gather_done = nullptr);

// Structural self-check (checkNumPoints); *h_bad = number of bad nodes.
int check_tree(const TreeStore* t, int32_t* d_bad, cudaStream_t s, int64_t* launches, int32_t* h_bad);

}  // namespace owm
