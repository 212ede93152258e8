// ORACLE / TEST INFRASTRUCTURE -- never part of the shipped product.
//
// Links the reference's own OWM CPU path (CPP-TBB-CPU/src/optim3_func.cpp,
// pulled in through CPP-TBB-CPU/include/optim3_func.hpp:95) unmodified, and
// exposes it as one C function so tests and the CPU baseline can drive it on
// an in-memory cloud.  TBB / oneDPL are replaced by the scheduling-only
// stand-ins under oracle/shim.
//
// What this file adds is the reference application's glue, restated from
// CPP-TBB-CPU/application/owm_optim3.cpp:
//   * cloud with sentinel point 0 = {0, 0, DBL_MAX}   (optim3_func.cpp:702-708)
//   * getRadius / getCenter -> parallel_qtree -> storeMinAndNumPoints
//                                                     (owm_optim3.cpp:67-88)
//   * Width/Height/Density/minNumPoints/Displace/nCols/nRows/nColsg/nRowsg
//                                                     (owm_optim3.cpp:92-132)
//   * stage1 (exact, -DNOMEMOA) or stage1memoA, std::sort, stage2, grid
//     quadtree of the LLPs, stage3                    (owm_optim3.cpp:143-205)
//   * output = stage-3 ids followed by the LLPs       (owm_optim3.cpp:229-230)
// The parameter arithmetic keeps the reference's types (uint32 / ushort /
// float radius) so truncations match.
#include "optim3_func.hpp"

#include <cfloat>
#include <cstdint>
#include <cstring>
#include <string>

extern "C" {

struct owmref_result {
  int64_t n_llp;      // number of stage-2 LLPs (last n_llp entries of seeds)
  int64_t n_stage3;   // number of stage-3 seeds (first n_stage3 entries)
  int64_t ncells;     // nCols * nRows
  int64_t ngrid;      // nColsg * nRowsg
  uint32_t min_num_points;  // value passed to stage1 (ushort-truncated)
  uint32_t ncols, nrows, ncols_grid, nrows_grid;
  double displace;
  double t_tree;      // seconds, tree build + memo refit
  double t_owm;       // seconds, mean over `loops` runs of stages 1..3
  double t_stage1;    // seconds, last run
  double t_stage2;
  double t_stage3;
};

// xyz: n points, AoS {x,y,z}, point k (0-based) becomes reference id k+1.
// bbox: {min_x, min_y, max_x, max_y} (the reference takes it from the file
// header, not from the data).
// policy: 0 = minRadius quadtree, 1 = maxNumber quadtree.
// memoA: 0 = exact stage1 (o3memoB), 1 = stage1memoA (o3memo, approximate).
// win_min: optional [ncells] copy of stage-1 output in step order.
// seeds: [seeds_cap] stage-3 ids then LLPs.  Returns 0, or -1 on bad input,
// -2 if seeds_cap is too small, -3 if win_min_cap is too small.
int owmref_run(const double* xyz, int64_t n, const double* bbox, uint32_t Wsize,
               uint32_t Bsize, double Overlap, int policy, float minRadius,
               int maxNumber, int level, int nthreads, int memoA, int loops,
               int* win_min, int64_t win_min_cap, int* seeds, int64_t seeds_cap,
               owmref_result* res) {
  if (n <= 0 || n >= 0xFFFFFFFFLL || Overlap <= 0.0 || Overlap >= 1.0 || loops < 1) return -1;
  tbb::global_control gc{tbb::global_control::max_allowed_parallelism,
                         (size_t)(nthreads > 0 ? nthreads : 1)};

  uint32_t Npoints = (uint32_t)n + 1;  // + sentinel
  Lpoint* cloud = static_cast<Lpoint*>(mallocWrap(Npoints * sizeof(Lpoint)));
  cloud[0] = {0.0, 0.0, std::numeric_limits<double>::max()};
  std::memcpy(&cloud[1], xyz, (size_t)n * sizeof(Lpoint));
  Vector2D min = {bbox[0], bbox[1]}, max = {bbox[2], bbox[3]};

  float maxRadius = 0.0;
  Vector2D radius = getRadius(min, max, maxRadius);
  Vector2D center = getCenter(min, radius);

  tbb::tick_count t0 = tbb::tick_count::now();
  Qtree qtreeIn = policy == 1 ? parallel_qtree(level, center, maxRadius, cloud, Npoints, maxNumber)
                              : parallel_qtree(level, center, maxRadius, cloud, Npoints, minRadius);
  storeMinAndNumPoints(cloud, qtreeIn, 0);
  double time_tree = (tbb::tick_count::now() - t0).seconds();

  double Width = round2d(max.x - min.x);
  double Height = round2d(max.y - min.y);
  double Density = (Npoints - 1) / (Width * Height);
  uint32_t minNumPoints = 0.5 * Density * Wsize * Wsize;
  double Displace = round2d(Wsize * (1 - Overlap));
  ushort nCols = (int)(round((Width + 2 * Wsize * Overlap) / Displace)) - 1;
  ushort nRows = (int)(round((Height + 2 * Wsize * Overlap) / Displace)) - 1;
  uint32_t Ncells = nCols * nRows;
  ushort nColsg = (int)floor(Width / Bsize) + 1;
  ushort nRowsg = (int)floor(Height / Bsize) + 1;
  uint32_t Ngrid = nColsg * nRowsg;

  res->ncells = Ncells;
  res->ngrid = Ngrid;
  res->min_num_points = (ushort)minNumPoints;
  res->ncols = nCols;
  res->nrows = nRows;
  res->ncols_grid = nColsg;
  res->nrows_grid = nRowsg;
  res->displace = Displace;
  res->t_tree = time_tree;

  if (win_min && win_min_cap < (int64_t)Ncells) {
    deleteQtree(qtreeIn);
    delete qtreeIn;
    free(cloud);
    return -3;
  }

  int* minIDs = new int[Ncells];
  std::vector<int> minGridIDs;
  uint32_t numLLPs = 0;
  double t_sum = 0;
  for (int run = 0; run < loops; ++run) {
    tbb::tick_count tf = tbb::tick_count::now();
    tbb::tick_count ts = tf;
    if (memoA)
      stage1memoA(Wsize, Overlap, nCols, nRows, minNumPoints, minIDs, cloud, qtreeIn, min);
    else
      stage1(Wsize, Overlap, nCols, nRows, minNumPoints, minIDs, cloud, qtreeIn, min);
    res->t_stage1 = (tbb::tick_count::now() - ts).seconds();
    if (win_min && run == loops - 1) std::memcpy(win_min, minIDs, Ncells * sizeof(int));

    ts = tbb::tick_count::now();
    std::sort(oneapi::dpl::execution::par_unseq, minIDs, minIDs + Ncells);
    numLLPs = stage2(Ncells, minIDs);
    res->t_stage2 = (tbb::tick_count::now() - ts).seconds();

    ts = tbb::tick_count::now();
    minGridIDs.clear();
    if (Bsize > 0) {
      Qtree grid = new Qtree_t(center, maxRadius);
      for (uint32_t i = 0; i < numLLPs; i++) insertPoint(minIDs[i], cloud, grid, minRadius);
      minGridIDs = stage3(Bsize, nColsg, nRowsg, cloud, qtreeIn, grid, min);
      deleteQtree(grid);
      delete grid;
    }
    res->t_stage3 = (tbb::tick_count::now() - ts).seconds();
    t_sum += (tbb::tick_count::now() - tf).seconds();
  }
  res->t_owm = t_sum / loops;

  int rc = 0;
  int64_t total = (int64_t)minGridIDs.size() + numLLPs;
  res->n_llp = numLLPs;
  res->n_stage3 = (int64_t)minGridIDs.size();
  if (seeds) {
    if (total > seeds_cap) {
      rc = -2;
    } else {
      int64_t k = 0;
      for (int id : minGridIDs) seeds[k++] = id;
      for (uint32_t i = 0; i < numLLPs; ++i) seeds[k++] = minIDs[i];
    }
  }
  delete[] minIDs;
  deleteQtree(qtreeIn);
  delete qtreeIn;
  free(cloud);
  return rc;
}

// The reference's own loader on a file: readXYZfile (optim3_func.cpp:665-722)
// accepts header files whose name contains one of its known header names
// (e.g. "ArzuaH.xyz").  out gets the n points after the sentinel, bbox4 =
// {min_x, min_y, max_x, max_y} from the header.  Returns 0, -1 when the
// reference's loader fails, -2 if cap is too small.
int owmref_read_xyz(const char* path, double* out, int64_t cap, int64_t* n, double* bbox4) {
  Lpoint* cloud = nullptr;
  uint32_t np = 0;
  Vector2D mn{0, 0}, mx{0, 0};
  if (readXYZfile(std::string(path), cloud, np, mn, mx) != 0) return -1;
  const int64_t pts = (int64_t)np - 1;  // np counts the sentinel
  int rc = 0;
  if (pts > cap) {
    rc = -2;
  } else {
    for (int64_t i = 0; i < pts; ++i) {
      out[3 * i] = cloud[i + 1].x;
      out[3 * i + 1] = cloud[i + 1].y;
      out[3 * i + 2] = cloud[i + 1].z;
    }
    *n = pts;
    bbox4[0] = mn.x;
    bbox4[1] = mn.y;
    bbox4[2] = mx.x;
    bbox4[3] = mx.y;
  }
  free(cloud);
  return rc;
}

// The reference's own GOLD score, check_results (optim3_func.cpp:725-794), on
// a gold file of "x y z" lines and 1-based ids into the n AoS points xyz
// (cloud[0] is the sentinel {0, 0, DBL_MAX}, as readXYZfile makes it).
// Returns the reference's percentage (-1 when it cannot read the file).
double owmref_check_results(const char* gold_path, const double* xyz, int64_t n, const int* ids, int64_t n_ids,
                            float displace) {
  if (n <= 0 || n >= 0xFFFFFFFFLL) return -2.0;
  Lpoint* cloud = static_cast<Lpoint*>(mallocWrap((size_t)(n + 1) * sizeof(Lpoint)));
  cloud[0] = {0.0, 0.0, std::numeric_limits<double>::max()};
  std::memcpy(&cloud[1], xyz, (size_t)n * sizeof(Lpoint));
  std::vector<int> v(ids, ids + n_ids);
  const double r = check_results(std::string(gold_path), v, cloud, displace);
  free(cloud);
  return r;
}

}  // extern "C"
