/*
 * ORACLE / TEST INFRASTRUCTURE -- CPU restatement of FastOWM's OWM
 * ground-seed path.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline may load this; the product never does.
 *
 * Semantics restated from the reference's exact CPU path (o3memoB build,
 * CPP-TBB-CPU/application/owm_optim3.cpp + CPP-TBB-CPU/src/optim3_func.cpp):
 *
 *  params   owm_optim3.cpp:92-132, optim3_func.cpp:1-3 (round2d)
 *  stage 1  optim3_func.cpp:541-561 (window centres and radius),
 *           :481-501 / :310-324 (makeBox), :326-332 / :406 / :442 (strict
 *           point containment), :426-478 (min + count per window; the tree
 *           memo only short-cuts the same set), sentinel start minidx = 0
 *           (:484, :495) whose z is DBL_MAX (:708).
 *  stage 2  owm_optim3.cpp:160,173 + optim3_func.cpp:610-625: sort, keep
 *           every id occurring at least twice, skip -1.
 *  stage 3  optim3_func.cpp:627-662 + owm_optim3.cpp:192-199: B x B cells
 *           whose box holds no LLP strictly inside get the min point of the
 *           cell when the cell holds any point.
 *  output   owm_optim3.cpp:229-230: stage-3 ids, then the LLPs.
 *  ingest   optim3_func.cpp:665-722 (readXYZfile): oracle_xyz_parse, the
 *           checker of the device text parser.
 *
 * Tie rule: the reference keeps the first minimum its tree visits (strict
 * `<` on z).  This restatement orders points by (z, id) lexicographically,
 * which is the same whenever z is tie-free, and is the declared rule for
 * clouds with ties.
 *
 * The tree of the reference is replaced by a uniform bucket grid: bucket
 * indices are a monotone function of x (resp. y), so every point strictly
 * inside a box lies in the bucket range spanned by the box edges, and each
 * candidate is tested with the reference's strict comparisons.  Node-square
 * effects of the reference's quadtree (points exactly on a window edge) are
 * not modelled; the compiled reference (oracle/_ref) is run beside this file
 * in the tests to show that they do not arise on the test clouds.
 *
 * Build: gcc -O2 -ffp-contract=off -fopenmp -shared -fPIC (FMA contraction
 * must be off: the window geometry is bit-exact IEEE double arithmetic).
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  int64_t npoints;
  uint32_t wsize, bsize;
  double overlap;
  double min_x, min_y, max_x, max_y;
  double width, height, density, displace;
  uint32_t min_num_points; /* as stage1 receives it: (ushort) */
  uint32_t ncols, nrows;   /* ushort-truncated like the reference application */
  uint32_t ncols_grid, nrows_grid;
  int64_t ncells, ngrid;
} oracle_params;

static double round2d(double z) { return round(z * 100.0) / 100.0; }

/* owm_optim3.cpp:92-132 with the reference application's integer types. */
int oracle_params_compute(const double* bbox, int64_t n, uint32_t Wsize, double Overlap,
                          uint32_t Bsize, oracle_params* p) {
  if (n <= 0 || n >= 0xFFFFFFFFLL || !(Overlap >= 0.0 && Overlap < 1.0) || Wsize == 0) return -1;
  memset(p, 0, sizeof(*p));
  p->npoints = n;
  p->wsize = Wsize;
  p->bsize = Bsize;
  p->overlap = Overlap;
  p->min_x = bbox[0];
  p->min_y = bbox[1];
  p->max_x = bbox[2];
  p->max_y = bbox[3];
  uint32_t Npoints = (uint32_t)n + 1;
  double Width = round2d(p->max_x - p->min_x);
  double Height = round2d(p->max_y - p->min_y);
  double Density = (Npoints - 1) / (Width * Height);
  uint32_t minNumPoints = 0.5 * Density * Wsize * Wsize;
  double Displace = round2d(Wsize * (1 - Overlap));
  unsigned short nCols, nRows;
  if (Overlap > 0.0) {
    nCols = (int)(round((Width + 2 * Wsize * Overlap) / Displace)) - 1;
    nRows = (int)(round((Height + 2 * Wsize * Overlap) / Displace)) - 1;
  } else {
    nCols = (int)floor(Width / Wsize) + 1;
    nRows = (int)floor(Height / Wsize) + 1;
  }
  p->width = Width;
  p->height = Height;
  p->density = Density;
  p->displace = Displace;
  p->min_num_points = (unsigned short)minNumPoints;
  p->ncols = nCols;
  p->nrows = nRows;
  p->ncells = (int64_t)nCols * nRows;
  if (Bsize > 0) {
    unsigned short nColsg = (int)floor(Width / Bsize) + 1;
    unsigned short nRowsg = (int)floor(Height / Bsize) + 1;
    p->ncols_grid = nColsg;
    p->nrows_grid = nRowsg;
    p->ngrid = (int64_t)nColsg * nRowsg;
  }
  return 0;
}

/* Window edges, optim3_func.cpp:544-555 and :492-497.  Wsize/2 is integer
 * division of a ushort; the radius travels as float then double. */
void oracle_window_box(const oracle_params* p, int64_t ii, int64_t jj, double* box) {
  unsigned short W = (unsigned short)p->wsize;
  double Displace = round2d(W * (1 - p->overlap));
  double initX = p->min_x - W / 2 + Displace;
  double initY = p->min_y - W / 2 + Displace;
  double cx = initX + (int)ii * Displace;
  double cy = initY + (int)jj * Displace;
  float rf = (float)(W / 2);
  double r = (double)rf;
  box[0] = cx - r;
  box[1] = cy - r;
  box[2] = cx + r;
  box[3] = cy + r;
}

/* Cell edges, optim3_func.cpp:630-651 and :481-486. */
void oracle_cell_box(const oracle_params* p, int64_t ii, int64_t jj, double* box) {
  unsigned short B = (unsigned short)p->bsize;
  double initX = p->min_x + B / 2;
  double initY = p->min_y + B / 2;
  double cx = initX + (int)ii * B;
  double cy = initY + (int)jj * B;
  float r = (float)(B / 2);
  box[0] = cx - r;
  box[1] = cy - r;
  box[2] = cx + r;
  box[3] = cy + r;
}

/* ---- bucket grid over the points ---- */
typedef struct {
  double x0, y0, g;
  int64_t nbx, nby;
  int64_t* start; /* [nbx*nby+1] */
  double* bx;     /* points sorted by bucket: x, y, z */
  double* by;
  double* bz;
  int64_t* bid; /* 1-based ids */
} bucket_grid;

static int64_t bucket_of(double v, double v0, double g, int64_t nb) {
  double t = floor((v - v0) / g);
  if (!(t >= 0)) return 0; /* also catches NaN */
  if (t >= (double)(nb - 1)) return nb - 1;
  return (int64_t)t;
}

static int grid_build(bucket_grid* G, const double* xyz, int64_t n, double x0, double y0,
                      double x1, double y1, double g) {
  G->x0 = x0;
  G->y0 = y0;
  G->g = g;
  G->nbx = (int64_t)((x1 - x0) / g) + 1;
  G->nby = (int64_t)((y1 - y0) / g) + 1;
  if (G->nbx < 1) G->nbx = 1;
  if (G->nby < 1) G->nby = 1;
  int64_t nb = G->nbx * G->nby;
  G->start = (int64_t*)calloc((size_t)nb + 1, sizeof(int64_t));
  int64_t* key = (int64_t*)malloc((size_t)n * sizeof(int64_t));
  G->bx = (double*)malloc((size_t)n * sizeof(double));
  G->by = (double*)malloc((size_t)n * sizeof(double));
  G->bz = (double*)malloc((size_t)n * sizeof(double));
  G->bid = (int64_t*)malloc((size_t)n * sizeof(int64_t));
  if (!G->start || !key || !G->bx || !G->by || !G->bz || !G->bid) {
    free(key);
    return -1;
  }
  for (int64_t i = 0; i < n; ++i) {
    int64_t k = bucket_of(xyz[3 * i + 1], y0, g, G->nby) * G->nbx +
                bucket_of(xyz[3 * i], x0, g, G->nbx);
    key[i] = k;
    G->start[k + 1]++;
  }
  for (int64_t b = 0; b < nb; ++b) G->start[b + 1] += G->start[b];
  int64_t* cur = (int64_t*)malloc((size_t)nb * sizeof(int64_t));
  if (!cur) {
    free(key);
    return -1;
  }
  memcpy(cur, G->start, (size_t)nb * sizeof(int64_t));
  for (int64_t i = 0; i < n; ++i) {
    int64_t d = cur[key[i]]++;
    G->bx[d] = xyz[3 * i];
    G->by[d] = xyz[3 * i + 1];
    G->bz[d] = xyz[3 * i + 2];
    G->bid[d] = i + 1;
  }
  free(cur);
  free(key);
  return 0;
}

static void grid_free(bucket_grid* G) {
  free(G->start);
  free(G->bx);
  free(G->by);
  free(G->bz);
  free(G->bid);
}

/* (z, id)-min and strict count over the points strictly inside box.
 * best starts at the sentinel (DBL_MAX, 0). */
static void box_query(const bucket_grid* G, const double* box, int64_t* count, int64_t* best_id,
                      double* best_z) {
  int64_t c = 0, bid = 0;
  double bz = DBL_MAX;
  int64_t i0 = bucket_of(box[0], G->x0, G->g, G->nbx), i1 = bucket_of(box[2], G->x0, G->g, G->nbx);
  int64_t j0 = bucket_of(box[1], G->y0, G->g, G->nby), j1 = bucket_of(box[3], G->y0, G->g, G->nby);
  for (int64_t j = j0; j <= j1; ++j) {
    for (int64_t i = i0; i <= i1; ++i) {
      int64_t b = j * G->nbx + i;
      for (int64_t k = G->start[b]; k < G->start[b + 1]; ++k) {
        double x = G->bx[k], y = G->by[k];
        if (x > box[0] && y > box[1] && x < box[2] && y < box[3]) {
          ++c;
          double z = G->bz[k];
          int64_t id = G->bid[k];
          if (z < bz || (z == bz && id < bid)) {
            bz = z;
            bid = id;
          }
        }
      }
    }
  }
  *count = c;
  *best_id = bid;
  *best_z = bz;
}

static double grid_pitch(const oracle_params* p) {
  double g = p->wsize > 1 ? (double)(p->wsize / 2) : 1.0;
  if (g <= 0) g = 1.0;
  return g;
}

/* Stage 1: win_min[ii*nrows + jj] = min id or -1 (optim3_func.cpp:549-560). */
int oracle_stage1(const double* xyz, int64_t n, const oracle_params* p, int64_t* win_min,
                  int nthreads) {
  bucket_grid G;
  double pad = (double)p->wsize;
  if (grid_build(&G, xyz, n, p->min_x - pad, p->min_y - pad, p->max_x + pad, p->max_y + pad,
                 grid_pitch(p)) != 0)
    return -1;
  int64_t ncells = p->ncells, nrows = p->nrows;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
#endif
  for (int64_t step = 0; step < ncells; ++step) {
    double box[4];
    oracle_window_box(p, step / nrows, step % nrows, box);
    int64_t c, id;
    double z;
    box_query(&G, box, &c, &id, &z);
    win_min[step] = (c >= (int64_t)p->min_num_points) ? id : -1;
  }
  (void)nthreads;
  grid_free(&G);
  return 0;
}

static int cmp_i64(const void* a, const void* b) {
  int64_t x = *(const int64_t*)a, y = *(const int64_t*)b;
  return (x > y) - (x < y);
}

/* Stage 2 (owm_optim3.cpp:160,173; optim3_func.cpp:610-625): sort in place,
 * compact ids with run length >= 2 to the front, return their number.  With
 * overlap 0 the reference counts the valid minima without compacting them
 * (owm_optim3.cpp:185-188), which leaves -1 entries inside the LLP prefix;
 * this restatement compacts the valid minima instead. */
int64_t oracle_stage2(int64_t* ids, int64_t ncells, double overlap) {
  qsort(ids, (size_t)ncells, sizeof(int64_t), cmp_i64);
  int64_t i = 0;
  while (i < ncells && ids[i] < 0) ++i;
  int64_t counter = 0;
  if (overlap == 0.0) {
    for (; i < ncells; ++i) ids[counter++] = ids[i];
    return counter;
  }
  while (i < ncells) {
    int64_t j = i + 1;
    while (j < ncells && ids[j] == ids[i]) ++j;
    if (j - i > 1) ids[counter++] = ids[i];
    i = j;
  }
  return counter;
}

/* Stage 3 (optim3_func.cpp:627-662): out gets, in cell order (jj outer, ii
 * inner), the min id of each cell that holds no LLP strictly inside and at
 * least one point.  Returns the number written (<= ngrid). */
int64_t oracle_stage3(const double* xyz, int64_t n, const oracle_params* p, const int64_t* llp,
                      int64_t n_llp, int64_t* out, int nthreads) {
  if (p->bsize == 0 || p->ngrid == 0) return 0;
  int64_t ncg = p->ncols_grid, nrg = p->nrows_grid;
  unsigned char* has = (unsigned char*)calloc((size_t)(ncg * nrg), 1);
  if (!has) return -1;
  double B = (double)p->bsize;
  for (int64_t k = 0; k < n_llp; ++k) {
    int64_t id = llp[k];
    double x, y;
    if (id <= 0) {
      x = 0.0; /* sentinel point {0, 0, DBL_MAX} */
      y = 0.0;
    } else {
      x = xyz[3 * (id - 1)];
      y = xyz[3 * (id - 1) + 1];
    }
    int64_t ic = (int64_t)floor((x - p->min_x) / B), jc = (int64_t)floor((y - p->min_y) / B);
    for (int64_t jj = jc - 1; jj <= jc + 1; ++jj) {
      if (jj < 0 || jj >= nrg) continue;
      for (int64_t ii = ic - 1; ii <= ic + 1; ++ii) {
        if (ii < 0 || ii >= ncg) continue;
        double box[4];
        oracle_cell_box(p, ii, jj, box);
        if (x > box[0] && y > box[1] && x < box[2] && y < box[3]) has[jj * ncg + ii] = 1;
      }
    }
  }
  bucket_grid G;
  double pad = B;
  double g = p->bsize > 1 ? (double)(p->bsize / 2) : 1.0;
  if (grid_build(&G, xyz, n, p->min_x - pad, p->min_y - pad, p->max_x + pad, p->max_y + pad, g) !=
      0) {
    free(has);
    return -1;
  }
  int64_t* cell_min = (int64_t*)malloc((size_t)(ncg * nrg) * sizeof(int64_t));
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
  for (int64_t c = 0; c < ncg * nrg; ++c) {
    cell_min[c] = -1;
    if (has[c]) continue;
    double box[4];
    oracle_cell_box(p, c % ncg, c / ncg, box);
    int64_t cnt, id;
    double z;
    box_query(&G, box, &cnt, &id, &z);
    if (cnt > 0) cell_min[c] = id;
  }
  (void)nthreads;
  int64_t m = 0;
  for (int64_t c = 0; c < ncg * nrg; ++c)
    if (cell_min[c] >= 0) out[m++] = cell_min[c];
  free(cell_min);
  free(has);
  grid_free(&G);
  return m;
}

/* Whole path: seeds = stage-3 ids then LLPs (owm_optim3.cpp:229-230).
 * seeds needs room for ngrid + ncells entries; returns the seed count or a
 * negative error. n_llp receives the LLP count. */
int64_t oracle_run(const double* xyz, int64_t n, const double* bbox, uint32_t W, double O,
                   uint32_t B, int64_t* seeds, int64_t* n_llp_out, int nthreads) {
  oracle_params p;
  if (oracle_params_compute(bbox, n, W, O, B, &p) != 0) return -1;
  int64_t* win = (int64_t*)malloc((size_t)(p.ncells > 0 ? p.ncells : 1) * sizeof(int64_t));
  if (!win) return -1;
  if (oracle_stage1(xyz, n, &p, win, nthreads) != 0) {
    free(win);
    return -1;
  }
  int64_t n_llp = oracle_stage2(win, p.ncells, O);
  int64_t* s3 = (int64_t*)malloc((size_t)(p.ngrid > 0 ? p.ngrid : 1) * sizeof(int64_t));
  int64_t n3 = oracle_stage3(xyz, n, &p, win, n_llp, s3, nthreads);
  if (n3 < 0) {
    free(win);
    free(s3);
    return -1;
  }
  memcpy(seeds, s3, (size_t)n3 * sizeof(int64_t));
  memcpy(seeds + n3, win, (size_t)n_llp * sizeof(int64_t));
  if (n_llp_out) *n_llp_out = n_llp;
  free(win);
  free(s3);
  return n3 + n_llp;
}

/* Cloud text (test infrastructure): readXYZfile (optim3_func.cpp:665-722)
 * restated line by line on a text buffer, with the C library's own sscanf
 * conversions, as the device ingest must reproduce them:
 *   * the first line decides: one number = header (the point count, then one
 *     value per line: min x, max x, min y, max y; :694-699), three or more =
 *     no header (the bbox is then the data's);
 *   * every later line is sscanf("%lf %lf %lf") (:711, the rest of the line
 *     skipped as at :715); lines of spaces, tabs and CRs are skipped, any
 *     other line with fewer than three numbers fails;
 *   * with a header, reading stops at the declared count (:710), and fewer
 *     points fail; non-finite values fail.
 * A line is the text up to its newline (a NUL ends what sscanf sees).
 * Returns 0 (points in out[0..3n), bbox4 = {min_x, min_y, max_x, max_y}) or
 * -5 (the loader's error) / -2 (cap too small). */
int oracle_xyz_parse(const char* text, int64_t nbytes, double* out, int64_t cap, int64_t* n_out, double* bbox4,
                     int* has_header) {
  int64_t pos = 0, n = 0, declared = -1;
  size_t lcap = 256;
  char* line = (char*)malloc(lcap);
  int rc = 0;
  int first = 1;
  double hb[4] = {0, 0, 0, 0};
  int hdr_left = 0;
  if (!line) return -5;
  *has_header = 0;
  while (pos < nbytes) {
    const char* nl = (const char*)memchr(text + pos, '\n', (size_t)(nbytes - pos));
    int64_t e = nl ? (int64_t)(nl - text) : nbytes;
    size_t len = (size_t)(e - pos);
    if (len + 2 > lcap) {
      lcap = len + 2;
      line = (char*)realloc(line, lcap);
      if (!line) return -5;
    }
    memcpy(line, text + pos, len);
    line[len] = '\n';
    line[len + 1] = 0;
    pos = e + 1;
    double a[3];
    if (first) {
      int k = sscanf(line, "%lf %lf %lf", &a[0], &a[1], &a[2]);
      first = 0;
      if (k == 1) {
        if (!(a[0] >= 1.0 && a[0] < 9.2e18)) { rc = -5; break; }
        declared = (int64_t)a[0];
        *has_header = 1;
        hdr_left = 4;
        continue;
      }
      if (k != 3) { rc = -5; break; }
    } else if (hdr_left > 0) {
      if (sscanf(line, "%lf", &hb[4 - hdr_left]) != 1) { rc = -5; break; }
      --hdr_left;
      continue;
    } else {
      if (declared >= 0 && n >= declared) break;
      if (sscanf(line, "%lf %lf %lf", &a[0], &a[1], &a[2]) != 3) {
        int blank = 1;
        for (char* c = line; *c; ++c)
          if (*c != ' ' && *c != '\n' && *c != '\r' && *c != '\t') blank = 0;
        if (blank) continue;
        rc = -5;
        break;
      }
    }
    if (!isfinite(a[0]) || !isfinite(a[1]) || !isfinite(a[2])) { rc = -5; break; }
    if (n >= cap) { rc = -2; break; }
    out[3 * n] = a[0];
    out[3 * n + 1] = a[1];
    out[3 * n + 2] = a[2];
    ++n;
  }
  free(line);
  if (rc) return rc;
  if (hdr_left > 0 || n == 0 || (declared >= 0 && n < declared)) return -5;
  if (declared >= 0) {
    bbox4[0] = hb[0];  /* min x */
    bbox4[1] = hb[2];  /* min y */
    bbox4[2] = hb[1];  /* max x */
    bbox4[3] = hb[3];  /* max y */
  } else {
    double x0 = out[0], x1 = out[0], y0 = out[1], y1 = out[1];
    for (int64_t i = 1; i < n; ++i) {
      x0 = out[3 * i] < x0 ? out[3 * i] : x0;
      x1 = out[3 * i] > x1 ? out[3 * i] : x1;
      y0 = out[3 * i + 1] < y0 ? out[3 * i + 1] : y0;
      y1 = out[3 * i + 1] > y1 ? out[3 * i + 1] : y1;
    }
    bbox4[0] = x0;
    bbox4[1] = y0;
    bbox4[2] = x1;
    bbox4[3] = y1;
  }
  *n_out = n;
  return 0;
}
