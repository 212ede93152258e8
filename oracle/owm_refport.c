/*
 * ORACLE / TEST INFRASTRUCTURE -- a C port of the reference's own CPU
 * algorithm for the OWM path, used as the timed CPU baseline where the
 * reference's sources are not available to compile (kind "port").  It is
 * never part of the product.
 *
 * It follows CPP-TBB-CPU/src/optim3_func.cpp step by step, in my own data
 * layout (one node array, index links instead of pointers):
 *   tree        quadtree over the square (center, maxRadius) of getRadius /
 *               getCenter (:6-26); child = (x >= cx) << 1 | (y >= cy)
 *               (:92-100); children centred at c -/+ r*0.5f with radius
 *               r*0.5 stored as float (:59-73); maxNumber policy: a full leaf
 *               splits and re-inserts its points (insertPointMaxNum,
 *               :160-184), or the minRadius rule (insertPoint, :103-123);
 *               the first `level` levels are pre-split and filled in
 *               parallel (parallel_qtree, :220-253)
 *   memo        per node min id and point count (storeMinAndNumPoints,
 *               :255-307), strict '<' on z, first child wins
 *   stage 1     findValidMinMemo (:426-478) with boxInside2D / boxOverlap2D
 *               on node squares (:334-358) and strict point tests; window
 *               geometry of stage1 (:541-561)
 *   stage 2     sort + ids occurring at least twice (:610-625)
 *   stage 3     grid quadtree of the LLPs with the minRadius policy
 *               (insertPoint, :103-123), countNeighbors (:503-539) and
 *               findValidMin (:390-424) over B x B cells (:627-662)
 * Ties keep the first minimum visited (strict '<'), like the reference.
 * Build: gcc -O3 -ffp-contract=off -fopenmp.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  double cx, cy;
  float r;
  int32_t child; /* index of the first of 4 children, -1 = leaf */
  uint32_t min, count;
  int32_t pts, npts, cap; /* leaf points: pool[pts .. pts+npts) */
} qnode;

typedef struct {
  qnode* n;
  int64_t nn, capn;
  uint32_t* pool; /* point ids of leaves */
  int64_t np, capp;
} qtree;

static const double* X; /* cloud with sentinel: point i at X[3*i] */

static int64_t qt_new_node(qtree* t, double cx, double cy, float r) {
  if (t->nn == t->capn) {
    t->capn = t->capn ? 2 * t->capn : 1024;
    t->n = (qnode*)realloc(t->n, (size_t)t->capn * sizeof(qnode));
  }
  qnode* q = &t->n[t->nn];
  q->cx = cx;
  q->cy = cy;
  q->r = r;
  q->child = -1;
  q->min = 0;
  q->count = 0;
  q->pts = -1;
  q->npts = 0;
  q->cap = 0;
  return t->nn++;
}

static void qt_split(qtree* t, int64_t i) {
  /* createQuadrants: children at c -/+ r*0.5f, radius r*0.5 (as float) */
  double cx = t->n[i].cx, cy = t->n[i].cy;
  float r = t->n[i].r;
  float nr = (float)(r * 0.5);
  int64_t c0 = -1;
  for (int k = 0; k < 4; ++k) {
    double ncx = cx + r * ((k & 2) ? 0.5f : -0.5f);
    double ncy = cy + r * ((k & 1) ? 0.5f : -0.5f);
    int64_t c = qt_new_node(t, ncx, ncy, nr);
    if (k == 0) c0 = c;
  }
  t->n[i].child = (int32_t)c0;
}

static int quadrant(const qnode* q, uint32_t p) {
  int c = 0;
  if (X[3 * p] >= q->cx) c |= 2;
  if (X[3 * p + 1] >= q->cy) c |= 1;
  return c;
}

static void leaf_push(qtree* t, int64_t i, uint32_t p) {
  qnode* q = &t->n[i];
  if (q->npts == q->cap) {
    int32_t nc = q->cap ? 2 * q->cap : 8;
    if (t->np + nc > t->capp) {
      t->capp = (t->np + nc) * 2;
      t->pool = (uint32_t*)realloc(t->pool, (size_t)t->capp * sizeof(uint32_t));
    }
    if (q->npts) memcpy(t->pool + t->np, t->pool + q->pts, (size_t)q->npts * sizeof(uint32_t));
    q->pts = (int32_t)t->np;
    t->np += nc;
    q->cap = nc;
  }
  t->pool[q->pts + q->npts++] = p;
  if (X[3 * p + 2] < X[3 * q->min + 2]) q->min = p;
  q->count++;
}

/* insertPointMaxNum: descend; a full leaf splits and re-inserts its points. */
static void insert_maxnum(qtree* t, int64_t i, uint32_t p, int maxn) {
  for (;;) {
    if (t->n[i].child < 0) {
      if (t->n[i].npts < maxn) {
        leaf_push(t, i, p);
        return;
      }
      /* overloaded leaf becomes internal: keep its stale min like the
       * reference (numPoints is reset and recomputed by the memo pass) */
      int32_t pts = t->n[i].pts, np = t->n[i].npts;
      t->n[i].count = 0;
      qt_split(t, i);
      uint32_t* tmp = (uint32_t*)malloc((size_t)np * sizeof(uint32_t));
      memcpy(tmp, t->pool + pts, (size_t)np * sizeof(uint32_t));
      for (int32_t k = 0; k < np; ++k) {
        int64_t c = t->n[i].child + quadrant(&t->n[i], tmp[k]);
        insert_maxnum(t, c, tmp[k], maxn);
      }
      free(tmp);
    }
    i = t->n[i].child + quadrant(&t->n[i], p);
  }
}

/* insertPoint with the minRadius policy (grid of stage 3). */
static void insert_minrad(qtree* t, int64_t i, uint32_t p, float minr) {
  for (;;) {
    if (t->n[i].child < 0) {
      if (t->n[i].r * 0.5 > minr) {
        qt_split(t, i);
      } else {
        leaf_push(t, i, p);
        return;
      }
    }
    i = t->n[i].child + quadrant(&t->n[i], p);
  }
}

static void memo(qtree* t, int64_t i) {
  if (t->n[i].child < 0) return;
  for (int k = 0; k < 4; ++k) {
    int64_t c = t->n[i].child + k;
    memo(t, c);
    t->n[i].count += t->n[c].count;
    if (X[3 * t->n[c].min + 2] < X[3 * t->n[i].min + 2]) t->n[i].min = t->n[c].min;
  }
}

/* A forest: the top `level` levels, then one subtree per level-L cell built
 * independently (the reference's phase-2 tasks), each in its own arena. */
typedef struct {
  qtree top;
  qtree* sub;   /* [ncells] */
  int64_t* leaf_of; /* top node index of each cell */
  int ncells;
} forest;

typedef struct {
  const forest* f;
} fctx;

/* node reference: (tree index, node index); tree -1 = top */
static int inside_box(double bx0, double by0, double bx1, double by1, const qnode* q) {
  if (q->cx + q->r > bx1 || q->cy + q->r > by1) return 0;
  if (q->cx - q->r < bx0 || q->cy - q->r < by0) return 0;
  return 1;
}
static int overlap_box(double bx0, double by0, double bx1, double by1, const qnode* q) {
  if (q->cx + q->r < bx0 || q->cy + q->r < by0) return 0;
  if (q->cx - q->r > bx1 || q->cy - q->r > by1) return 0;
  return 1;
}

/* findValidMinMemo over one tree (recursive, quadrant order 0..3) */
static void fvm_memo(const qtree* t, int64_t i, double bx0, double by0, double bx1, double by1, int* cnt,
                     uint32_t* mn) {
  const qnode* q = &t->n[i];
  if (q->child < 0 && q->npts > 0) {
    if (inside_box(bx0, by0, bx1, by1, q)) {
      if (X[3 * q->min + 2] < X[3 * *mn + 2]) *mn = q->min;
      *cnt += (int)q->count;
    } else {
      double mx = X[3 * q->min], my = X[3 * q->min + 1];
      const uint32_t* pp = t->pool + q->pts;
      if (mx > bx0 && my > by0 && mx < bx1 && my < by1) {
        if (X[3 * q->min + 2] < X[3 * *mn + 2]) *mn = q->min;
        for (int32_t k = 0; k < q->npts; ++k) {
          double x = X[3 * pp[k]], y = X[3 * pp[k] + 1];
          if (x > bx0 && y > by0 && x < bx1 && y < by1) (*cnt)++;
        }
      } else {
        for (int32_t k = 0; k < q->npts; ++k) {
          double x = X[3 * pp[k]], y = X[3 * pp[k] + 1];
          if (x > bx0 && y > by0 && x < bx1 && y < by1) {
            if (X[3 * pp[k] + 2] < X[3 * *mn + 2]) *mn = pp[k];
            (*cnt)++;
          }
        }
      }
    }
  } else {
    if (inside_box(bx0, by0, bx1, by1, q)) {
      if (X[3 * q->min + 2] < X[3 * *mn + 2]) *mn = q->min;
      *cnt += (int)q->count;
    } else if (q->child >= 0) {
      for (int k = 0; k < 4; ++k) {
        int64_t c = q->child + k;
        if (overlap_box(bx0, by0, bx1, by1, &t->n[c])) fvm_memo(t, c, bx0, by0, bx1, by1, cnt, mn);
      }
    }
  }
}

/* findValidMin (no memo): used by stage 3 */
static void fvm(const qtree* t, int64_t i, double bx0, double by0, double bx1, double by1, int* cnt, uint32_t* mn) {
  const qnode* q = &t->n[i];
  if (q->child < 0) {
    const uint32_t* pp = t->pool + q->pts;
    if (inside_box(bx0, by0, bx1, by1, q)) {
      for (int32_t k = 0; k < q->npts; ++k)
        if (X[3 * pp[k] + 2] < X[3 * *mn + 2]) *mn = pp[k];
      *cnt += q->npts;
    } else {
      for (int32_t k = 0; k < q->npts; ++k) {
        double x = X[3 * pp[k]], y = X[3 * pp[k] + 1];
        if (x > bx0 && y > by0 && x < bx1 && y < by1) {
          if (X[3 * pp[k] + 2] < X[3 * *mn + 2]) *mn = pp[k];
          (*cnt)++;
        }
      }
    }
  } else {
    for (int k = 0; k < 4; ++k) {
      int64_t c = q->child + k;
      if (overlap_box(bx0, by0, bx1, by1, &t->n[c])) fvm(t, c, bx0, by0, bx1, by1, cnt, mn);
    }
  }
}

static void count_nb(const qtree* t, int64_t i, double bx0, double by0, double bx1, double by1, int* cnt) {
  const qnode* q = &t->n[i];
  if (q->child < 0) {
    if (inside_box(bx0, by0, bx1, by1, q)) {
      *cnt += q->npts;
    } else {
      const uint32_t* pp = t->pool + q->pts;
      for (int32_t k = 0; k < q->npts; ++k) {
        double x = X[3 * pp[k]], y = X[3 * pp[k] + 1];
        if (x > bx0 && y > by0 && x < bx1 && y < by1) (*cnt)++;
      }
    }
  } else {
    for (int k = 0; k < 4; ++k) {
      int64_t c = q->child + k;
      if (overlap_box(bx0, by0, bx1, by1, &t->n[c])) count_nb(t, c, bx0, by0, bx1, by1, cnt);
    }
  }
}

/* The cloud tree as one array: pre-split top levels, then the level-L cells'
 * subtrees appended (built in parallel in separate arenas, then copied). */
static void build_cloud_tree(qtree* T, int64_t N, double cx, double cy, float R, int level, int policy, int maxn,
                             float minr, int nthreads) {
  memset(T, 0, sizeof(*T));
  qt_new_node(T, cx, cy, R);
  /* tree_phase1: split every node down to `level` */
  int64_t lo = 0, hi = 1;
  for (int l = 0; l < level; ++l) {
    for (int64_t i = lo; i < hi; ++i) qt_split(T, i);
    lo = hi;
    hi = T->nn;
  }
  int64_t ncell = hi - lo, cell0 = lo;
  /* phase 1: route every point to its level-L cell (counting sort, input order) */
  int32_t* cell = (int32_t*)malloc((size_t)(N + 1) * sizeof(int32_t));
  int64_t* start = (int64_t*)calloc((size_t)ncell + 1, sizeof(int64_t));
#pragma omp parallel for num_threads(nthreads) schedule(static)
  for (int64_t p = 1; p <= N; ++p) {
    int64_t i = 0;
    while (T->n[i].child >= 0) i = T->n[i].child + quadrant(&T->n[i], (uint32_t)p);
    cell[p] = (int32_t)(i - cell0);
  }
  for (int64_t p = 1; p <= N; ++p) start[cell[p] + 1]++;
  for (int64_t c = 0; c < ncell; ++c) start[c + 1] += start[c];
  uint32_t* order = (uint32_t*)malloc((size_t)(N > 0 ? N : 1) * sizeof(uint32_t));
  int64_t* cur = (int64_t*)malloc((size_t)ncell * sizeof(int64_t));
  memcpy(cur, start, (size_t)ncell * sizeof(int64_t));
  for (int64_t p = 1; p <= N; ++p) order[cur[cell[p]]++] = (uint32_t)p;
  free(cur);
  free(cell);
  /* phase 2: each cell's subtree: split once, fill by the policy's rule */
  qtree* sub = (qtree*)calloc((size_t)ncell, sizeof(qtree));
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 1)
  for (int64_t c = 0; c < ncell; ++c) {
    qtree* s = &sub[c];
    const qnode* q = &T->n[cell0 + c];
    qt_new_node(s, q->cx, q->cy, q->r);
    qt_split(s, 0);
    for (int64_t k = start[c]; k < start[c + 1]; ++k) {
      uint32_t p = order[k];
      int64_t c0 = s->n[0].child + quadrant(&s->n[0], p);
      if (policy)
        insert_maxnum(s, c0, p, maxn);
      else
        insert_minrad(s, c0, p, minr);
    }
  }
  /* splice: cell node takes the subtree's children */
  for (int64_t c = 0; c < ncell; ++c) {
    qtree* s = &sub[c];
    int64_t noff = T->nn - 1; /* node k>0 of s -> T index noff + k */
    int64_t poff = T->np;
    for (int64_t k = 1; k < s->nn; ++k) {
      int64_t dst = qt_new_node(T, 0, 0, 0);
      T->n[dst] = s->n[k];
      if (T->n[dst].child >= 0) T->n[dst].child = (int32_t)(T->n[dst].child + noff);
      if (T->n[dst].pts >= 0) T->n[dst].pts = (int32_t)(T->n[dst].pts + poff);
    }
    if (T->np + s->np > T->capp) {
      T->capp = T->np + s->np + 1024;
      T->pool = (uint32_t*)realloc(T->pool, (size_t)T->capp * sizeof(uint32_t));
    }
    if (s->np) memcpy(T->pool + T->np, s->pool, (size_t)s->np * sizeof(uint32_t));
    T->np += s->np;
    T->n[cell0 + c].child = (int32_t)(s->n[0].child + noff);
    free(s->n);
    free(s->pool);
  }
  free(sub);
  free(order);
  free(start);
  /* storeMinAndNumPoints */
  memo(T, 0);
}

static double round2d(double z) { return round(z * 100.0) / 100.0; }

static int cmp_int(const void* a, const void* b) {
  int x = *(const int*)a, y = *(const int*)b;
  return (x > y) - (x < y);
}

/* Whole path like the reference application.  xyz: n points (no sentinel);
 * policy 1 = maxNumber leaves, 0 = minRadius leaves (the -DMAXNUMBER switch).
 * seeds: stage-3 ids then LLPs; returns their count (or -1).  Times in s. */
int64_t refport_run(const double* xyz, int64_t n, const double* bbox, uint32_t Wsize, double Overlap,
                    uint32_t Bsize, int policy, int maxNumber, float minRadius, int level, int nthreads, int64_t* seeds,
                    int64_t cap, int64_t* n_llp, double* t_tree, double* t_owm) {
  if (n <= 0 || n >= 0xFFFFFFFFLL || !(Overlap > 0.0 && Overlap < 1.0)) return -1;
  if (nthreads <= 0) nthreads = 1;
  uint32_t Npoints = (uint32_t)n + 1;
  double* cloud = (double*)malloc((size_t)Npoints * 3 * sizeof(double));
  cloud[0] = 0.0;
  cloud[1] = 0.0;
  cloud[2] = DBL_MAX;
  memcpy(cloud + 3, xyz, (size_t)n * 3 * sizeof(double));
  X = cloud;
  double minx = bbox[0], miny = bbox[1], maxx = bbox[2], maxy = bbox[3];
  double rx = (maxx - minx) / 2.0, ry = (maxy - miny) / 2.0;
  float maxRadius = rx >= ry ? (float)rx : (float)ry;
  double cx = minx + rx, cy = miny + ry;
#ifdef _OPENMP
  double t0 = omp_get_wtime();
#else
  double t0 = 0;
#endif
  qtree T;
  build_cloud_tree(&T, n, cx, cy, maxRadius, level, policy, maxNumber, minRadius, nthreads);
#ifdef _OPENMP
  double t1 = omp_get_wtime();
#else
  double t1 = 0;
#endif
  double Width = round2d(maxx - minx), Height = round2d(maxy - miny);
  double Density = (Npoints - 1) / (Width * Height);
  uint32_t minNumPoints = 0.5 * Density * Wsize * Wsize;
  unsigned short thr = (unsigned short)minNumPoints;
  double Displace = round2d(Wsize * (1 - Overlap));
  unsigned short nCols = (int)(round((Width + 2 * Wsize * Overlap) / Displace)) - 1;
  unsigned short nRows = (int)(round((Height + 2 * Wsize * Overlap) / Displace)) - 1;
  uint32_t Ncells = (uint32_t)nCols * nRows;
  unsigned short W16 = (unsigned short)Wsize, B16 = (unsigned short)Bsize;
  double initX = minx - W16 / 2 + Displace, initY = miny - W16 / 2 + Displace;
  double rw = (double)(float)(W16 / 2);
  int* minIDs = (int*)malloc((size_t)Ncells * sizeof(int));
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64)
  for (int64_t step = 0; step < (int64_t)Ncells; ++step) {
    int ii = (int)(step / nRows), jj = (int)(step % nRows);
    double ccx = initX + ii * Displace, ccy = initY + jj * Displace;
    int cnt = 0;
    uint32_t mn = 0;
    fvm_memo(&T, 0, ccx - rw, ccy - rw, ccx + rw, ccy + rw, &cnt, &mn);
    minIDs[step] = cnt >= thr ? (int)mn : -1;
  }
  qsort(minIDs, Ncells, sizeof(int), cmp_int);
  uint32_t i = 0, counter = 0;
  while (i < Ncells && minIDs[i] < 0) ++i;
  while (i < Ncells) {
    uint32_t j = i + 1;
    while (j < Ncells && minIDs[j] == minIDs[i]) ++j;
    if (j - i > 1) minIDs[counter++] = minIDs[i];
    i = j;
  }
  int64_t nout = 0;
  if (Bsize > 0) {
    qtree G;
    memset(&G, 0, sizeof(G));
    qt_new_node(&G, cx, cy, maxRadius);
    for (uint32_t k = 0; k < counter; ++k) insert_minrad(&G, 0, (uint32_t)minIDs[k], minRadius);
    unsigned short nColsg = (int)floor(Width / Bsize) + 1, nRowsg = (int)floor(Height / Bsize) + 1;
    double gx0 = minx + B16 / 2, gy0 = miny + B16 / 2;
    double rb = (double)(float)(B16 / 2);
    int64_t ng = (int64_t)nColsg * nRowsg;
    int64_t* cm = (int64_t*)malloc((size_t)ng * sizeof(int64_t));
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 8)
    for (int64_t c = 0; c < ng; ++c) {
      int ii = (int)(c % nColsg), jj = (int)(c / nColsg);
      double ccx = gx0 + ii * B16, ccy = gy0 + jj * B16;
      int cnt = 0;
      count_nb(&G, 0, ccx - rb, ccy - rb, ccx + rb, ccy + rb, &cnt);
      cm[c] = -1;
      if (cnt == 0) {
        uint32_t mn = 0;
        fvm(&T, 0, ccx - rb, ccy - rb, ccx + rb, ccy + rb, &cnt, &mn);
        if (cnt > 0) cm[c] = mn;
      }
    }
    for (int64_t c = 0; c < ng; ++c)
      if (cm[c] >= 0 && nout < cap) seeds[nout++] = cm[c];
    free(cm);
    free(G.n);
    free(G.pool);
  }
  for (uint32_t k = 0; k < counter && nout < cap; ++k) seeds[nout++] = minIDs[k];
#ifdef _OPENMP
  double t2 = omp_get_wtime();
#else
  double t2 = 0;
#endif
  if (n_llp) *n_llp = counter;
  if (t_tree) *t_tree = t1 - t0;
  if (t_owm) *t_owm = t2 - t1;
  free(minIDs);
  free(T.n);
  free(T.pool);
  free(cloud);
  return nout;
}
