// Host-side parts of the OWM path that carry no device work: the reference application's
// parameter arithmetic, cloud file I/O and the tolerant GOLD score (the
// seeded synthetic cloud generator is owm_synth.c).
//
// Built with -ffp-contract=off: the parameters must give the same bits on
// x86-64 and aarch64 (GCC contracts a+b*c on aarch64 by default).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "owm_gb300.h"

namespace {

double round2d(double z) { return std::round(z * 100.0) / 100.0; }  // optim3_func.cpp:1-3

}  // namespace

extern "C" {

const char* owm_status_string(int s) {
  switch (s) {
    case OWM_OK: return "ok";
    case OWM_EINVAL: return "invalid argument";
    case OWM_ENOMEM: return "out of memory or over budget";
    case OWM_ECUDA: return "CUDA error or no CUDA device";
    case OWM_ETIMEOUT: return "bounded device wait expired";
    case OWM_EIO: return "file read/parse error";
    case OWM_ERANGE: return "output capacity too small";
    case OWM_EAGAIN: return "not ready";
    default: return "unknown status";
  }
}

int owm_version(void) { return 10000; }

// owm_optim3.cpp:92-132, with the reference application's types: Npoints counts the
// sentinel (so Density uses Npoints-1), minNumPoints is uint32 then handed
// to stage1 as ushort, nCols/nRows/nColsg/nRowsg are ushort.
int owm_params_compute(const owm_bbox* bbox, int64_t npoints, uint32_t Wsize, double Overlap,
                       uint32_t Bsize, owm_params* p) {
  if (!bbox || !p || npoints <= 0 || npoints >= 0xFFFFFFFFLL || Wsize == 0 || Wsize > 65535 ||
      Bsize > 65535 || !(Overlap >= 0.0 && Overlap < 1.0))
    return OWM_EINVAL;
  if (!std::isfinite(bbox->min_x) || !std::isfinite(bbox->min_y) || !std::isfinite(bbox->max_x) ||
      !std::isfinite(bbox->max_y) || bbox->max_x < bbox->min_x || bbox->max_y < bbox->min_y)
    return OWM_EINVAL;
  std::memset(p, 0, sizeof(*p));
  uint32_t Npoints = (uint32_t)npoints + 1;
  double Width = round2d(bbox->max_x - bbox->min_x);
  double Height = round2d(bbox->max_y - bbox->min_y);
  if (!(Width > 0.0) || !(Height > 0.0)) return OWM_EINVAL;  // density undefined
  double Density = (Npoints - 1) / (Width * Height);
  uint32_t minNumPoints = 0.5 * Density * Wsize * Wsize;
  double Displace = round2d(Wsize * (1 - Overlap));
  if (!(Displace > 0.0)) return OWM_EINVAL;  // overlap so close to 1 that windows never move
  unsigned short nCols, nRows;
  if (Overlap > 0.0) {
    nCols = (int)(std::round((Width + 2 * Wsize * Overlap) / Displace)) - 1;
    nRows = (int)(std::round((Height + 2 * Wsize * Overlap) / Displace)) - 1;
  } else {
    nCols = (int)std::floor(Width / Wsize) + 1;
    nRows = (int)std::floor(Height / Wsize) + 1;
  }
  p->npoints = npoints;
  p->wsize = Wsize;
  p->bsize = Bsize;
  p->overlap = Overlap;
  p->bbox = *bbox;
  p->width = Width;
  p->height = Height;
  p->density = Density;
  p->displace = Displace;
  p->min_num_points = (unsigned short)minNumPoints;
  p->ncols = nCols;
  p->nrows = nRows;
  p->ncells = (int64_t)nCols * nRows;
  if (Bsize > 0) {
    unsigned short nColsg = (int)std::floor(Width / Bsize) + 1;
    unsigned short nRowsg = (int)std::floor(Height / Bsize) + 1;
    p->ncols_grid = nColsg;
    p->nrows_grid = nRowsg;
    p->ngrid = (int64_t)nColsg * nRowsg;
  }
  return OWM_OK;
}

int owm_bbox_of(const double* xyz, int64_t n, owm_bbox* out) {
  if (!xyz || !out || n <= 0) return OWM_EINVAL;
  double x0 = xyz[0], x1 = xyz[0], y0 = xyz[1], y1 = xyz[1];
  for (int64_t i = 1; i < n; ++i) {
    double x = xyz[3 * i], y = xyz[3 * i + 1];
    x0 = x < x0 ? x : x0;
    x1 = x > x1 ? x : x1;
    y0 = y < y0 ? y : y0;
    y1 = y > y1 ? y : y1;
  }
  out->min_x = x0;
  out->min_y = y0;
  out->max_x = x1;
  out->max_y = y1;
  return OWM_OK;
}

void owm_host_free(void* p) { std::free(p); }

// readXYZfile (optim3_func.cpp:665-722), header variant: "N minx maxx miny
// maxy" then "x y z ..." lines.  Without a header the bbox is the data's.
// A line is the text up to its newline, however long (getline).
int owm_xyz_read(const char* path, double** xyz_out, int64_t* n_out, owm_bbox* bbox) {
  if (!path || !xyz_out || !n_out || !bbox) return OWM_EINVAL;
  FILE* f = std::fopen(path, "r");
  if (!f) return OWM_EIO;
  struct LineBuf {
    char* p = nullptr;
    size_t cap = 0;
    ~LineBuf() { std::free(p); }
    char* data() { return p; }
  } line;
  auto next_line = [&](void) -> bool { return ::getline(&line.p, &line.cap, f) >= 0; };
  // Decide header vs no header from the first non-empty line.
  if (!next_line()) {
    std::fclose(f);
    return OWM_EIO;
  }
  double a[3];
  int k = std::sscanf(line.data(), "%lf %lf %lf", &a[0], &a[1], &a[2]);
  std::vector<double> pts;
  int64_t declared = -1;
  owm_bbox hb{};
  bool have_header = false;
  if (k == 1) {
    declared = (int64_t)a[0];
    double v[4];
    for (int i = 0; i < 4; ++i) {
      if (!next_line() || std::sscanf(line.data(), "%lf", &v[i]) != 1) {
        std::fclose(f);
        return OWM_EIO;
      }
    }
    hb.min_x = v[0];
    hb.max_x = v[1];
    hb.min_y = v[2];
    hb.max_y = v[3];
    have_header = true;
    if (declared <= 0) {
      std::fclose(f);
      return OWM_EIO;
    }
    pts.reserve((size_t)declared * 3);
  } else if (k == 3) {
    pts.insert(pts.end(), a, a + 3);
  } else {
    std::fclose(f);
    return OWM_EIO;
  }
  while (next_line()) {
    if (have_header && (int64_t)pts.size() / 3 >= declared) break;
    if (std::sscanf(line.data(), "%lf %lf %lf", &a[0], &a[1], &a[2]) != 3) {
      // blank trailing lines are fine; anything else is a parse error
      bool blank = true;
      for (char* c = line.data(); *c; ++c)
        if (*c != ' ' && *c != '\n' && *c != '\r' && *c != '\t') blank = false;
      if (blank) continue;
      std::fclose(f);
      return OWM_EIO;
    }
    pts.insert(pts.end(), a, a + 3);
  }
  std::fclose(f);
  int64_t n = (int64_t)pts.size() / 3;
  if (n == 0 || (have_header && n < declared)) return OWM_EIO;  // short file
  for (double v : pts)
    if (!std::isfinite(v)) return OWM_EIO;
  double* out = (double*)std::malloc(pts.size() * sizeof(double));
  if (!out) return OWM_ENOMEM;
  std::memcpy(out, pts.data(), pts.size() * sizeof(double));
  *xyz_out = out;
  *n_out = n;
  if (have_header)
    *bbox = hb;
  else
    owm_bbox_of(out, n, bbox);
  return OWM_OK;
}

// Output dump format of owm_optim3.cpp:243-262 ("%.2f %.2f %.2f").
int owm_xyz_write_ids(const char* path, const double* xyz, int64_t n, const int64_t* ids,
                      int64_t n_ids) {
  if (!path || !xyz || (!ids && n_ids > 0)) return OWM_EINVAL;
  FILE* f = std::fopen(path, "w");
  if (!f) return OWM_EIO;
  for (int64_t k = 0; k < n_ids; ++k) {
    int64_t id = ids[k];
    if (id < 1 || id > n) {
      std::fclose(f);
      return OWM_EINVAL;
    }
    const double* p = xyz + 3 * (id - 1);
    std::fprintf(f, "%.2f %.2f %.2f\n", p[0], p[1], p[2]);
  }
  return std::fclose(f) == 0 ? OWM_OK : OWM_EIO;
}

// check_results (optim3_func.cpp:725-794): both lists sorted by z; an output
// point counts when some gold point lies strictly inside its displace/2 box
// with |dz| < 0.01; the score is count / n_gold * 100.  Id 0 is the
// reference's sentinel point {0, 0, DBL_MAX} (it looks up cloud[0] like any
// other id); ids outside 0..n, undefined behaviour there, are skipped here.
double owm_check_results(const double* gold, int64_t n_gold, const double* xyz, int64_t n,
                         const int64_t* ids, int64_t n_ids, float displace) {
  if (!gold || n_gold <= 0 || !xyz) return -1.0;
  struct P { double x, y, z; };
  std::vector<P> g((size_t)n_gold), v;
  for (int64_t i = 0; i < n_gold; ++i) g[(size_t)i] = {gold[3 * i], gold[3 * i + 1], gold[3 * i + 2]};
  for (int64_t k = 0; k < n_ids; ++k) {
    int64_t id = ids[k];
    if (id == 0) {
      v.push_back({0.0, 0.0, DBL_MAX});
      continue;
    }
    if (id < 1 || id > n) continue;
    const double* p = xyz + 3 * (id - 1);
    v.push_back({p[0], p[1], p[2]});
  }
  auto byz = [](const P& a, const P& b) { return a.z < b.z; };
  std::sort(g.begin(), g.end(), byz);
  std::sort(v.begin(), v.end(), byz);
  int64_t count = 0;
  double r = displace * 0.5;
  for (const P& p : v) {
    double x0 = p.x - r, x1 = p.x + r, y0 = p.y - r, y1 = p.y + r;
    for (const P& q : g) {
      if (q.x > x0 && q.y > y0 && q.x < x1 && q.y < y1 && std::fabs(p.z - q.z) < 0.01) {
        ++count;
        break;
      }
    }
  }
  return count / (double)n_gold * 100.0;
}

}  // extern "C"
