// Host-side parts of the OWM path that carry no device work: the driver's
// parameter arithmetic, cloud file I/O, the tolerant GOLD score, and the
// seeded synthetic cloud generator.
//
// Built with -ffp-contract=off: params and the generator must give the same
// bits on x86-64 and aarch64 (GCC contracts a+b*c on aarch64 by default).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
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

// owm_optim3.cpp:92-132, with the driver's types: Npoints counts the
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
// with |dz| < 0.01; the score is count / n_gold * 100.
double owm_check_results(const double* gold, int64_t n_gold, const double* xyz, int64_t n,
                         const int64_t* ids, int64_t n_ids, float displace) {
  if (!gold || n_gold <= 0 || !xyz) return -1.0;
  struct P { double x, y, z; };
  std::vector<P> g((size_t)n_gold), v;
  for (int64_t i = 0; i < n_gold; ++i) g[(size_t)i] = {gold[3 * i], gold[3 * i + 1], gold[3 * i + 2]};
  for (int64_t k = 0; k < n_ids; ++k) {
    int64_t id = ids[k];
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

// ---------------------------------------------------------------------------
// Synthetic clouds.  Counter-based: every random number is a pure function of
// (seed, point index, stream, draw), so the cloud does not depend on the
// thread count and is bit-identical on every machine (only +,-,*,/, floor,
// round and integer ops are used; no libm transcendental).
namespace {

inline uint64_t mix64(uint64_t z) {  // SplitMix64 finaliser
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
inline uint64_t rng(uint64_t seed, uint64_t idx, uint64_t stream, uint64_t draw) {
  return mix64(mix64(mix64(seed ^ (stream * 0xD1B54A32D192ED03ull)) + idx) + draw * 0x9E3779B97F4A7C15ull);
}
inline double u01(uint64_t r) { return (double)(r >> 11) * (1.0 / 9007199254740992.0); }

// Value noise on an integer lattice with smoothstep blending; lattice values
// in [-1, 1] from a hash of (ix, iy, octave, seed).
double lattice(uint64_t seed, int64_t ix, int64_t iy, int oct) {
  uint64_t h = mix64(seed * 0x632BE59BD9B4E019ull + (uint64_t)ix * 0x9E3779B97F4A7C15ull +
                     (uint64_t)iy * 0xC2B2AE3D27D4EB4Full + (uint64_t)oct * 0x165667B19E3779F9ull);
  return u01(h) * 2.0 - 1.0;
}
double value_noise(uint64_t seed, double x, double y, int oct) {
  double fx = std::floor(x), fy = std::floor(y);
  int64_t ix = (int64_t)fx, iy = (int64_t)fy;
  double tx = x - fx, ty = y - fy;
  double sx = tx * tx * (3.0 - 2.0 * tx), sy = ty * ty * (3.0 - 2.0 * ty);
  double v00 = lattice(seed, ix, iy, oct), v10 = lattice(seed, ix + 1, iy, oct);
  double v01 = lattice(seed, ix, iy + 1, oct), v11 = lattice(seed, ix + 1, iy + 1, oct);
  double a = v00 + (v10 - v00) * sx;
  double b = v01 + (v11 - v01) * sx;
  return a + (b - a) * sy;
}
// 6-octave fBm, local coordinates (m); total amplitude <= amp.
double fbm(uint64_t seed, double lx, double ly, double wavelength, double amp) {
  double sum = 0.0, a = 1.0, f = 1.0 / wavelength, norm = 0.0;
  for (int o = 0; o < 6; ++o) {
    sum += a * value_noise(seed, lx * f, ly * f, o);
    norm += a;
    a *= 0.5;
    f *= 2.0;
  }
  return amp * sum / norm;
}

struct Hole { double cx, cy, r2; };
struct Strip { double x0, x1, cum; };

}  // namespace

extern "C" {

int owm_synth_config(int config, int64_t tile, owm_synth_spec* s, uint32_t* W, double* O, uint32_t* B,
                     int32_t* max_number, uint64_t* seed) {
  if (!s) return OWM_EINVAL;
  std::memset(s, 0, sizeof(*s));
  uint64_t sd = (uint64_t)config * 1000ull + (uint64_t)tile;
  s->wavelength = 80.0;
  s->noise_sigma = 0.05;
  s->lift_lo = 0.5;
  s->lift_hi = 25.0;
  s->tie_free = 1;
  uint32_t w = 10, b = 20;
  double o = 0.8;
  int32_t mn = 32;
  switch (config) {
    case 1:
      s->n = 1000000;
      s->x0 = 500000.0; s->x1 = 500200.0; s->y0 = 4700000.0; s->y1 = 4700250.0;
      s->amplitude = 15.0;
      s->lifted_frac = 0.30;
      break;
    case 2:
      s->n = 100000000;
      s->x0 = 600000.0; s->x1 = 602000.0; s->y0 = 4500000.0; s->y1 = 4502000.0;
      s->amplitude = 40.0;
      s->lifted_frac = 0.25;
      w = 12;
      break;
    case 3:
      s->n = 20000000;
      s->x0 = 700000.0; s->x1 = 700800.0; s->y0 = 4600000.0; s->y1 = 4600800.0;
      s->amplitude = 15.0;
      s->lifted_frac = 0.20;
      s->z_quantum = 0.01;
      s->tie_free = 0;
      s->strips = 1;
      s->holes = 8;
      b = 15;
      break;
    case 4:
    case 5: {
      // per-tile draws from the tile's own seed (stream 7)
      double lo = config == 4 ? 5e4 : 1e4, hi = config == 4 ? 2e6 : 5e6;
      double u = u01(rng(sd, 0, 7, 0));
      // log-uniform count: lo * (hi/lo)^u, written with a product of squares
      // of a fixed-point exponent so no libm pow/exp is needed.
      double ratio = hi / lo, val = 1.0, base = ratio, e = u;
      for (int it = 0; it < 40; ++it) {  // binary expansion of e
        base = std::sqrt(base);          // correctly rounded everywhere
        e *= 2.0;
        if (e >= 1.0) {
          val *= base;
          e -= 1.0;
        }
      }
      s->n = (int64_t)(lo * val);
      double side = 100.0 + 400.0 * u01(rng(sd, 0, 7, 1));
      side = std::floor(side);
      double ox = 400000.0 + (double)(tile % 64) * 1000.0;
      double oy = 4400000.0 + (double)(tile / 64) * 1000.0;
      s->x0 = ox; s->x1 = ox + side; s->y0 = oy; s->y1 = oy + side;
      s->amplitude = 10.0 + 30.0 * u01(rng(sd, 0, 7, 2));
      s->lifted_frac = 0.10 + 0.30 * u01(rng(sd, 0, 7, 3));
      w = 8 + (uint32_t)(u01(rng(sd, 0, 7, 4)) * 9.0);
      if (w > 16) w = 16;
      break;
    }
    default:
      return OWM_EINVAL;
  }
  if (W) *W = w;
  if (O) *O = o;
  if (B) *B = b;
  if (max_number) *max_number = mn;
  if (seed) *seed = sd;
  return OWM_OK;
}

int owm_synth_cloud(const owm_synth_spec* s, uint64_t seed, double* xyz, owm_bbox* bbox,
                    int nthreads) {
  if (!s || !xyz || s->n <= 0 || !(s->x1 > s->x0) || !(s->y1 > s->y0)) return OWM_EINVAL;
  const int64_t n = s->n;
  const double wx = s->x1 - s->x0, wy = s->y1 - s->y0;

  // Strips (60 m bands along y, density U(5,60)) and holes, drawn from
  // stream 11 of the cloud seed.
  std::vector<Strip> strips;
  if (s->strips) {
    double cum = 0.0;
    int k = 0;
    for (double x = s->x0; x < s->x1; x += 60.0, ++k) {
      double x1 = x + 60.0 < s->x1 ? x + 60.0 : s->x1;
      double dens = 5.0 + 55.0 * u01(rng(seed, (uint64_t)k, 11, 0));
      cum += dens * (x1 - x);
      strips.push_back({x, x1, cum});
    }
    for (auto& st : strips) st.cum /= cum;
    strips.back().cum = 1.0;
  }
  std::vector<Hole> holes;
  for (int h = 0; h < s->holes; ++h) {
    double cx = s->x0 + wx * u01(rng(seed, (uint64_t)h, 12, 0));
    double cy = s->y0 + wy * u01(rng(seed, (uint64_t)h, 12, 1));
    double r = 30.0 + 90.0 * u01(rng(seed, (uint64_t)h, 12, 2));
    holes.push_back({cx, cy, r * r});
  }
  int idbits = 1;
  while (((int64_t)1 << idbits) < n + 1) ++idbits;
  const uint64_t idmask = ((uint64_t)1 << idbits) - 1;

  auto gen = [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) {
      double x = 0, y = 0;
      for (int attempt = 0; attempt < 64; ++attempt) {
        double ux = u01(rng(seed, (uint64_t)i, 1, (uint64_t)attempt));
        double uy = u01(rng(seed, (uint64_t)i, 2, (uint64_t)attempt));
        if (!strips.empty()) {
          // pick the strip by cumulative weight, then uniform inside it
          size_t lo = 0, hi = strips.size() - 1;
          while (lo < hi) {
            size_t mid = (lo + hi) / 2;
            if (ux < strips[mid].cum) hi = mid; else lo = mid + 1;
          }
          double prev = lo == 0 ? 0.0 : strips[lo - 1].cum;
          double t = (ux - prev) / (strips[lo].cum - prev);
          if (t >= 1.0) t = 0.9999999999;
          x = strips[lo].x0 + (strips[lo].x1 - strips[lo].x0) * t;
        } else {
          x = s->x0 + wx * ux;
        }
        y = s->y0 + wy * uy;
        bool in_hole = false;
        for (const Hole& h : holes) {
          double dx = x - h.cx, dy = y - h.cy;
          if (dx * dx + dy * dy < h.r2) { in_hole = true; break; }
        }
        if (!in_hole) break;  // after 64 hits the last draw is kept
      }
      double lx = x - s->x0, ly = y - s->y0;
      double z = 100.0 + fbm(seed, lx, ly, s->wavelength, s->amplitude);
      // ground noise: Irwin-Hall(12) - 6 ~ N(0, 1)
      double g = 0.0;
      for (int k = 0; k < 12; ++k) g += u01(rng(seed, (uint64_t)i, 3, (uint64_t)k));
      z += (g - 6.0) * s->noise_sigma;
      if (u01(rng(seed, (uint64_t)i, 4, 0)) < s->lifted_frac)
        z += s->lift_lo + (s->lift_hi - s->lift_lo) * u01(rng(seed, (uint64_t)i, 5, 0));
      if (s->z_quantum > 0.0) z = std::round(z / s->z_quantum) * s->z_quantum;
      if (s->tie_free) {
        // replace the low mantissa bits by the point index: all z distinct,
        // moved by < 2^idbits ulp (~2e-6 m at z ~ 100 m for 1e8 points)
        uint64_t bits;
        std::memcpy(&bits, &z, 8);
        bits = (bits & ~idmask) | ((uint64_t)i & idmask);
        std::memcpy(&z, &bits, 8);
      }
      xyz[3 * i] = x;
      xyz[3 * i + 1] = y;
      xyz[3 * i + 2] = z;
    }
  };
  int nt = nthreads > 0 ? nthreads : (int)std::max(1u, std::thread::hardware_concurrency());
  if (n < 65536) nt = 1;
  std::vector<std::thread> ts;
  for (int t = 0; t < nt; ++t) {
    int64_t b = n * t / nt, e = n * (t + 1) / nt;
    if (t == nt - 1) gen(b, e); else ts.emplace_back(gen, b, e);
  }
  for (auto& t : ts) t.join();
  if (bbox) owm_bbox_of(xyz, n, bbox);
  return OWM_OK;
}

}  // extern "C"
