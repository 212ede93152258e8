/*
 * Seeded synthetic LiDAR clouds for the project's five workloads.
 *
 * Counter-based: every random number is a pure function of (seed, point
 * index, stream, draw), so a cloud does not depend on the thread count and is
 * bit-identical on every machine (only +, -, *, /, floor, round, sqrt and
 * integer operations; no transcendental libm call).  Compile with
 * -ffp-contract=off (GCC contracts a + b*c on aarch64 by default).
 *
 * Plain C with no dependency on the rest of the library, so the same file is
 * compiled twice: into libowm_gb300.so as owm_synth_config / owm_synth_cloud,
 * and into the CPU oracle library with OWM_SYNTH_PREFIX=oracle_ (its
 * oracle_synth_* functions), which lets the CPU baseline generate the very same
 * cloud without loading the GPU library.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "owm_gb300.h"

#ifndef OWM_SYNTH_PREFIX
#define OWM_SYNTH_PREFIX owm_
#endif
#define OWM_SYNTH_CAT2(a, b) a##b
#define OWM_SYNTH_CAT(a, b) OWM_SYNTH_CAT2(a, b)
#define SYNTH_FN(name) OWM_SYNTH_CAT(OWM_SYNTH_PREFIX, name)

static inline uint64_t mix64(uint64_t z) { /* SplitMix64 finaliser */
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static inline uint64_t rng(uint64_t seed, uint64_t idx, uint64_t stream, uint64_t draw) {
  return mix64(mix64(mix64(seed ^ (stream * 0xD1B54A32D192ED03ull)) + idx) + draw * 0x9E3779B97F4A7C15ull);
}
static inline double u01(uint64_t r) { return (double)(r >> 11) * (1.0 / 9007199254740992.0); }

/* Value noise on an integer lattice with smoothstep blending; lattice values
 * in [-1, 1] from a hash of (ix, iy, octave, seed). */
static double lattice(uint64_t seed, int64_t ix, int64_t iy, int oct) {
  uint64_t h = mix64(seed * 0x632BE59BD9B4E019ull + (uint64_t)ix * 0x9E3779B97F4A7C15ull +
                     (uint64_t)iy * 0xC2B2AE3D27D4EB4Full + (uint64_t)oct * 0x165667B19E3779F9ull);
  return u01(h) * 2.0 - 1.0;
}
static double value_noise(uint64_t seed, double x, double y, int oct) {
  double fx = floor(x), fy = floor(y);
  int64_t ix = (int64_t)fx, iy = (int64_t)fy;
  double tx = x - fx, ty = y - fy;
  double sx = tx * tx * (3.0 - 2.0 * tx), sy = ty * ty * (3.0 - 2.0 * ty);
  double v00 = lattice(seed, ix, iy, oct), v10 = lattice(seed, ix + 1, iy, oct);
  double v01 = lattice(seed, ix, iy + 1, oct), v11 = lattice(seed, ix + 1, iy + 1, oct);
  double a = v00 + (v10 - v00) * sx;
  double b = v01 + (v11 - v01) * sx;
  return a + (b - a) * sy;
}
/* 6-octave fBm, local coordinates (m); total amplitude <= amp. */
static double fbm(uint64_t seed, double lx, double ly, double wavelength, double amp) {
  double sum = 0.0, a = 1.0, f = 1.0 / wavelength, norm = 0.0;
  for (int o = 0; o < 6; ++o) {
    sum += a * value_noise(seed, lx * f, ly * f, o);
    norm += a;
    a *= 0.5;
    f *= 2.0;
  }
  return amp * sum / norm;
}

typedef struct { double cx, cy, r2; } Hole;
typedef struct { double x0, x1, cum; } Strip;

int SYNTH_FN(synth_config)(int config, int64_t tile, owm_synth_spec* s, uint32_t* W, double* O, uint32_t* B,
                           int32_t* max_number, uint64_t* seed) {
  if (!s) return OWM_EINVAL;
  memset(s, 0, sizeof(*s));
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
      /* per-tile draws from the tile's own seed (stream 7) */
      double lo = config == 4 ? 5e4 : 1e4, hi = config == 4 ? 2e6 : 5e6;
      double u = u01(rng(sd, 0, 7, 0));
      /* log-uniform count: lo * (hi/lo)^u, written with a product of square
       * roots over the binary expansion of u, so no libm pow/exp is needed */
      double ratio = hi / lo, val = 1.0, base = ratio, e = u;
      for (int it = 0; it < 40; ++it) {
        base = sqrt(base); /* correctly rounded everywhere */
        e *= 2.0;
        if (e >= 1.0) {
          val *= base;
          e -= 1.0;
        }
      }
      s->n = (int64_t)(lo * val);
      double side = 100.0 + 400.0 * u01(rng(sd, 0, 7, 1));
      side = floor(side);
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

typedef struct {
  const owm_synth_spec* s;
  uint64_t seed;
  double* xyz;
  const Strip* strips;
  int nstrips;
  const Hole* holes;
  int nholes;
  uint64_t idmask;
  int64_t b, e;
} GenJob;

static void gen_range(const GenJob* J) {
  const owm_synth_spec* s = J->s;
  const uint64_t seed = J->seed;
  const double wx = s->x1 - s->x0, wy = s->y1 - s->y0;
  for (int64_t i = J->b; i < J->e; ++i) {
    double x = 0, y = 0;
    for (int attempt = 0; attempt < 64; ++attempt) {
      double ux = u01(rng(seed, (uint64_t)i, 1, (uint64_t)attempt));
      double uy = u01(rng(seed, (uint64_t)i, 2, (uint64_t)attempt));
      if (J->nstrips > 0) {
        /* pick the strip by cumulative weight, then uniform inside it */
        int lo = 0, hi = J->nstrips - 1;
        while (lo < hi) {
          int mid = (lo + hi) / 2;
          if (ux < J->strips[mid].cum) hi = mid; else lo = mid + 1;
        }
        double prev = lo == 0 ? 0.0 : J->strips[lo - 1].cum;
        double t = (ux - prev) / (J->strips[lo].cum - prev);
        if (t >= 1.0) t = 0.9999999999;
        x = J->strips[lo].x0 + (J->strips[lo].x1 - J->strips[lo].x0) * t;
      } else {
        x = s->x0 + wx * ux;
      }
      y = s->y0 + wy * uy;
      int in_hole = 0;
      for (int h = 0; h < J->nholes; ++h) {
        double dx = x - J->holes[h].cx, dy = y - J->holes[h].cy;
        if (dx * dx + dy * dy < J->holes[h].r2) { in_hole = 1; break; }
      }
      if (!in_hole) break; /* after 64 hits the last draw is kept */
    }
    double lx = x - s->x0, ly = y - s->y0;
    double z = 100.0 + fbm(seed, lx, ly, s->wavelength, s->amplitude);
    /* ground noise: Irwin-Hall(12) - 6 ~ N(0, 1) */
    double g = 0.0;
    for (int k = 0; k < 12; ++k) g += u01(rng(seed, (uint64_t)i, 3, (uint64_t)k));
    z += (g - 6.0) * s->noise_sigma;
    if (u01(rng(seed, (uint64_t)i, 4, 0)) < s->lifted_frac)
      z += s->lift_lo + (s->lift_hi - s->lift_lo) * u01(rng(seed, (uint64_t)i, 5, 0));
    if (s->z_quantum > 0.0) z = round(z / s->z_quantum) * s->z_quantum;
    if (s->tie_free) {
      /* replace the low mantissa bits by the point index: all z distinct,
       * moved by < 2^idbits ulp (~2e-6 m at z ~ 100 m for 1e8 points) */
      uint64_t bits;
      memcpy(&bits, &z, 8);
      bits = (bits & ~J->idmask) | ((uint64_t)i & J->idmask);
      memcpy(&z, &bits, 8);
    }
    J->xyz[3 * i] = x;
    J->xyz[3 * i + 1] = y;
    J->xyz[3 * i + 2] = z;
  }
}

static void* gen_thread(void* arg) {
  gen_range((const GenJob*)arg);
  return NULL;
}

int SYNTH_FN(synth_cloud)(const owm_synth_spec* s, uint64_t seed, double* xyz, owm_bbox* bbox, int nthreads) {
  if (!s || !xyz || s->n <= 0 || !(s->x1 > s->x0) || !(s->y1 > s->y0) || s->holes < 0) return OWM_EINVAL;
  const int64_t n = s->n;
  const double wx = s->x1 - s->x0, wy = s->y1 - s->y0;

  /* strips (60 m bands along y, density U(5,60)) and holes, drawn from
   * streams 11 and 12 of the cloud seed */
  Strip* strips = NULL;
  int nstrips = 0;
  if (s->strips) {
    int cap = (int)((s->x1 - s->x0) / 60.0) + 2;
    strips = (Strip*)malloc(sizeof(Strip) * (size_t)cap);
    if (!strips) return OWM_ENOMEM;
    double cum = 0.0;
    int k = 0;
    for (double x = s->x0; x < s->x1; x += 60.0, ++k) {
      double x1 = x + 60.0 < s->x1 ? x + 60.0 : s->x1;
      double dens = 5.0 + 55.0 * u01(rng(seed, (uint64_t)k, 11, 0));
      cum += dens * (x1 - x);
      if (nstrips == cap) break; /* unreachable: cap covers the loop */
      strips[nstrips].x0 = x;
      strips[nstrips].x1 = x1;
      strips[nstrips].cum = cum;
      ++nstrips;
    }
    for (int i = 0; i < nstrips; ++i) strips[i].cum /= cum;
    strips[nstrips - 1].cum = 1.0;
  }
  Hole* holes = s->holes > 0 ? (Hole*)malloc(sizeof(Hole) * (size_t)s->holes) : NULL;
  if (s->holes > 0 && !holes) {
    free(strips);
    return OWM_ENOMEM;
  }
  for (int h = 0; h < s->holes; ++h) {
    double cx = s->x0 + wx * u01(rng(seed, (uint64_t)h, 12, 0));
    double cy = s->y0 + wy * u01(rng(seed, (uint64_t)h, 12, 1));
    double r = 30.0 + 90.0 * u01(rng(seed, (uint64_t)h, 12, 2));
    holes[h].cx = cx;
    holes[h].cy = cy;
    holes[h].r2 = r * r;
  }
  int idbits = 1;
  while (((int64_t)1 << idbits) < n + 1) ++idbits;
  const uint64_t idmask = ((uint64_t)1 << idbits) - 1;

  long hw = sysconf(_SC_NPROCESSORS_ONLN);
  int nt = nthreads > 0 ? nthreads : (int)(hw > 0 ? hw : 1);
  if (n < 65536) nt = 1;
  if (nt > 1024) nt = 1024;
  GenJob* jobs = (GenJob*)malloc(sizeof(GenJob) * (size_t)nt);
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nt);
  if (!jobs || !th) {
    free(jobs);
    free(th);
    free(strips);
    free(holes);
    return OWM_ENOMEM;
  }
  int started = 0;
  for (int t = 0; t < nt; ++t) {
    GenJob J = {s, seed, xyz, strips, nstrips, holes, s->holes, idmask, n * t / nt, n * (t + 1) / nt};
    jobs[t] = J;
  }
  for (int t = 0; t + 1 < nt; ++t) {
    if (pthread_create(&th[t], NULL, gen_thread, &jobs[t]) != 0) break;
    ++started;
  }
  for (int t = started; t < nt; ++t) gen_range(&jobs[t]); /* the rest (at least the last) here */
  for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
  free(jobs);
  free(th);
  free(strips);
  free(holes);
  if (bbox) {
    double x0 = xyz[0], x1 = xyz[0], y0 = xyz[1], y1 = xyz[1];
    for (int64_t i = 1; i < n; ++i) {
      double x = xyz[3 * i], y = xyz[3 * i + 1];
      x0 = x < x0 ? x : x0;
      x1 = x > x1 ? x : x1;
      y0 = y < y0 ? y : y0;
      y1 = y > y1 ? y : y1;
    }
    bbox->min_x = x0;
    bbox->min_y = y0;
    bbox->max_x = x1;
    bbox->max_y = y1;
  }
  return OWM_OK;
}
