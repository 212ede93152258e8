// Cloud ingest on the device: the text of an .xyz file, parsed by GPU threads
// into a device cloud.  The file format and its rules are those of
// readXYZfile (CPP-TBB-CPU/src/optim3_func.cpp:665-722) as owm_xyz_read
// restates it line by line: an optional header (the point count, then
// min x, max x, min y, max y, one value per line), then one "x y z ..." line
// per point read with sscanf("%lf %lf %lf"); blank lines are skipped, any
// other line with fewer than three numbers is an error, non-finite values
// are rejected, and with a header the points after the declared count are
// not read.  map_file_atof_tbb_th (SYCL-CUDA-GPU/basic/utils.h:338-395) is
// the reference's fixed-column form of the same loader.
//
// Pipeline (text resident on the device, 16 bytes of readable slack):
//   k_nl_count   newlines per 2 KB segment (one warp, coalesced 16-byte loads)
//   scan         segment offsets
//   k_nl_starts  line start positions (byte masks, warp scan per round)
//   k_parse      one thread per line: the sscanf grammar on 16-byte loads,
//                values by Clinger's exact fast path (significand <= 2^53,
//                |decimal exponent| <= 22: one correctly rounded IEEE
//                multiply or divide), hex floats by exact rounding; a line
//                with any other decimal field is queued
//   k_parse_slow the queued lines again, every decimal field correctly
//                rounded by big-integer comparison with the halfway points
//                of the candidate doubles (a candidate from a table of
//                correctly rounded powers of ten, moved one double at a time)
//   resolve      first error line, points before it; the per-line values
//                become the cloud as they are when the first n lines are all
//                points, else blank lines are compacted out
// The values equal what the C library's correctly rounded conversion gives
// for the same text, bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "owm_ctx.cuh"

namespace owm {

namespace {

constexpr int kLinePoint = 0, kLineBlank = 1, kLineError = 2, kLineSlow = 3;
constexpr int kPowMin = -300, kPowMax = 300;

__constant__ double c_pow10[kPowMax - kPowMin + 1];  // correctly rounded 10^k, k = -300..300

// ---- text access ---------------------------------------------------------------
// Byte p of the line being parsed, through one cached 16-byte word; 0 past
// the line's end (a NUL byte also ends what sscanf sees).
struct TextCursor {
  using Pos = int64_t;  // positions in the text
  const uint4* __restrict__ base;
  int64_t end;
  int64_t wi;
  uint4 w;
  __device__ __forceinline__ TextCursor(const char* text, int64_t e) : base(reinterpret_cast<const uint4*>(text)), end(e), wi(-1) {}
  __device__ __forceinline__ uint32_t at(int64_t p) {
    if (p >= end) return 0;
    const int64_t i = p >> 4;
    if (i != wi) {
      w = __ldg(base + i);
      wi = i;
    }
    const uint32_t q = (uint32_t)(p >> 2) & 3u;
    const uint32_t word = q == 0 ? w.x : q == 1 ? w.y : q == 2 ? w.z : w.w;
    return (word >> ((uint32_t)(p & 3) * 8u)) & 0xFFu;
  }
};

// The same view of text staged in shared memory: bytes [origin, ...) of the
// text at base.
struct SmemCursor {
  using Pos = int32_t;  // positions relative to the start of the staged span
  const unsigned char* base;
  int32_t end;
  __device__ __forceinline__ uint32_t at(int32_t p) const { return p < end ? (uint32_t)base[p] : 0u; }
};

__device__ __forceinline__ bool is_space(uint32_t c) { return c == ' ' || (c >= 9 && c <= 13); }
__device__ __forceinline__ bool is_digit(uint32_t c) { return c - '0' < 10u; }
__device__ __forceinline__ int hex_val(uint32_t c) {
  if (c - '0' < 10u) return (int)(c - '0');
  const uint32_t l = c | 0x20u;
  if (l - 'a' < 6u) return (int)(l - 'a') + 10;
  return -1;
}

// ---- exact rounding of m * 2^e2 (+ sticky: the value is a little above) -----
__device__ double round_bits(uint64_t m, bool sticky, int64_t e2, bool neg) {
  const uint64_t sign = neg ? 0x8000000000000000ull : 0ull;
  if (m == 0) return __longlong_as_double((long long)sign);
  const int bl = 64 - __clzll((long long)m);
  const int64_t E = e2 + bl - 1;  // the value lies in [2^E, 2^(E+1))
  if (E > 1023) return __longlong_as_double((long long)(sign | 0x7FF0000000000000ull));
  const int64_t prec = E >= -1022 ? 53 : E + 1075;  // significant bits kept
  if (prec <= 0) {
    // below 2^-1074: 0, or the smallest subnormal when above half of it
    const bool up = prec == 0 && (sticky || (m & (m - 1)) != 0);
    return __longlong_as_double((long long)(sign | (up ? 1ull : 0ull)));
  }
  const int shift = bl - (int)prec;
  uint64_t mant;
  if (shift <= 0) {
    mant = m << (-shift);
  } else {
    mant = m >> shift;
    const uint64_t rem = m & ((1ull << shift) - 1), half = 1ull << (shift - 1);
    if (rem > half || (rem == half && (sticky || (mant & 1)))) ++mant;
  }
  uint64_t bits;
  if (E >= -1022)
    bits = ((uint64_t)(E + 1022) << 52) + mant;  // a carry to 2^53 moves into the exponent (inf past 1023)
  else
    bits = mant;  // subnormal: mant counts units of 2^-1074 (2^52 = smallest normal)
  return __longlong_as_double((long long)(sign | bits));
}

__device__ __forceinline__ void split_double(uint64_t bits, uint64_t* m, int64_t* q) {
  const uint64_t ef = bits >> 52, fr = bits & 0xFFFFFFFFFFFFFull;
  if (ef == 0) {
    *m = fr;
    *q = -1074;
  } else {
    *m = fr | 0x10000000000000ull;
    *q = (int64_t)ef - 1075;
  }
}

// ---- exact w / 10^k on 32-bit multiplies (1 <= k <= 13) ----------------------------
// The double of an integer w <= 2^53, from its bits (no FP64 instruction).
__device__ __forceinline__ double u53_to_double(uint64_t w) {
  if (w == 0) return 0.0;
  const int lz = __clzll((long long)w);
  return __longlong_as_double((long long)(((uint64_t)(1085 - lz) << 52) + ((w << lz) >> 11)));
}

// ---- w / 10^k with one multiply and an exact residual -------------------------------
// For an integer w <= 2^53 and 1 <= k <= 22, q0 = RN(w * RN(10^-k)) lies within
// 1.5 units in the last place of q* = w / 10^k.  With q0 = M * 2^E (E + k < 0
// here), w - 10^k * q0 = 2^(E+k) * I for an integer |I| <= 2.5 * 5^k < 2^53
// (also after a step of one unit), so the FMA residual
// rem = fma(-q0, 10^k, w) is exact and rem / 10^k = q* - q0.  Half a unit of
// q0 is 10^k * 2^(E-1) in residual terms (a power-of-two multiple of 10^k:
// exact); comparing |rem| with it as bit patterns (positive doubles order like
// their bits) moves q0 to the correctly rounded quotient, ties to even.  Two
// FP64 operations per step instead of a divide: on GB300 the FP64 pipe is the
// parse kernel's limit.
__device__ __forceinline__ double div_pow10_fma(uint64_t w, double dk, double rk) {
  const double x = u53_to_double(w);
  uint64_t qb = (uint64_t)__double_as_longlong(__dmul_rn(x, rk));
  const uint64_t db = (uint64_t)__double_as_longlong(dk);
  for (int it = 0; it < 4; ++it) {
    const double q = __longlong_as_double((long long)qb);
    const uint64_t rb = (uint64_t)__double_as_longlong(__fma_rn(-q, dk, x));
    const uint64_t ra = rb & 0x7FFFFFFFFFFFFFFFull;
    const uint64_t hb = db + ((uint64_t)((int64_t)(qb >> 52) - 1076) << 52);  // q is normal (q* >= 10^-22)
    const bool below = (rb >> 63) != 0;  // q > q*
    // the interval below a power of two is half as wide
    const uint64_t h = (below && !(qb & 0xFFFFFFFFFFFFFull)) ? hb - (1ull << 52) : hb;
    if (ra < h || (ra == h && !(qb & 1))) break;
    qb += below ? ~0ull : 1ull;  // one double towards q* (ties towards the even neighbour)
  }
  return __longlong_as_double((long long)qb);
}

// ---- big integers for the exact decimal path ----------------------------------
constexpr int kBigWords = 160;    // 5120 bits: decimal significands of up to 800 digits, scaled
constexpr int kMaxBigDigits = 800;

struct Big {
  uint32_t w[kBigWords];
  int n;
  __device__ void set_u64(uint64_t v) {
    w[0] = (uint32_t)v;
    w[1] = (uint32_t)(v >> 32);
    n = w[1] ? 2 : (w[0] ? 1 : 0);
  }
  __device__ void mul_add(uint32_t m, uint32_t a) {
    uint64_t carry = a;
    for (int i = 0; i < n; ++i) {
      const uint64_t t = (uint64_t)w[i] * m + carry;
      w[i] = (uint32_t)t;
      carry = t >> 32;
    }
    if (carry && n < kBigWords) w[n++] = (uint32_t)carry;
  }
  __device__ void mul_pow5(int64_t e) {
    while (e >= 13) {
      mul_add(1220703125u, 0);  // 5^13
      e -= 13;
    }
    uint32_t p = 1;
    while (e-- > 0) p *= 5u;
    if (p != 1) mul_add(p, 0);
  }
  __device__ void shl(int64_t bits) {
    if (n == 0 || bits <= 0) return;
    const int ws = (int)(bits >> 5), bs = (int)(bits & 31);
    int nn = n + ws + 1;
    if (nn > kBigWords) nn = kBigWords;  // sized so this never truncates (see the bounds in exact_decimal)
    for (int i = nn - 1; i >= 0; --i) {
      const int s = i - ws;
      uint32_t v = 0;
      if (s >= 0 && s < n) v = w[s] << bs;
      if (bs && s - 1 >= 0 && s - 1 < n) v |= w[s - 1] >> (32 - bs);
      w[i] = v;
    }
    n = nn;
    while (n > 0 && w[n - 1] == 0) --n;
  }
};

__device__ int big_cmp(const Big& a, const Big& b) {
  if (a.n != b.n) return a.n < b.n ? -1 : 1;
  for (int i = a.n - 1; i >= 0; --i)
    if (a.w[i] != b.w[i]) return a.w[i] < b.w[i] ? -1 : 1;
  return 0;
}

// Sign of D * 10^E - (2m + 1) * 2^(q - 1), D with `sticky` nonzero digits
// beyond it: the value against the halfway point above the double m * 2^q.
__device__ int cmp_halfway(const Big& D, int64_t E, bool sticky, uint64_t m, int64_t q, Big& L, Big& R) {
  L = D;
  R.set_u64(2 * m + 1);
  if (E >= 0)
    L.mul_pow5(E);
  else
    R.mul_pow5(-E);
  const int64_t e2 = E - (q - 1);
  if (e2 >= 0)
    L.shl(e2);
  else
    R.shl(-e2);
  int c = big_cmp(L, R);
  if (c == 0 && sticky) c = 1;
  return c;
}

// ---- field grammar -------------------------------------------------------------
constexpr int kFieldOk = 0, kFieldFail = 1, kFieldNonFinite = 2, kFieldSlow = 3;

struct Decimal {
  uint64_t w;     // first (up to) 19 significant digits
  int32_t nd;     // significant digits in all (a line is shorter than 2^31 bytes)
  int32_t dexp;   // value = (w + fraction of the dropped digits) * 10^dexp (|exponent| saturates at 10^8)
  bool sticky;    // a dropped digit is nonzero
};

// Exact decimal conversion of the mantissa at [ms, me) (digits and at most
// one '.') times 10^ev; `dec` is its 19-digit summary.
template <class Cursor>
__device__ double exact_decimal(Cursor& tc, typename Cursor::Pos ms, typename Cursor::Pos me, int64_t ev,
                                const Decimal& dec, bool neg,
                                Big* big) {
  const uint64_t sign = neg ? 0x8000000000000000ull : 0ull;
  const int64_t lead = (dec.nd < 19 ? dec.nd : 19) - 1 + dec.dexp;  // value in [10^lead, 10^(lead+1))
  if (lead >= 309) return __longlong_as_double((long long)(sign | 0x7FF0000000000000ull));
  if (lead <= -325) return __longlong_as_double((long long)sign);
  // D: the first kMaxBigDigits significant digits; E: its decimal exponent
  Big& D = big[0];
  D.n = 0;
  int64_t nd = 0, E = 0;
  bool seen_dot = false, sticky = false;
  uint32_t chunk = 0, cmul = 1;
  for (typename Cursor::Pos p = ms; p < me; ++p) {
    const uint32_t c = tc.at(p);
    if (c == '.') {
      seen_dot = true;
      continue;
    }
    const uint32_t d = c - '0';
    if (nd == 0 && d == 0) {
      if (seen_dot) --E;
      continue;
    }
    if (nd < kMaxBigDigits) {
      chunk = chunk * 10u + d;
      cmul *= 10u;
      if (cmul == 1000000000u) {
        D.mul_add(cmul, chunk);
        chunk = 0;
        cmul = 1;
      }
      ++nd;
      if (seen_dot) --E;
    } else {
      if (d) sticky = true;
      if (!seen_dot) ++E;
    }
  }
  if (cmul != 1) D.mul_add(cmul, chunk);
  E += ev;
  // candidate: w * 10^dexp in two correctly rounded steps (within a few units
  // in the last place, subnormal and overflowing results included)
  const int64_t a = dec.dexp < kPowMin ? kPowMin : (dec.dexp > kPowMax ? kPowMax : dec.dexp);
  const int64_t b = dec.dexp - a;  // |b| <= 50 by the lead bounds above
  double cand = __dmul_rn(__dmul_rn((double)dec.w, c_pow10[a - kPowMin]), c_pow10[b - kPowMin]);
  uint64_t bits = (uint64_t)__double_as_longlong(cand);
  if (bits == 0) bits = 1;                                   // start from the smallest subnormal
  if (bits >= 0x7FF0000000000000ull) bits = 0x7FEFFFFFFFFFFFFFull;  // ... or the largest finite double
  Big& L = big[1];
  Big& R = big[2];
  for (int it = 0; it < 64; ++it) {
    uint64_t m;
    int64_t q;
    split_double(bits, &m, &q);
    const int up = cmp_halfway(D, E, sticky, m, q, L, R);
    if (up > 0 || (up == 0 && (m & 1))) {
      if (bits == 0x7FEFFFFFFFFFFFFFull) return __longlong_as_double((long long)(sign | 0x7FF0000000000000ull));
      ++bits;
      continue;
    }
    uint64_t pm;
    int64_t pq;
    split_double(bits - 1, &pm, &pq);  // bits - 1 == 0: the halfway point 2^-1075 below the smallest subnormal
    const int down = cmp_halfway(D, E, sticky, pm, pq, L, R);
    if (down < 0 || (down == 0 && !(pm & 1))) {
      if (bits == 1) return __longlong_as_double((long long)sign);
      --bits;
      continue;
    }
    return __longlong_as_double((long long)(sign | bits));
  }
  return __longlong_as_double((long long)(sign | 0x7FF8000000000000ull));  // unreachable: a NaN fails the load
}

// One sscanf %lf conversion at p (whitespace already skipped).  On success
// *v and *end are set.  kExact: decimal fields that need the slow path are
// converted here (big = 3 scratch integers); otherwise they report
// kFieldSlow.
template <bool kExact, class Cursor>
__device__ int parse_field(Cursor& tc, typename Cursor::Pos p, double* v, typename Cursor::Pos* end, Big* big) {
  bool neg = false;
  uint32_t c = tc.at(p);
  if (c == '+' || c == '-') {
    neg = c == '-';
    c = tc.at(++p);
  }
  const uint32_t lc = c | 0x20u;
  if (lc == 'i' || lc == 'n') return kFieldNonFinite;  // inf/nan (or a failed match): the load fails either way
  if (c == '0' && (tc.at(p + 1) | 0x20u) == 'x') {
    // hex: [hex digits][. [hex digits]], then p[+-][digits]; fails only when
    // nothing follows "0x"
    p += 2;
    uint64_t m = 0;
    int hd = 0;
    int64_t bexp = 0;
    bool sticky = false, seen_dot = false, consumed = false;
    for (;;) {
      c = tc.at(p);
      const int hv = hex_val(c);
      if (hv >= 0) {
        consumed = true;
        if (hd == 0 && hv == 0) {
          if (seen_dot) bexp -= 4;
        } else if (hd < 16) {
          m = m * 16u + (uint64_t)hv;
          ++hd;
          if (seen_dot) bexp -= 4;
        } else {
          ++hd;
          if (hv) sticky = true;
          if (!seen_dot) bexp += 4;
        }
        ++p;
      } else if (c == '.' && !seen_dot) {
        seen_dot = consumed = true;
        ++p;
      } else {
        break;
      }
    }
    if (!consumed) return kFieldFail;
    if ((tc.at(p) | 0x20u) == 'p') {
      c = tc.at(++p);
      bool eneg = false;
      if (c == '+' || c == '-') {
        eneg = c == '-';
        ++p;
      }
      int64_t ev = 0;
      while (is_digit(c = tc.at(p))) {
        if (ev < 100000000) ev = ev * 10 + (c - '0');
        ++p;
      }
      bexp += eneg ? -ev : ev;
    }
    *v = round_bits(m, sticky, bexp, neg);
    *end = p;
    return isfinite(*v) ? kFieldOk : kFieldNonFinite;
  }
  // decimal: [digits][. [digits]] with at least one digit, then e[+-][digits]
  const typename Cursor::Pos ms = p;
  Decimal dec{0, 0, 0, false};
  bool any = false, seen_dot = false;
  for (;;) {
    c = tc.at(p);
    if (is_digit(c)) {
      any = true;
      const uint32_t d = c - '0';
      if (dec.nd == 0 && d == 0) {
        if (seen_dot) --dec.dexp;
      } else if (dec.nd < 19) {
        dec.w = dec.w * 10u + d;
        ++dec.nd;
        if (seen_dot) --dec.dexp;
      } else {
        ++dec.nd;
        if (d) dec.sticky = true;
        if (!seen_dot) ++dec.dexp;
      }
      ++p;
    } else if (c == '.' && !seen_dot) {
      seen_dot = true;
      ++p;
    } else {
      break;
    }
  }
  if (!any) return kFieldFail;
  const typename Cursor::Pos me = p;
  int64_t ev = 0;
  if ((tc.at(p) | 0x20u) == 'e') {
    c = tc.at(++p);
    bool eneg = false;
    if (c == '+' || c == '-') {
      eneg = c == '-';
      ++p;
    }
    while (is_digit(c = tc.at(p))) {
      if (ev < 100000000) ev = ev * 10 + (c - '0');
      ++p;
    }
    if (eneg) ev = -ev;
  }
  *end = p;
  dec.dexp += ev;
  if (dec.w == 0) {  // every digit is zero
    *v = neg ? -0.0 : 0.0;
    return kFieldOk;
  }
  if (!dec.sticky && dec.w <= (1ull << 53)) {
    int64_t e = dec.dexp;
    uint64_t w = dec.w;
    while (e > 22 && w <= (1ull << 53) / 10) {  // move powers of ten into an exact significand
      w *= 10;
      --e;
    }
    if (e >= -22 && e <= 22) {
      // e >= 0: one correctly rounded multiply of exact operands (Clinger);
      // e < 0: the quotient from an exact residual (div_pow10_fma)
      const double r = e >= 0 ? __dmul_rn(u53_to_double(w), c_pow10[e - kPowMin])
                              : div_pow10_fma(w, c_pow10[-e - kPowMin], c_pow10[e - kPowMin]);
      *v = neg ? -r : r;
      return isfinite(r) ? kFieldOk : kFieldNonFinite;
    }
  }
  if (!kExact) return kFieldSlow;
  *v = exact_decimal(tc, ms, me, ev, dec, neg, big);
  return isfinite(*v) ? kFieldOk : kFieldNonFinite;
}

// sscanf(line, "%lf %lf %lf") and owm_xyz_read's verdict on the line
// [s, e) read through tc.
template <bool kExact, class Cursor>
__device__ int parse_line(Cursor& tc, typename Cursor::Pos s, double* out, Big* big) {
  typename Cursor::Pos p = s;
  int f = 0;
#pragma unroll
  for (; f < 3; ++f) {
    uint32_t c;
    while ((c = tc.at(p)) != 0 && is_space(c)) ++p;
    if (c == 0) break;
    typename Cursor::Pos end;
    const int r = parse_field<kExact, Cursor>(tc, p, out + f, &end, big);
    if (r == kFieldSlow) return kLineSlow;
    if (r == kFieldNonFinite) return kLineError;
    if (r == kFieldFail) break;
    p = end;
  }
  if (f == 3) return kLinePoint;
  // blank lines (spaces, tabs, CR only, up to a NUL) are skipped
  for (p = s;; ++p) {
    const uint32_t c = tc.at(p);
    if (c == 0) return kLineBlank;
    if (c != ' ' && c != '\t' && c != '\r' && c != '\n') return kLineError;
  }
}

// ---- kernels -------------------------------------------------------------------
constexpr int64_t kSegBytes = 2048;  // one warp per segment: four rounds of 32 lanes x 16 bytes

// 0xFF in every byte of x that is a newline.
__device__ __forceinline__ uint32_t nl_bytes(uint32_t x) { return __vcmpeq4(x, 0x0A0A0A0Au); }

// Newline masks of lane's 16 bytes at o (bytes at or past `end` masked off).
__device__ __forceinline__ void nl_masks(const char* __restrict__ text, int64_t o, int64_t end, uint32_t m[4]) {
  if (o >= end) {
    m[0] = m[1] = m[2] = m[3] = 0;
    return;
  }
  const uint4 w = __ldg(reinterpret_cast<const uint4*>(text + o));
  m[0] = nl_bytes(w.x);
  m[1] = nl_bytes(w.y);
  m[2] = nl_bytes(w.z);
  m[3] = nl_bytes(w.w);
  const int64_t valid = end - o;  // bytes of this word inside the range
  if (valid < 16) {
    for (int j = 0; j < 4; ++j) {
      const int64_t vb = valid - 4 * j;  // valid bytes of word j
      if (vb <= 0)
        m[j] = 0;
      else if (vb < 4)
        m[j] &= (1u << (8 * vb)) - 1;
    }
  }
}

// Newlines of segment s = [begin + s*kSegBytes, ...) within [begin, end); one
// warp per segment, coalesced 16-byte loads.  begin is 16-byte aligned.
__global__ void __launch_bounds__(256) k_nl_count(const char* __restrict__ text, int64_t begin, int64_t end,
                                                  int64_t nseg, uint32_t* __restrict__ seg_count) {
  const int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (s >= nseg) return;  // warp-uniform
  const int lane = threadIdx.x & 31;
  uint32_t cnt = 0;
  for (int r = 0; r < 4; ++r) {
    uint32_t m[4];
    nl_masks(text, begin + s * kSegBytes + r * 512 + lane * 16, end, m);
    cnt += (__popc(m[0]) + __popc(m[1]) + __popc(m[2]) + __popc(m[3])) >> 3;
  }
  for (int o = 16; o >= 1; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if (lane == 0) seg_count[s] = cnt;
}

// starts[k + 1] = position after the k-th newline of [begin, end) (k from 0),
// in order; seg_off = scanned segment counts.
__global__ void __launch_bounds__(256) k_nl_starts(const char* __restrict__ text, int64_t begin, int64_t end,
                                                   int64_t nseg, const uint32_t* __restrict__ seg_off,
                                                   int64_t* __restrict__ starts) {
  const int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (s >= nseg) return;  // warp-uniform
  const int lane = threadIdx.x & 31;
  int64_t base = seg_off[s];
  for (int r = 0; r < 4; ++r) {
    const int64_t o = begin + s * kSegBytes + r * 512 + lane * 16;
    uint32_t m[4];
    nl_masks(text, o, end, m);
    const uint32_t c = (__popc(m[0]) + __popc(m[1]) + __popc(m[2]) + __popc(m[3])) >> 3;
    uint32_t inc = c;
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, inc, d);
      if (lane >= d) inc += t;
    }
    int64_t k = base + inc - c;  // this lane's first newline index
    for (int j = 0; j < 4; ++j) {
      uint32_t mj = m[j];
      while (mj) {
        const int byte = (__ffs(mj) - 1) >> 3;
        starts[++k] = o + 4 * j + byte + 1;
        mj &= ~(0xFFu << (8 * byte));
      }
    }
    base += __shfl_sync(0xffffffffu, inc, 31);
  }
}

struct ParseOut {
  double* vals;             // [nlines][4]: cloud records x, y, z, 0
  double* xy;               // [nlines][2]: the cloud's x, y array
  uint8_t* status;          // [nlines]
  int64_t* slow;            // queued line indices
  unsigned long long* nslow;
  unsigned long long* first_error;  // lowest error line (atomic min)
  unsigned long long* nblank;       // blank lines
};

// Line i's point as record i of a cloud (two 16-byte stores: the whole
// 32-byte record, pad included) and entry i of its x, y array.
__device__ __forceinline__ void put_record(const ParseOut& o, int64_t i, const double* v) {
  double2* d = reinterpret_cast<double2*>(o.vals + 4 * i);
  d[0] = make_double2(v[0], v[1]);
  d[1] = make_double2(v[2], 0.0);
  reinterpret_cast<double2*>(o.xy)[i] = make_double2(v[0], v[1]);
}

// One thread per line i: [starts[i], starts[i+1] - 1) (the newline excluded).
// A warp takes 32 consecutive lines: their text is one contiguous span, which
// the warp stages in shared memory with coalesced 16-byte loads, so every
// lane then reads its line a byte per load (spans over kStageBytes are read
// from global memory instead).
constexpr int kStageBytes = 4096;

__global__ void __launch_bounds__(256, 4) k_parse(const char* __restrict__ text, const int64_t* __restrict__ starts,
                                               int64_t nlines, int64_t nbytes, ParseOut o) {
  __shared__ __align__(16) unsigned char stage[8][kStageBytes];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t l0 = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; l0 < nlines; l0 += nwarps * 32) {
    const int64_t l1 = l0 + 32 < nlines ? l0 + 32 : nlines;
    const int64_t b0 = starts[l0] & ~(int64_t)15;  // 16-byte aligned start of the span
    const int64_t b1 = starts[l1] - 1 < nbytes ? starts[l1] - 1 : nbytes;  // end of the last line
    const bool staged = b1 - b0 <= kStageBytes;     // warp-uniform
    if (staged) {
      for (int64_t q = b0 + lane * 16; q < b1; q += 512)  // q - b0 <= kStageBytes - 16
        *reinterpret_cast<uint4*>(stage[wib] + (q - b0)) = __ldg(reinterpret_cast<const uint4*>(text + q));
      __syncwarp();
    }
    const int64_t i = l0 + lane;
    int st = -1;
    if (i < nlines) {
      const int64_t s = starts[i], e = starts[i + 1] - 1;
      double v[3];
      if (staged) {
        SmemCursor tc{stage[wib], (int32_t)(e - b0)};
        st = parse_line<false>(tc, (int32_t)(s - b0), v, nullptr);
      } else {
        TextCursor tc(text, e);
        st = parse_line<false>(tc, s, v, nullptr);
      }
      o.status[i] = (uint8_t)st;
      if (st == kLinePoint) {
        put_record(o, i, v);
      } else if (st == kLineSlow) {
        o.slow[atomicAdd(o.nslow, 1ull)] = i;
      } else if (st == kLineError) {
        atomicMin(o.first_error, (unsigned long long)i);
      }
    }
    const uint32_t blank = __ballot_sync(0xffffffffu, st == kLineBlank);
    if (lane == 0 && blank) atomicAdd(o.nblank, (unsigned long long)__popc(blank));
    __syncwarp();  // the stage is refilled in the next round
  }
}

// The queued lines, every field correctly rounded (three big integers of
// scratch per thread, in local memory: this kernel alone carries them).
__global__ void __launch_bounds__(128) k_parse_slow(const char* __restrict__ text,
                                                    const int64_t* __restrict__ starts, ParseOut o) {
  Big big[3];
  const int64_t ns = (int64_t)*o.nslow;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < ns; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = o.slow[k];
    double v[3];
    TextCursor tc(text, starts[i + 1] - 1);
    const int st = parse_line<true>(tc, starts[i], v, big);
    o.status[i] = (uint8_t)st;
    if (st == kLinePoint) {
      put_record(o, i, v);
    } else {
      atomicMin(o.first_error, (unsigned long long)i);  // a queued line is a point or an error
    }
  }
}

// First error line (atomic min) and point flags.
__global__ void k_line_flags(const uint8_t* __restrict__ status, int64_t nlines, uint32_t* __restrict__ is_point,
                             unsigned long long* __restrict__ first_error) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nlines;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int st = status[i];
    is_point[i] = st == kLinePoint;
    if (st == kLineError || st == kLineSlow) atomicMin(first_error, (unsigned long long)i);
  }
}

// Points [0, n) of the flagged lines, in line order, into out (cloud records)
// and out_xy (its x, y array).
__global__ void k_compact_points(const double* __restrict__ vals, const uint32_t* __restrict__ is_point,
                                 const uint32_t* __restrict__ pos, int64_t nlines, int64_t n, double* __restrict__ out,
                                 double* __restrict__ out_xy) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nlines;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (!is_point[i] || pos[i] >= (uint64_t)n) continue;
    const int64_t j = pos[i];
    const double2* r = reinterpret_cast<const double2*>(vals + 4 * i);
    double2* d = reinterpret_cast<double2*>(out + 4 * j);
    const double2 a = r[0];
    d[0] = a;
    d[1] = r[1];
    reinterpret_cast<double2*>(out_xy)[j] = a;
  }
}

int grid_of(int64_t n, int block) {
  int64_t g = (n + block - 1) / block;
  return (int)std::max<int64_t>(1, std::min<int64_t>(g, 152 * 16));
}

size_t a256(size_t b) { return (b + 255) & ~(size_t)255; }

// Powers of ten for the device, once per device: the C library's correctly
// rounded conversion of "1e<k>".
std::mutex g_pow_mu;
std::vector<int> g_pow_ready;

int ensure_pow10(int device) {
  std::lock_guard<std::mutex> lk(g_pow_mu);
  if ((int)g_pow_ready.size() <= device) g_pow_ready.resize(device + 1, 0);
  if (g_pow_ready[device]) return OWM_OK;
  double tab[kPowMax - kPowMin + 1];
  char buf[16];
  for (int k = kPowMin; k <= kPowMax; ++k) {
    std::snprintf(buf, sizeof(buf), "1e%d", k);
    tab[k - kPowMin] = std::strtod(buf, nullptr);
  }
  OWM_CUDA_TRY(cudaMemcpyToSymbol(c_pow10, tab, sizeof(tab)));
  g_pow_ready[device] = 1;
  return OWM_OK;
}

// First line [s, e) of host text at or after `from` (e excludes '\n');
// false at the end of the text.
bool host_line(const char* text, int64_t nbytes, int64_t from, int64_t* s, int64_t* e) {
  if (from >= nbytes) return false;
  const void* nl = std::memchr(text + from, '\n', (size_t)(nbytes - from));
  *s = from;
  *e = nl ? (const char*)nl - text : nbytes;
  return true;
}

}  // namespace

// Header of owm_xyz_read on host text: *data_off = first data byte,
// *declared = -1 without a header.  Same sscanf calls as the host loader.
int xyz_header(const char* text, int64_t nbytes, int64_t* data_off, int64_t* declared, owm_bbox* hb) {
  int64_t s, e;
  if (!host_line(text, nbytes, 0, &s, &e)) return OWM_EIO;
  std::vector<char> line((size_t)(e - s) + 2);
  auto load = [&](int64_t a, int64_t b) {
    line.assign((size_t)(b - a) + 2, 0);
    std::memcpy(line.data(), text + a, (size_t)(b - a));
    line[(size_t)(b - a)] = '\n';
  };
  load(s, e);
  double a[3];
  const int k = std::sscanf(line.data(), "%lf %lf %lf", &a[0], &a[1], &a[2]);
  if (k == 3) {
    *data_off = 0;
    *declared = -1;
    return OWM_OK;
  }
  if (k != 1) return OWM_EIO;
  if (!(a[0] >= 1.0 && a[0] < 9.2e18)) return OWM_EIO;
  *declared = (int64_t)a[0];
  double v[4];
  int64_t from = e + 1;
  for (int i = 0; i < 4; ++i) {
    if (!host_line(text, nbytes, from, &s, &e)) return OWM_EIO;
    load(s, e);
    if (std::sscanf(line.data(), "%lf", &v[i]) != 1) return OWM_EIO;
    from = e + 1;
  }
  hb->min_x = v[0];
  hb->max_x = v[1];
  hb->min_y = v[2];
  hb->max_y = v[3];
  *data_off = from < nbytes ? from : nbytes;
  return OWM_OK;
}

// Parses device text [0, nbytes) (16 bytes of slack after it, 16-byte
// aligned) whose data lines start at data_off, into the cloud's buffer.
int parse_device_text(owm_ctx* c, const char* dtext, int64_t nbytes, int64_t data_off, int64_t declared,
                      DeviceBuffer* out_mem, DeviceBuffer* out_xy, int64_t* n_out, int64_t* launches) {
  cudaStream_t s = c->stream;
  int rc = ensure_pow10(c->device);
  if (rc) return rc;
  // tiles start at a 16-byte boundary below data_off; bytes before it are not counted
  const int64_t begin = data_off & ~(int64_t)15;
  const int64_t span = nbytes - begin;
  const int64_t ntiles = std::max<int64_t>(1, (span + kSegBytes - 1) / kSegBytes);  // segments
  // newline positions in [begin, data_off) must not count: the count runs from data_off
  // itself, so tiles use the exact byte range [data_off, nbytes)
  // working buffers, released on every return (early CUDA-error returns included)
  DeviceBuffer tmp, vbuf, xybuf, work;
  struct Release {
    DeviceBuffer* b[4];
    cudaStream_t s;
    ~Release() {
      for (DeviceBuffer* x : b) x->release(s);
    }
  } release_all{{&tmp, &vbuf, &xybuf, &work}, s};
  const size_t tb = a256((size_t)ntiles * 4) * 2 + a256(scan_temp_bytes(ntiles)) + 256;
  rc = tmp.reserve(tb, s);
  if (rc) return rc;
  char* tp = static_cast<char*>(tmp.ptr);
  uint32_t* tcount = reinterpret_cast<uint32_t*>(tp);
  uint32_t* toff = reinterpret_cast<uint32_t*>(tp + a256((size_t)ntiles * 4));
  void* stemp = tp + 2 * a256((size_t)ntiles * 4);
  uint32_t* d_total = reinterpret_cast<uint32_t*>(c->d_small + kCountSlot);
  const unsigned seg_blocks = (unsigned)((ntiles * 32 + 255) / 256);  // one warp per segment
  OWM_LAUNCH("k_nl_count", s, k_nl_count<<<seg_blocks, 256, 0, s>>>(dtext, begin, nbytes, ntiles, tcount));
  count_launch(launches);
  // newlines between begin and data_off belong to the header: subtract them on the host
  OWM_CUDA_TRY(exclusive_scan_u32(tcount, toff, ntiles, d_total, stemp, scan_temp_bytes(ntiles), s, launches));
  uint32_t total_nl = 0;
  OWM_CUDA_TRY(cudaMemcpyAsync(&total_nl, d_total, 4, cudaMemcpyDeviceToHost, s));
  OWM_CUDA_TRY(cudaStreamSynchronize(s));
  // header newlines inside [begin, data_off): at most 15 bytes, counted on the device copy's host twin
  int64_t hdr_nl = 0;
  if (data_off > begin) {
    char hb[16];
    OWM_CUDA_TRY(cudaMemcpy(hb, dtext + begin, (size_t)(data_off - begin), cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < data_off - begin; ++i) hdr_nl += hb[i] == '\n';
  }
  const int64_t nl = (int64_t)total_nl - hdr_nl;
  char last = '\n';
  if (nbytes > data_off) OWM_CUDA_TRY(cudaMemcpy(&last, dtext + nbytes - 1, 1, cudaMemcpyDeviceToHost));
  const int64_t nlines = nl + (nbytes > data_off && last != '\n' ? 1 : 0);
  if (nlines <= 0) return OWM_EIO;
  // line starts: starts[0] = data_off; starts[k] (k >= 1) after the k-th data newline
  // (k_nl_starts numbers newlines from begin, so its index is shifted by hdr_nl)
  // per-line values in their own buffer: when the first n lines are all
  // points it becomes the cloud as it is (no compaction)
  rc = vbuf.reserve((size_t)nlines * 8 * kCloudStride, s);
  if (!rc) rc = xybuf.reserve((size_t)nlines * 8 * kCloudXyStride, s);
  if (rc) return rc;
  const size_t lb = a256((size_t)(nlines + 1 + hdr_nl + 1) * 8) + a256((size_t)nlines) +
                    2 * a256((size_t)nlines * 4) + a256((size_t)nlines * 8) + a256(scan_temp_bytes(nlines)) + 1024;
  rc = work.reserve(lb, s);
  if (rc) return rc;
  char* wp = static_cast<char*>(work.ptr);
  auto take = [&](size_t b) {
    void* q = wp;
    wp += a256(b);
    return q;
  };
  int64_t* starts_all = (int64_t*)take((size_t)(nlines + 1 + hdr_nl + 1) * 8);
  double* vals = static_cast<double*>(vbuf.ptr);
  uint8_t* status = (uint8_t*)take((size_t)nlines);
  uint32_t* is_point = (uint32_t*)take((size_t)nlines * 4);
  uint32_t* pos = (uint32_t*)take((size_t)nlines * 4);
  int64_t* slow = (int64_t*)take((size_t)nlines * 8);
  void* ctemp = take(scan_temp_bytes(nlines));
  unsigned long long* dwords = reinterpret_cast<unsigned long long*>(c->d_small + kBboxSlot);  // [0] nslow, [1] first error
  OWM_LAUNCH("k_nl_starts", s, k_nl_starts<<<seg_blocks, 256, 0, s>>>(dtext, begin, nbytes, ntiles, toff, starts_all));
  count_launch(launches);
  int64_t* starts = starts_all + hdr_nl;  // starts[0] is the slot before the first data newline
  const int64_t first = data_off, endpos = nbytes + 1;
  OWM_CUDA_TRY(cudaMemcpyAsync(starts, &first, 8, cudaMemcpyHostToDevice, s));
  if (nlines > nl) OWM_CUDA_TRY(cudaMemcpyAsync(starts + nlines, &endpos, 8, cudaMemcpyHostToDevice, s));
  const unsigned long long init[3] = {0ull, ~0ull, 0ull};  // queued lines, first error line, blank lines
  OWM_CUDA_TRY(cudaMemcpyAsync(dwords, init, 24, cudaMemcpyHostToDevice, s));
  ParseOut po{vals, static_cast<double*>(xybuf.ptr), status, slow, dwords, dwords + 1, dwords + 2};
  OWM_LAUNCH("k_parse", s, k_parse<<<grid_of((nlines + 31) / 32 * 32, 256), 256, 0, s>>>(dtext, starts, nlines, nbytes, po));
  OWM_LAUNCH("k_parse_slow", s, k_parse_slow<<<152 * 2, 128, 0, s>>>(dtext, starts, po));
  count_launch(launches, 2);
  unsigned long long h[3];
  OWM_CUDA_TRY(cudaMemcpyAsync(h, dwords, 24, cudaMemcpyDeviceToHost, s));
  OWM_CUDA_TRY(cudaStreamSynchronize(s));
  // points before the first error line: the loader stops at that line unless
  // the declared count was reached before it.  Without blank lines every line
  // before it is a point; with blank lines the point flags are scanned.
  const bool scanned = h[2] != 0;
  int64_t npts = h[1] != ~0ull ? (int64_t)h[1] : nlines;
  int64_t before = npts;
  if (scanned) {
    OWM_LAUNCH("k_line_flags", s, k_line_flags<<<grid_of(nlines, 256), 256, 0, s>>>(status, nlines, is_point, dwords + 1));
    count_launch(launches);
    uint32_t* d_npts = reinterpret_cast<uint32_t*>(c->d_small + kCountSlot);
    OWM_CUDA_TRY(exclusive_scan_u32(is_point, pos, nlines, d_npts, ctemp, scan_temp_bytes(nlines), s, launches));
    uint32_t np = 0;
    OWM_CUDA_TRY(cudaMemcpyAsync(&np, d_npts, 4, cudaMemcpyDeviceToHost, s));
    OWM_CUDA_TRY(cudaStreamSynchronize(s));
    npts = np;
    before = np;
    if (h[1] != ~0ull) {
      uint32_t pb = 0;
      OWM_CUDA_TRY(cudaMemcpy(&pb, pos + h[1], 4, cudaMemcpyDeviceToHost));
      before = pb;
    }
  }
  int64_t n;
  if (declared >= 0) {
    if (before < declared) rc = OWM_EIO;  // an error line or a short file before the declared count
    n = declared;
  } else {
    if (h[1] != ~0ull) rc = OWM_EIO;
    n = npts;
  }
  if (!rc && (n <= 0 || n >= 0x7FFFFFFFLL)) rc = OWM_EIO;
  bool in_place = false;  // the first n lines are all points
  if (!rc && !scanned) {
    in_place = n <= before;  // no blank line: lines before the first error are points
  } else if (!rc && n <= nlines) {
    uint32_t pn = (uint32_t)npts;
    if (n < nlines) OWM_CUDA_TRY(cudaMemcpy(&pn, pos + n, 4, cudaMemcpyDeviceToHost));
    in_place = (int64_t)pn == n;
  }
  if (!rc && in_place) {
    out_mem->release(s);
    *out_mem = vbuf;
    vbuf.ptr = nullptr;
    vbuf.cap = 0;
    out_xy->release(s);
    *out_xy = xybuf;
    xybuf.ptr = nullptr;
    xybuf.cap = 0;
  } else if (!rc) {
    rc = out_mem->reserve((size_t)n * 8 * kCloudStride, s);
    if (!rc) rc = out_xy->reserve((size_t)n * 8 * kCloudXyStride, s);
    if (!rc) {
      OWM_LAUNCH("k_compact_points", s, k_compact_points<<<grid_of(nlines, 256), 256, 0, s>>>(
          vals, is_point, pos, nlines, n, static_cast<double*>(out_mem->ptr), static_cast<double*>(out_xy->ptr)));
      count_launch(launches);
    }
  }
  OWM_CUDA_TRY(cudaStreamSynchronize(s));
  if (!rc) *n_out = n;
  return rc;
}

}  // namespace owm
