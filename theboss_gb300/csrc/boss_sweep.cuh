// boss_sweep.cuh -- device-side building blocks of the permanent sweeps.
//
// Every permanent in theboss's hot path is a signed, binomially weighted sum over
// the codes r of a reflected mixed-radix Gray ("Guan") code of a product of
// row sums:
//     sum_r  sign(r) * prod_i C(mult_i, r_i) * prod_f s_f(r),
//     s_f(r) = base_f + sum_i r_i * D_if
// where i runs over the iterated side's distinct modes ("digits", multiplicity
// mult_i, r_i in [0, mult_i]) and f over the product side's particles ("factors":
// a mode occupied p times contributes p identical factors, which is theboss's
// pow(sum, p)):
//   * Ryser (ryser_permanent_calculator.py:45-64): base = 0, D = U,
//     sign (-1)^(n + |r|);
//   * Glynn / Chin-Huh (chin_huh_permanent_calculator.py:38-59,
//     glynn_gray_permanent_calculator.py:41-84): base_f = sum_i mult_i U_if,
//     D = -2U, sign (-1)^|r|, scale 2^-n.
// The binomial weight follows bs_permanent_calculator_base.py:151-164.
//
// GB300 mapping.  The FP64 pipe issues 2 lanes/clk/SM, 1/64 of FP32, so only
// products and sums of products use it, and the integer pipes take what they can:
//   * the row sums are exact 64-bit fixed-point integers (value = int * 2^-fx),
//     updated with integer adds and converted to FP64 with integer instructions
//     (fx_to_double), so the 2 adds per factor and code leave the FP64 pipe and
//     the sums never drift;
//   * the first factors of every product are multiplied in block floating point
//     on the integer pipe (62-bit mantissas, accumulate_product_bf), the rest on
//     the FP64 pipe, 4 instructions per factor (accumulate_product);
//   * the last multiply of every product is fused into the accumulation (4 DFMA);
//   * sign flips are integer XORs on the sign bit.
//
// Work split: the codes of a sweep are cut into one contiguous range per thread
// (lengths differ by at most one), each thread decodes its start code in closed
// form and walks the Gray code: step t flips binary digit ctz(t); when ctz(t)
// reaches a multi-valued digit the thread re-decodes.  Binary digits are ordered
// first so that happens once per 2^nb codes.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace boss {

constexpr int kMaxDigits = 64;       // distinct modes on the iterated side
constexpr int kMaxFactors = 32;      // particles on the product side
constexpr int kMaxMinorDigits = 32;  // digits of an all-minors sweep
constexpr int kSegLog = 16;          // all-minors bookkeeping is settled every 2^16 codes

enum SweepKind : int32_t { kRyser = 0, kGlynn = 1 };

// One sweep (a permanent or an all-minors problem).  Plain old data in device
// memory; built by the host planner or by the sampler's device-side planner.
struct SweepProblem {
  int32_t nd;        // digits, binary ones first
  int32_t nb;        // leading binary digits
  int32_t nf;        // product factors
  int32_t kind;      // SweepKind
  int32_t parity0;   // sign parity of the r = 0 code
  int32_t fx;        // fixed-point fraction bits of the row sums
  int32_t has_base;  // base sums present
  int32_t out_idx;   // result index
  int64_t n_codes;       // codes in the sweep
  int64_t thread_begin;  // first global thread of this sweep
  int64_t n_threads;     // threads working on it
  int64_t mat_off;   // D: nd x nf fixed-point complex (longlong2), row-major
  int64_t base_off;  // nf fixed-point complex
  int64_t part_off;  // partials: n_threads complex (perms) or n_threads x (nd + fixed_digit) (all-minors)
  int64_t ff_off;    // float-pair all-minors only: nb x nf rows of D as float pairs (float4: re hi, re lo,
                     // im hi, im lo, each factor in its own scale), then nf int32 exponent biases
  double scale;      // final real scale
  int32_t fixed_digit;  // gradients, all-minors: a binary digit held at r = 0 (Glynn halving) adds a weight-1 row
  int32_t group;     // all-minors: each aligned group of `group` threads (1, 2, 4, .., 128; above 32 only when the
                     // launch's threads fill whole blocks) sums its minors, so the partials are
                     // (n_threads / group) x nd; n_threads and thread_begin are multiples of it, and
                     // every sweep of the launch has the same
  uint8_t mult[kMaxDigits];
};

// ---------------------------------------------------------------------------
// Integer-pipe helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ double xor_sign(double x, uint32_t neg_mask) {
  return __hiloint2double(__double2hiint(x) ^ (int)neg_mask, __double2loint(x));
}

// x * 2^-fx as a double, rounded to nearest (ties away from zero), using integer
// instructions only.  bias_exp = 1023 + 63 - fx.  Requires the result to be a
// normal double or zero.
__device__ __forceinline__ double fx_to_double(long long x, int bias_exp) {
  const unsigned long long sgn = (unsigned long long)(x >> 63);
  const unsigned long long ax = ((unsigned long long)x ^ sgn) - sgn;
  const int lz = __clzll((long long)ax);
  const unsigned long long y = ax << (lz & 63);
  const unsigned long long yr = y + 0x400ull;
  const unsigned long long carry = (yr < y) ? 1ull : 0ull;
  const unsigned long long mant = (yr >> 11) & 0xFFFFFFFFFFFFFull;
  const unsigned long long e = (unsigned long long)(bias_exp - lz) + carry;
  const unsigned long long bits = (sgn << 63) | (e << 52) | mant;
  return __longlong_as_double(ax ? (long long)bits : 0ll);
}

// Compiler-only barrier: keeps the scheduler from hoisting all of a row's loads
// at once (at large NF that alone would exhaust the register file).
__device__ __forceinline__ void load_fence() { asm volatile("" ::: "memory"); }

__device__ __forceinline__ double binom_small(int n, int k) {
  double r = 1.0;
  for (int i = 1; i <= k; ++i) r = r * (double)(n - k + i) / (double)i;
  return r;
}

// Digit value of code t: digit i is the plain mixed-radix digit d_i when the
// number of completed cycles of digits 0..i is even, mult_i - d_i when odd (the
// closed form of the reflected mixed-radix code); binary digits reduce to
// bit_i(t) ^ bit_(i+1)(t).
__device__ __forceinline__ uint32_t digit_value(const SweepProblem& P, uint64_t t, int i) {
  if (i < P.nb) return (uint32_t)(((t >> i) ^ (t >> (i + 1))) & 1ull);
  uint64_t th = t >> P.nb;
  uint32_t r = 0;
  for (int j = P.nb; j <= i; ++j) {
    const uint32_t mu = P.mult[j];
    const uint64_t b = (uint64_t)mu + 1ull;
    const uint64_t q = th / b;
    const uint32_t dgt = (uint32_t)(th - q * b);
    th = q;
    r = (q & 1ull) ? (mu - dgt) : dgt;
  }
  return r;
}

// Full state at code t: fixed-point sums, sign parity, binomial weight of the
// multi-valued digits, and the bits of the binary digits.
template <int NF>
__device__ __forceinline__ void decode_code(const SweepProblem& P, const longlong2* __restrict__ D,
                                            const longlong2* __restrict__ base, uint64_t t, long long (&sr)[NF],
                                            long long (&si)[NF], uint64_t& gbits, uint32_t& parity, double& weight) {
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    if (P.has_base) {
      const longlong2 b = base[f];
      sr[f] = b.x;
      si[f] = b.y;
    } else {
      sr[f] = 0;
      si[f] = 0;
    }
  }
  parity = (uint32_t)P.parity0;
  weight = 1.0;
  gbits = (t ^ (t >> 1));
  if (P.nb < 64) gbits &= (1ull << P.nb) - 1ull;
  uint64_t bits = gbits;
  while (bits) {
    const int i = __ffsll((long long)bits) - 1;
    bits &= bits - 1ull;
    parity ^= 1u;
    const longlong2* row = D + (size_t)i * NF;
#pragma unroll
    for (int f = 0; f < NF; ++f) {
      if (f > 0 && (f & 7) == 0) load_fence();
      const longlong2 d = row[f];
      sr[f] += d.x;
      si[f] += d.y;
    }
  }
  uint64_t th = t >> P.nb;
  for (int i = P.nb; i < P.nd; ++i) {
    const uint32_t mu = P.mult[i];
    const uint64_t b = (uint64_t)mu + 1ull;
    const uint64_t q = th / b;
    const uint32_t dgt = (uint32_t)(th - q * b);
    th = q;
    const uint32_t r = (q & 1ull) ? (mu - dgt) : dgt;
    if (r) {
      parity ^= (r & 1u);
      weight *= binom_small((int)mu, (int)r);
      const longlong2* row = D + (size_t)i * NF;
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        const longlong2 d = row[f];
        sr[f] += (long long)r * d.x;
        si[f] += (long long)r * d.y;
      }
    }
  }
}

// Binary digit i moves from `bit` to 1 - bit: sums +/-= D_i.
template <int NF>
__device__ __forceinline__ void flip_binary(const longlong2* __restrict__ D, int i, uint32_t bit, long long (&sr)[NF],
                                            long long (&si)[NF]) {
  const longlong2* row = D + (size_t)i * NF;
  const long long sgn = bit ? -1ll : 0ll;  // -x = (x ^ -1) + 1: one three-input add per word
  const long long one = (long long)bit;
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    if (f > 0 && (f & 7) == 0) load_fence();
    const longlong2 d = row[f];
    sr[f] = sr[f] + (d.x ^ sgn) + one;
    si[f] = si[f] + (d.y ^ sgn) + one;
  }
}

// ---------------------------------------------------------------------------
// 128-bit integer helpers for the exact products of two fixed-point factors.
// ---------------------------------------------------------------------------
struct I128 {
  unsigned long long lo;
  long long hi;
};
// High half of the signed 128-bit product (floor(a b / 2^64)); a host build uses __int128.
__host__ __device__ __forceinline__ long long mulhi_s64(long long a, long long b) {
#ifdef __CUDA_ARCH__
  return __mul64hi(a, b);
#else
  return (long long)(((__int128)a * (__int128)b) >> 64);
#endif
}
__host__ __device__ __forceinline__ int clz_u64(unsigned long long x) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}
__host__ __device__ __forceinline__ I128 mul_s64(long long a, long long b) {
  I128 r;
  r.lo = (unsigned long long)a * (unsigned long long)b;
  r.hi = mulhi_s64(a, b);
  return r;
}
__host__ __device__ __forceinline__ I128 add128(I128 x, I128 y) {
  I128 r;
  r.lo = x.lo + y.lo;
  r.hi = x.hi + y.hi + (r.lo < x.lo ? 1 : 0);
  return r;
}
__host__ __device__ __forceinline__ I128 sub128(I128 x, I128 y) {
  I128 r;
  r.lo = x.lo - y.lo;
  r.hi = x.hi - y.hi - (x.lo < y.lo ? 1 : 0);
  return r;
}
// ---------------------------------------------------------------------------
// Block floating point on the integer pipe.  A complex value is (re + i im) 2^e,
// two 64-bit integers sharing one exponent, normalised so that the larger
// component lies in [2^61, 2^62] in magnitude.  GB300 issues the 64-bit integer
// multiplies on its FMA pipe and the shifts and adds on its ALU pipe, both far
// faster than its FP64 pipe (2 lanes/clk/SM), so a chain of factors can be
// multiplied with no FP64 instruction at all:
//   * bf_pair: the exact 128-bit product of two fixed-point factors, truncated
//     once to 62 bits (relative error below 2^-60);
//   * bf_mul: the product of two normalised values from the high halves of the
//     four 64 x 64 -> 128-bit products (|product| >= 2^122 before the shift, two
//     truncations of one unit per component: relative error below 2^-56.5 of
//     the product's magnitude);
//   * bf_to_double: one rounding to FP64 (2^-53) at the end.
// An FP64 complex product errs by up to about 2^-52 of its magnitude, so a chain
// of these products is at least as accurate as the FP64 chain it replaces.
// ---------------------------------------------------------------------------
struct BFloat {
  long long re, im;
  int e;
};
__host__ __device__ __forceinline__ double bits_to_double(unsigned long long b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double d;
  __builtin_memcpy(&d, &b, sizeof d);
  return d;
#endif
}
// (re + i im) 2^e normalised, for |re|, |im| <= 2^62.  The shift comes from the
// leading bit of the one's-complement magnitudes (|x| or |x| - 1), so a negative
// power of two may land on -2^62; zero stays zero (its exponent drops by 62).
__host__ __device__ __forceinline__ BFloat bf_norm(long long re, long long im, int e) {
  const unsigned long long m = (unsigned long long)(re ^ (re >> 63)) | (unsigned long long)(im ^ (im >> 63));
  const int s = clz_u64(m) - 2;  // >= 0
  BFloat r;
  r.re = (long long)((unsigned long long)re << s);
  r.im = (long long)((unsigned long long)im << s);
  r.e = e - s;
  return r;
}
__host__ __device__ __forceinline__ int clz_u32(unsigned x) {
#ifdef __CUDA_ARCH__
  return __clz((int)x);
#else
  return x ? __builtin_clz(x) : 32;
#endif
}
// Bits [s, s + 32) of (hi, lo) for 0 <= s < 32 (and the left-shift form).
__host__ __device__ __forceinline__ unsigned fshr32(unsigned lo, unsigned hi, int s) {
#ifdef __CUDA_ARCH__
  return __funnelshift_r(lo, hi, s);
#else
  return (unsigned)((((unsigned long long)hi << 32) | lo) >> (s & 31));
#endif
}
__host__ __device__ __forceinline__ unsigned fshl32(unsigned lo, unsigned hi, int s) {
#ifdef __CUDA_ARCH__
  return __funnelshift_l(lo, hi, s);
#else
  return (unsigned)(((((unsigned long long)hi << 32) | lo) << (s & 31)) >> 32);
#endif
}
__host__ __device__ __forceinline__ unsigned lo32(long long x) { return (unsigned)(unsigned long long)x; }
__host__ __device__ __forceinline__ unsigned hi32(long long x) { return (unsigned)((unsigned long long)x >> 32); }
__host__ __device__ __forceinline__ long long join32(unsigned hi, unsigned lo) {
  return (long long)(((unsigned long long)hi << 32) | lo);
}
// One's-complement magnitude of a 64-bit value's high word (the leading bit of |x| or |x| - 1).
__host__ __device__ __forceinline__ unsigned mag_hi32(long long x) {
  const unsigned h = hi32(x);
  return h ^ (unsigned)((int)h >> 31);
}
__host__ __device__ __forceinline__ BFloat bf_mul(const BFloat& x, const BFloat& y) {
  // |x.re| ... |y.im| <= 2^62: every high half lies in [-2^60, 2^60], the sums in [-2^61, 2^61]
  const long long re = mulhi_s64(x.re, y.re) - mulhi_s64(x.im, y.im);
  const long long im = mulhi_s64(x.re, y.im) + mulhi_s64(x.im, y.re);
  // |x|, |y| >= 2^61, so |x y| 2^-64 >= 2^58 and the larger component is at least
  // 2^57: its leading bit is in the high word and the normalising shift is 0..5
  // (30 for a zero product, which stays zero).
  const int s = clz_u32(mag_hi32(re) | mag_hi32(im)) - 2;
  BFloat z;
  z.re = join32(fshl32(lo32(re), hi32(re), s), lo32(re) << (s & 31));
  z.im = join32(fshl32(lo32(im), hi32(im), s), lo32(im) << (s & 31));
  z.e = x.e + y.e + 64 - s;
  return z;
}
// The 128-bit value (hi, lo) shifted right by r (arithmetic; 1 <= r <= 63), low 64 bits.
__host__ __device__ __forceinline__ long long shr128_lo(I128 x, int r) {
  return (long long)((x.lo >> r) | ((unsigned long long)x.hi << (64 - r)));
}
// (a + ib)(c + id) 2^e for fixed-point factors |a|, |b|, |c|, |d| < 2^61: exact
// 128-bit products (|re|, |im| < 2^123), then one truncation to the normal form.
__host__ __device__ __forceinline__ BFloat bf_pair(long long a, long long b, long long c, long long d, int e) {
  const I128 re = sub128(mul_s64(a, c), mul_s64(b, d));
  const I128 im = add128(mul_s64(a, d), mul_s64(b, c));
  BFloat z;
  const unsigned mt = mag_hi32(re.hi) | mag_hi32(im.hi);
  if (mt != 0) {
    // |value| >= 2^96 (the usual case): the leading bit (127 - clz) lies in the top
    // word, below bit 123, so the shift r = 66 - clz is 32 + rp with rp in [3, 29]
    // and the result is two 32-bit funnel shifts per component.
    const int rp = 34 - clz_u32(mt);
    z.re = join32(fshr32(lo32(re.hi), hi32(re.hi), rp), fshr32(hi32((long long)re.lo), lo32(re.hi), rp));
    z.im = join32(fshr32(lo32(im.hi), hi32(im.hi), rp), fshr32(hi32((long long)im.lo), lo32(im.hi), rp));
    z.e = e + 32 + rp;
    return z;
  }
  const long long sr = re.hi >> 63, si = im.hi >> 63;
  const unsigned long long mh = (unsigned long long)(re.hi ^ sr) | (unsigned long long)(im.hi ^ si);
  if (mh != 0) {
    const int r = 66 - clz_u64(mh);  // the leading bit (127 - clz, below bit 96 here) goes to bit 61: r in [3, 34]
    z.re = shr128_lo(re, r);
    z.im = shr128_lo(im, r);
    z.e = e + r;
    return z;
  }
  // Both high halves are sign bits: |re|, |im| < 2^64 (about 2^-58 of the largest products).
  const unsigned long long ml = (re.lo ^ (unsigned long long)sr) | (im.lo ^ (unsigned long long)si);
  const int r = 2 - clz_u64(ml);  // in [-62, 2]
  if (r > 0) {
    z.re = shr128_lo(re, r);
    z.im = shr128_lo(im, r);
  } else {  // |value| < 2^62: the low half is the value
    z.re = (long long)(re.lo << -r);
    z.im = (long long)(im.lo << -r);
  }
  z.e = e + r;
  return z;
}
// x 2^e rounded to the nearest double (ties away from zero); integer instructions
// except outside FP64's normal range (rare), which goes through ldexp.
__host__ __device__ __forceinline__ double bf_to_double(long long x, int e) {
  const unsigned long long sgn = (unsigned long long)(x >> 63);
  const unsigned long long ax = ((unsigned long long)x ^ sgn) - sgn;
  const int lz = clz_u64(ax);
  const unsigned long long y = ax << (lz & 63);
  const unsigned long long yr = y + 0x400ull;
  const unsigned long long carry = (yr < y) ? 1ull : 0ull;
  const unsigned long long mant = (yr >> 11) & 0xFFFFFFFFFFFFFull;
  const int be = e + 1086 - lz + (int)carry;
  if (be >= 1 && be <= 2046 && ax != 0) return bits_to_double((sgn << 63) | ((unsigned long long)be << 52) | mant);
  return ax ? ldexp((double)x, e) : 0.0;
}
// Product of the fixed-point factors [LO, HI) (unit 2^efx each) as a balanced
// tree: exact pairs at the leaves, bf_mul above them.
template <int LO, int HI, int NF>
__host__ __device__ __forceinline__ BFloat bf_product(const long long (&sr)[NF], const long long (&si)[NF], int efx) {
  if constexpr (HI - LO == 1) {
    return bf_norm(sr[LO], si[LO], efx);
  } else if constexpr (HI - LO == 2) {
    return bf_pair(sr[LO], si[LO], sr[LO + 1], si[LO + 1], 2 * efx);
  } else {
    constexpr int MID = LO + 2 * ((HI - LO + 2) / 4);
    return bf_mul(bf_product<LO, MID, NF>(sr, si, efx), bf_product<MID, HI, NF>(sr, si, efx));
  }
}

// acc += sign * prod_f s_f with the first K factors multiplied in block floating
// point on the integer pipe and the others on the FP64 pipe (the last one fused
// into the accumulation).  K = NF leaves 2 FP64 adds per code.
template <int NF, int K>
__device__ __forceinline__ void accumulate_product_bf(const long long (&sr)[NF], const long long (&si)[NF],
                                                      int bias_exp, uint32_t neg_mask, double& ar, double& ai) {
  static_assert(K >= 2 && K <= NF, "block-float factors");
  const int efx = bias_exp - 1086;  // a factor's unit: 2^-fx
  const BFloat p = bf_product<0, K, NF>(sr, si, efx);
  double pr = bf_to_double(p.re, p.e), pi = bf_to_double(p.im, p.e);
  if constexpr (K == NF) {
    ar += xor_sign(pr, neg_mask);
    ai += xor_sign(pi, neg_mask);
  } else {
#pragma unroll
    for (int f = K; f < NF - 1; ++f) {
      const double br = fx_to_double(sr[f], bias_exp);
      const double bi = fx_to_double(si[f], bias_exp);
      const double t_re = fma(pr, br, -(pi * bi));
      const double t_im = fma(pr, bi, pi * br);
      pr = t_re;
      pi = t_im;
    }
    pr = xor_sign(pr, neg_mask);
    pi = xor_sign(pi, neg_mask);
    const double br = fx_to_double(sr[NF - 1], bias_exp);
    const double bi = fx_to_double(si[NF - 1], bias_exp);
    ar = fma(pr, br, ar);
    ar = fma(-pi, bi, ar);
    ai = fma(pr, bi, ai);
    ai = fma(pi, br, ai);
  }
}

// acc += sign * prod_f s_f on the FP64 pipe: complex products (4 instructions
// each), the last fused with the accumulation (4 DFMA): 4 (nf - 1) FP64
// instructions per code.
template <int NF>
__device__ __forceinline__ void accumulate_product(const long long (&sr)[NF], const long long (&si)[NF], int bias_exp,
                                                   uint32_t neg_mask, double& ar, double& ai) {
  if (NF == 1) {
    ar += xor_sign(fx_to_double(sr[0], bias_exp), neg_mask);
    ai += xor_sign(fx_to_double(si[0], bias_exp), neg_mask);
    return;
  }
  double pr = fx_to_double(sr[0], bias_exp), pi = fx_to_double(si[0], bias_exp);
#pragma unroll
  for (int f = 1; f < NF - 1; ++f) {
    const double br = fx_to_double(sr[f], bias_exp);
    const double bi = fx_to_double(si[f], bias_exp);
    const double t_re = fma(pr, br, -(pi * bi));
    const double t_im = fma(pr, bi, pi * br);
    pr = t_re;
    pi = t_im;
  }
  pr = xor_sign(pr, neg_mask);
  pi = xor_sign(pi, neg_mask);
  const double br = fx_to_double(sr[NF - 1], bias_exp);
  const double bi = fx_to_double(si[NF - 1], bias_exp);
  ar = fma(pr, br, ar);
  ar = fma(-pi, bi, ar);
  ai = fma(pr, bi, ai);
  ai = fma(pi, br, ai);
}

// ---------------------------------------------------------------------------
// Float pairs on the FP32 pipe.  GB300 issues FP32 at 64x the FP64 rate, so the
// float-pair all-minors sweep keeps each value as an unevaluated sum hi + lo of
// two floats (about 47 significant bits) and uses the classical error-free
// transformations: Knuth's two-sum, the FMA two-product and Dekker's fast
// two-sum (T. J. Dekker, "A floating-point technique for extending the available
// precision", Numer. Math. 18, 1971).
// ---------------------------------------------------------------------------

// x * 2^(fbias - 190) as hi + lo: the 24 leading bits of |x| in hi, the next 23
// (truncated) in lo.  With |x| < 2^(p + 1) and fbias = 189 - p the value is below
// 1 in magnitude and every exponent field stays in [41, 126].  Integer work only.
__device__ __forceinline__ void fx_to_ff(long long x, int fbias, float& hi, float& lo) {
  const unsigned long long sgn = (unsigned long long)(x >> 63);
  const unsigned long long ax = ((unsigned long long)x ^ sgn) - sgn;
  const int lz = __clzll((long long)ax);
  const unsigned long long y = ax << (lz & 63);
  const uint32_t yh = (uint32_t)(y >> 32), yl = (uint32_t)y;
  const int ex = fbias - lz;  // exponent field of the leading bit
  const uint32_t s32 = (uint32_t)sgn & 0x80000000u;
  const uint32_t hb = (((uint32_t)(ex - 1)) << 23) + (yh >> 8);  // the leading bit carries into the field
  const uint32_t nxt = __funnelshift_r(yl, yh, 17) & 0x7FFFFFu;  // bits 39..17 of y
  const uint32_t eb = ((uint32_t)(ex - 23)) << 23;
  const float l = __uint_as_float(eb | nxt) - __uint_as_float(eb);  // exact (Sterbenz)
  hi = ax ? __uint_as_float(hb | s32) : 0.0f;
  lo = ax ? __uint_as_float(__float_as_uint(l) ^ s32) : 0.0f;
}

struct ffc {  // complex float pair
  float rh, rl, ih, il;
};

// (h, l) += sg * (bh, bl), sg = +-1: two-sum of the high parts, the low parts
// added to its error, renormalised by a fast two-sum.
__device__ __forceinline__ void ff_acc(float& h, float& l, float sg, float bh, float bl) {
  const float s = fmaf(sg, bh, h);
  const float bb = s - h;
  const float err = (h - (s - bb)) + fmaf(sg, bh, -bb);
  const float lo = err + fmaf(sg, bl, l);
  h = s + lo;
  l = lo - (h - s);
}

// p + e = a * b up to the a_lo * b_lo term (the FMA two-product of the high parts
// plus the cross terms).  __fmul_rn: p must stay a rounded product, never fused
// into a later add.
__device__ __forceinline__ void ff_prod(float ah, float al, float bh, float bl, float& p, float& e) {
  p = __fmul_rn(ah, bh);
  e = fmaf(ah, bh, -p);
  e = fmaf(ah, bl, e);
  e = fmaf(al, bh, e);
}

// (p1 + e1) + sg * (p2 + e2), normalised.
__device__ __forceinline__ void ff_combine(float p1, float e1, float sg, float p2, float e2, float& h, float& l) {
  const float s = fmaf(sg, p2, p1);
  const float bb = s - p1;
  const float err = (p1 - (s - bb)) + fmaf(sg, p2, -bb);
  const float lo = err + fmaf(sg, e2, e1);
  h = s + lo;
  l = lo - (h - s);
}

__device__ __forceinline__ ffc ff_cmul(const ffc& a, const ffc& b) {
  float p1, e1, p2, e2, p3, e3, p4, e4;
  ff_prod(a.rh, a.rl, b.rh, b.rl, p1, e1);
  ff_prod(a.ih, a.il, b.ih, b.il, p2, e2);
  ff_prod(a.rh, a.rl, b.ih, b.il, p3, e3);
  ff_prod(a.ih, a.il, b.rh, b.rl, p4, e4);
  ffc r;
  ff_combine(p1, e1, -1.0f, p2, e2, r.rh, r.rl);
  ff_combine(p3, e3, 1.0f, p4, e4, r.ih, r.il);
  return r;
}

// The sweep's inner loop skips the renormalisations: a running sum's low part
// then collects the two-sums' exact errors (cascaded summation), and a product's
// low part stays within a few 2^-24 of the complex magnitude, so the next
// product's cross terms lose nothing measurable (about 2^-46 per product against
// 2^-48).  Sums are resynchronised or renormalised before they leave the loop.
__device__ __forceinline__ void ff_add_lazy(float& h, float& l, float sg, float bh, float bl) {
  const float s = fmaf(sg, bh, h);
  const float bb = s - h;
  const float err = (h - (s - bb)) + fmaf(sg, bh, -bb);
  h = s;
  l = err + fmaf(sg, bl, l);
}

__device__ __forceinline__ ffc ff_cmul_lazy(const ffc& a, const ffc& b) {
  float p1, e1, p2, e2, p3, e3, p4, e4;
  ff_prod(a.rh, a.rl, b.rh, b.rl, p1, e1);
  ff_prod(a.ih, a.il, b.ih, b.il, p2, e2);
  ff_prod(a.rh, a.rl, b.ih, b.il, p3, e3);
  ff_prod(a.ih, a.il, b.rh, b.rl, p4, e4);
  ffc r;
  r.rh = p1;
  r.rl = e1;
  ff_add_lazy(r.rh, r.rl, -1.0f, p2, e2);
  r.ih = p3;
  r.il = e3;
  ff_add_lazy(r.ih, r.il, 1.0f, p4, e4);
  return r;
}

// (h, l) * (bh, bl), normalised.
__device__ __forceinline__ void ff_mul(float& h, float& l, float bh, float bl) {
  float p, e;
  ff_prod(h, l, bh, bl, p, e);
  h = p + e;
  l = e - (h - p);
}

__device__ __forceinline__ double ff_to_double(float h, float l) { return (double)h + (double)l; }

// x as a float pair (hi = x rounded to float, lo = the rest rounded): 48 bits.
__device__ __forceinline__ void double_to_ff(double x, float& hi, float& lo) {
  hi = __double2float_rn(x);
  lo = __double2float_rn(x - (double)hi);
}

// |re + i im|^2 for float pairs (re = rs + rc, im = is + ic, unnormalised as a
// compensated sum leaves them), as a normalised float pair.
__device__ __forceinline__ float2 ff_abs2(float rs, float rc, float is, float ic) {
  float rh = rs + rc, ih = is + ic;
  float rl = rc - (rh - rs), il = ic - (ih - is);  // fast two-sums: |s| >= |c|, or s = 0
  float p, e, q, f;
  ff_prod(rh, rl, rh, rl, p, e);
  ff_prod(ih, il, ih, il, q, f);
  ff_combine(p, e, 1.0f, q, f, rh, rl);
  return make_float2(rh, rl);
}

// Compensated dot-product step (Ogita, Rump and Oishi, "Accurate sum and dot
// product", SIAM J. Sci. Comput. 26, 2005): s + c accumulates sg * a * b for
// float pairs a, b, the products' errors and the sums' errors collected in c.
__device__ __forceinline__ void ff_dot_acc(float& s, float& c, float sg, float ah, float al, float bh, float bl) {
  float p, e;
  ff_prod(ah, al, bh, bl, p, e);
  const float t = fmaf(sg, p, s);
  const float bb = t - s;
  const float q = (s - (t - bb)) + fmaf(sg, p, -bb);
  c += fmaf(sg, e, q);
  s = t;
}

__device__ __forceinline__ double warp_sum(double v) {
  // Fixed butterfly order: every lane ends with the same, run-to-run identical sum.
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// This thread's code range inside its sweep: lengths differ by at most one.
__device__ __forceinline__ void thread_range(const SweepProblem& P, int64_t q, int64_t& a, int64_t& len) {
  const int64_t per = P.n_codes / P.n_threads, rem = P.n_codes % P.n_threads;
  a = q * per + (q < rem ? q : rem);
  len = per + (q < rem ? 1 : 0);
}

// The same split in whole units of 2^c codes (lengths differ by at most one
// unit; the last unit of the sweep may be short).  Every range then starts at a
// multiple of 2^c, so at every step the lanes of a warp flip the same binary
// digit whenever that digit is below c: their per-digit updates touch the same
// row, and rows laid out by lane are read and written in whole lines.
__device__ __forceinline__ void thread_range_aligned(const SweepProblem& P, int64_t q, int c, int64_t& a,
                                                     int64_t& len) {
  const int64_t units = (P.n_codes + (1ll << c) - 1) >> c;
  const int64_t per = units / P.n_threads, rem = units % P.n_threads;
  a = (q * per + (q < rem ? q : rem)) << c;
  const int64_t want = (per + (q < rem ? 1 : 0)) << c;
  len = (a >= P.n_codes) ? 0 : (a + want <= P.n_codes ? want : P.n_codes - a);
}

__device__ __forceinline__ int find_problem(const SweepProblem* __restrict__ probs, int n, int64_t gt) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (probs[mid].thread_begin <= gt) lo = mid; else hi = mid - 1;
  }
  return lo;
}

}  // namespace boss
