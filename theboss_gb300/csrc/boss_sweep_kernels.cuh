// boss_sweep_kernels.cuh -- the sweep kernels, templated on the number of product
// factors NF so that the row sums live in registers with no padding.  Explicit
// instantiations are spread over boss_sweep_nf*.cu so they compile in parallel.
#pragma once
#include "boss_internal.h"

namespace boss {

// Factors of a single permanent's product chain multiplied in block floating
// point on the integer pipe (0: all on the FP64 pipe, accumulate_product<NF>).
template <int NF>
constexpr int kPermBF = NF >= 10 ? NF - 8 : (NF >= 2 ? NF : 0);

template <int NF>
__device__ __forceinline__ void perm_product(const long long (&sr)[NF], const long long (&si)[NF], int bias_exp,
                                             uint32_t neg_mask, double& ar, double& ai) {
  if constexpr (kPermBF<NF> >= 2)
    accumulate_product_bf<NF, kPermBF<NF>>(sr, si, bias_exp, neg_mask, ar, ai);
  else
    accumulate_product<NF>(sr, si, bias_exp, neg_mask, ar, ai);
}

// One permanent per sweep problem; every thread writes one complex partial.
template <int NF>
__global__ void __launch_bounds__(128, 3) perm_sweep_kernel(const SweepProblem* __restrict__ probs, int n_probs,
                                                         const longlong2* __restrict__ pool, int64_t total_threads,
                                                         double2* __restrict__ partials) {
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gt >= total_threads) return;
  const SweepProblem& P = probs[find_problem(probs, n_probs, gt)];
  const int64_t q = gt - P.thread_begin;
  int64_t a, len;
  thread_range(P, q, a, len);
  double tr = 0.0, ti = 0.0;
  if (len > 0) {
    const longlong2* D = pool + P.mat_off;
    const longlong2* base = pool + P.base_off;
    const int bias = 1023 + 63 - P.fx;
    const int nb = P.nb;
    long long sr[NF], si[NF];
    uint64_t g;
    uint32_t parity;
    double w;
    decode_code<NF>(P, D, base, (uint64_t)a, sr, si, g, parity, w);
    double ar = 0.0, ai = 0.0;
    perm_product<NF>(sr, si, bias, parity << 31, ar, ai);
    const uint64_t end = (uint64_t)(a + len);
    for (uint64_t t = (uint64_t)a + 1; t < end; ++t) {
      const int i = __ffsll((long long)t) - 1;
      if (i < nb) {
        const uint32_t bit = (uint32_t)(g >> i) & 1u;
        g ^= 1ull << i;
        flip_binary<NF>(D, i, bit, sr, si);
        parity ^= 1u;
      } else {  // a multi-valued digit moves: settle the weight and re-decode
        tr = fma(w, ar, tr);
        ti = fma(w, ai, ti);
        ar = 0.0;
        ai = 0.0;
        decode_code<NF>(P, D, base, t, sr, si, g, parity, w);
      }
      perm_product<NF>(sr, si, bias, parity << 31, ar, ai);
    }
    tr = fma(w, ar, tr);
    ti = fma(w, ai, ti);
  }
  partials[P.part_off + q] = make_double2(tr, ti);
}

// Closes the current segment of an all-minors sweep: every digit receives R
// times its weight w_j = mult_j - 2 r_j (binary digits: +-1) times prod C(mult, r),
// the held digit (row nd) R times 1 -- halved, see minors_sweep_kernel.
// M: this thread's minors, row j at M[j * STRIDE].
template <int STRIDE>
__device__ __forceinline__ void settle_minors(const SweepProblem& P, double2* M, double Rr, double Ri, double w,
                                              uint64_t g, uint64_t t_seg) {
  const double wr = 0.5 * w * Rr, wi = 0.5 * w * Ri;
  for (int j = 0; j < P.nb; ++j) {
    const uint32_t neg = (uint32_t)((g >> j) & 1ull) << 31;
    double2 v = M[j * STRIDE];
    v.x += xor_sign(wr, neg);
    v.y += xor_sign(wi, neg);
    M[j * STRIDE] = v;
  }
  for (int j = P.nb; j < P.nd; ++j) {
    const double f = (double)P.mult[j] - 2.0 * (double)digit_value(P, t_seg, j);
    double2 v = M[j * STRIDE];
    v.x = fma(wr, f, v.x);
    v.y = fma(wi, f, v.y);
    M[j * STRIDE] = v;
  }
  if (P.fixed_digit) {
    double2 v = M[P.nd * STRIDE];
    v.x += wr;
    v.y += wi;
    M[P.nd * STRIDE] = v;
  }
}

// Factors of the all-minors product chain multiplied in block floating point on
// the integer pipe (0: all on the FP64 pipe, accumulate_product<NF>): 8 up to 16
// factors (4 blocks per SM), nf - 8 above (3 blocks, more registers per thread).
template <int NF>
constexpr int kMinorsBF = NF >= 2 ? (NF < 8 ? NF : (NF <= 16 ? 8 : NF - 8)) : 0;

// Blocks of 128 threads per SM the all-minors kernel is compiled for: 4 (128
// registers, a few spilled words at NF 11..16) up to NF = 16, where the fourth
// block's warps hide more latency than the spills cost; 3 above.
template <int NF>
constexpr int kMinorsMinBlocks = NF <= 16 ? 4 : 3;

template <int NF>
__device__ __forceinline__ void minors_product(const long long (&sr)[NF], const long long (&si)[NF], int bias_exp,
                                               uint32_t neg_mask, double& ar, double& ai) {
  if constexpr (kMinorsBF<NF> >= 2)
    accumulate_product_bf<NF, kMinorsBF<NF>>(sr, si, bias_exp, neg_mask, ar, ai);
  else
    accumulate_product<NF>(sr, si, bias_exp, neg_mask, ar, ai);
}

// All-minors sweep (C&C-B), in Glynn form.  theboss sums each minor over the
// Ryser codes with r_i = 0 (bs_cc_ryser_submatrices_permanent_calculator.py:96-119).
// Here a row of variables x is appended: perm([U[T, S]; x]) = sum_i x_i S_i minor_i,
// and Glynn's formula for it gives
//     S_i minor_i = scale * sum_r sign(r) prod C(mult, r) w_i(r) prod_f s_f(r),
// w_i = mult_i - 2 r_i (s_f from the base sums with rows -2U): every code counts
// for every digit, and one single-occupied digit is held at r = 0 (Glynn's
// halving; its row has w = 1 and comes last) -- half of theboss's codes.  A
// running signed total R of the products is kept and a minor is touched only
// when its digit flips: w_i goes +1 -> -1 (or back), so the minor receives
// (w_before - w_after) R = +-2R.  The kernel accumulates half of every minor
// (flips add +-R, settles w R / 2); the problem's scale carries the factor 2.
// Segments of 2^16 codes (and every change of a multi-valued digit) are closed
// by settle_minors and R restarts from zero.  minors_walk is one thread's part
// (thread q of the sweep's threads); its minors live in shared memory, row j at
// M[j * STRIDE].
template <int NF, int STRIDE>
__device__ __forceinline__ void minors_walk(const SweepProblem& P, const longlong2* __restrict__ D,
                                            const longlong2* __restrict__ base, int64_t q, double2* M) {
  const int nd = P.nd + P.fixed_digit;
  for (int j = 0; j < nd; ++j) M[j * STRIDE] = make_double2(0.0, 0.0);
  int64_t a, len;
  thread_range(P, q, a, len);
  if (len > 0) {
    const int bias = 1023 + 63 - P.fx;
    const int nb = P.nb;
    const int low = nb < kSegLog ? nb : kSegLog;
    const bool weighted = P.nd > P.nb;
    long long sr[NF], si[NF];
    uint64_t g, t_seg = (uint64_t)a;
    uint32_t parity;
    double w;
    decode_code<NF>(P, D, base, (uint64_t)a, sr, si, g, parity, w);
    double Rr = 0.0, Ri = 0.0;
    minors_product<NF>(sr, si, bias, parity << 31, Rr, Ri);
    const uint64_t end = (uint64_t)(a + len);
    for (uint64_t t = (uint64_t)a + 1; t < end; ++t) {
      const int i = __ffsll((long long)t) - 1;
      if (i < low) {
        const uint32_t bit = (uint32_t)(g >> i) & 1u;
        double vr = Rr, vi = Ri;
        if (weighted) {
          vr *= w;
          vi *= w;
        }
        double2 v = M[i * STRIDE];
        v.x += xor_sign(vr, bit << 31);
        v.y += xor_sign(vi, bit << 31);
        M[i * STRIDE] = v;
        g ^= 1ull << i;
        flip_binary<NF>(D, i, bit, sr, si);
        parity ^= 1u;
      } else {
        settle_minors<STRIDE>(P, M, Rr, Ri, w, g, t_seg);
        Rr = 0.0;
        Ri = 0.0;
        t_seg = t;
        if (i < nb) {
          const uint32_t bit = (uint32_t)(g >> i) & 1u;
          g ^= 1ull << i;
          flip_binary<NF>(D, i, bit, sr, si);
          parity ^= 1u;
        } else {
          decode_code<NF>(P, D, base, t, sr, si, g, parity, w);
        }
      }
      minors_product<NF>(sr, si, bias, parity << 31, Rr, Ri);
    }
    settle_minors<STRIDE>(P, M, Rr, Ri, w, g, t_seg);
  }
}

// One launch over many all-minors sweeps (128 threads per block); every thread
// writes nd + held complex partials, or its group of `group` threads writes their sum.
template <int NF>
__global__ void __launch_bounds__(128, kMinorsMinBlocks<NF>) minors_sweep_kernel(const SweepProblem* __restrict__ probs, int n_probs,
                                                           const longlong2* __restrict__ pool, int64_t total_threads,
                                                           double2* __restrict__ partials, int64_t uniform_threads) {
  extern __shared__ double2 minors_smem[];
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gt >= total_threads) return;
  const SweepProblem& P =
      probs[uniform_threads > 0 ? (int)(gt / uniform_threads) : find_problem(probs, n_probs, gt)];
  const int64_t q = gt - P.thread_begin;
  const int nd = P.nd + P.fixed_digit;  // minors written per thread
  double2* M = minors_smem + threadIdx.x;
  minors_walk<NF, 128>(P, pool + P.mat_off, pool + P.base_off, q, M);
  const int G = P.group;
  if (G > 32) {
    // Groups of 64 or 128 threads (the planner allows them only when the launch's
    // threads fill whole blocks, so no thread of this block has exited): each warp
    // sums its lanes' minors (lane l: digit l, nd <= 32) into the warp's first
    // column of row l, then thread t of each group adds up digit t over its warps,
    // both in a fixed order.
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    __syncwarp();
    if (lane < nd) {
      const double2* row = minors_smem + lane * 128 + wp * 32;
      double sx = 0.0, sy = 0.0;
      for (int i = 0; i < 32; ++i) {
        const double2 v = row[(i + lane) & 31];  // staggered: fewer bank conflicts
        sx += v.x;
        sy += v.y;
      }
      minors_smem[lane * 128 + wp * 32] = make_double2(sx, sy);
    }
    __syncthreads();
    const int tin = threadIdx.x & (G - 1), w0 = (threadIdx.x - tin) >> 5;
    if (tin < nd) {
      double sx = 0.0, sy = 0.0;
      for (int wv = 0; wv < (G >> 5); ++wv) {
        const double2 v = minors_smem[tin * 128 + (w0 + wv) * 32];
        sx += v.x;
        sy += v.y;
      }
      partials[P.part_off + (q / G) * nd + tin] = make_double2(sx, sy);
    }
  } else if (G > 1) {  // each aligned group of G lanes (one sweep's threads) sums its minors:
                // lane l of the group adds up digits l, l + G, .. over the group, in a fixed order
    const int lane = threadIdx.x & 31;
    const int64_t warp0 = gt - lane;  // lanes past the launch's last thread have exited
    const unsigned live = (warp0 + 32 <= total_threads) ? 0xffffffffu : ((1u << (total_threads - warp0)) - 1u);
    __syncwarp(live);
    const int gl = lane & (G - 1);
    const double2* grp = minors_smem + (threadIdx.x - gl);
    double2* out = partials + P.part_off + (q / G) * nd;
    for (int j = gl; j < nd; j += G) {
      double sx = 0.0, sy = 0.0;
      for (int i = 0; i < G; ++i) {
        const double2 v = grp[j * 128 + ((i + gl) & (G - 1))];  // staggered: fewer bank conflicts
        sx += v.x;
        sy += v.y;
      }
      out[j] = make_double2(sx, sy);
    }
  } else {
    double2* out = partials + P.part_off + q * nd;
    for (int j = 0; j < nd; ++j) out[j] = M[j * 128];
  }
}

// ---------------------------------------------------------------------------
// Float-pair all-minors sweep: the same walk as minors_walk with every product,
// running total and minor kept as float pairs on the FP32 pipe (boss_sweep.cuh).
//   * Each factor f has its own scale 2^-(p_f + 1), |s_f| < 2^(p_f + 1) in
//     fixed-point units, so every float-pair factor is below 1 in magnitude and
//     the products neither overflow nor leave the normal range at the sizes of
//     the sampler; the planner folds 2^(sum_f (p_f + 1) - nf fx) into the scale.
//   * The exact 64-bit sums stay the reference, in shared memory (registers hold
//     the float-pair sums only): every kFFResync codes (counted from the
//     thread's first code, so the lanes of a warp resynchronise together) they
//     are brought up to the current code by the digits that flipped since, and
//     converted (fx_to_ff); in between the float-pair sums move by the
//     float-pair rows of D.  The drift between two resynchronisations is a few
//     units of 2^-47 of the rows per code in between.
// ---------------------------------------------------------------------------
constexpr int kFFMaxFactors = 24;  // above this the float-pair sums exhaust the registers
// Codes between two resynchronisations of the float-pair sums with the exact
// ones: the all-minors sweeps 32 (measured at n = 20, 10^4 samples: 8 -> 16 -> 32
// -> 64 gave 1.72, 1.55, 1.47, 1.43 ms per step, and max error against
// double-double at k = 22 of 2.9e-12, 3.6e-12, 5.6e-12, 6.8e-12), single
// permanents 16 (their larger sweeps cancel more).
constexpr uint64_t kFFResync = 32;
constexpr uint64_t kFFPermResync = 16;
// Resident blocks of 128 threads the register allocation must allow.
#ifndef BOSS_FF_MINB_LO
#define BOSS_FF_MINB_LO 4
#endif
#ifndef BOSS_FF_MINB_HI
#define BOSS_FF_MINB_HI 2
#endif
#ifndef BOSS_FF_SPLIT
#define BOSS_FF_SPLIT 12
#endif
template <int NF>
constexpr int kFFMinBlocks = NF <= BOSS_FF_SPLIT ? BOSS_FF_MINB_LO : BOSS_FF_MINB_HI;

// Decodes code t into the exact sums (shared memory, SS[f * 128]) and their
// float pairs S.
template <int NF>
__device__ __forceinline__ void decode_code_ff(const SweepProblem& P, const longlong2* __restrict__ D,
                                               const longlong2* __restrict__ base, const int* __restrict__ fb,
                                               uint64_t t, longlong2* SS, ffc (&S)[NF], uint64_t& g,
                                               uint32_t& parity, double& w) {
  long long sr[NF], si[NF];
  decode_code<NF>(P, D, base, t, sr, si, g, parity, w);
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    SS[f * 128] = make_longlong2(sr[f], si[f]);
    const int b = fb[f];
    fx_to_ff(sr[f], b, S[f].rh, S[f].rl);
    fx_to_ff(si[f], b, S[f].ih, S[f].il);
  }
}

// Brings the exact sums from code g_int to code g (the binary digits in which
// they differ) and reconverts the float pairs, one factor at a time.
template <int NF>
__device__ __forceinline__ void resync_ff(const longlong2* __restrict__ D, const int* __restrict__ fb, uint64_t g,
                                          uint64_t g_int, longlong2* SS, ffc (&S)[NF]) {
  const uint64_t diff = g ^ g_int;
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    longlong2 v = SS[f * 128];
    for (uint64_t dd = diff; dd; dd &= dd - 1) {
      const int j = __ffsll((long long)dd) - 1;
      const longlong2 d = D[(size_t)j * NF + f];
      const long long sgn = ((g_int >> j) & 1ull) ? -1ll : 0ll;  // r_j 1 -> 0 subtracts the row
      v.x += (d.x ^ sgn) - sgn;
      v.y += (d.y ^ sgn) - sgn;
    }
    SS[f * 128] = v;
    const int b = fb[f];
    fx_to_ff(v.x, b, S[f].rh, S[f].rl);
    fx_to_ff(v.y, b, S[f].ih, S[f].il);
  }
}

// settle_minors with float pairs: every digit's row receives w_j * w * R / 2.
template <int STRIDE>
__device__ __forceinline__ void settle_minors_ff(const SweepProblem& P, float4* M, const ffc& R, float wh, float wl,
                                                 uint64_t g, uint64_t t_seg) {
  float xr = R.rh, xlr = R.rl, xi = R.ih, xli = R.il;
  ff_mul(xr, xlr, 0.5f * wh, 0.5f * wl);  // halving is exact
  ff_mul(xi, xli, 0.5f * wh, 0.5f * wl);
  for (int j = 0; j < P.nb; ++j) {
    const float sg = ((g >> j) & 1ull) ? -1.0f : 1.0f;
    float4 v = M[j * STRIDE];
    ff_acc(v.x, v.y, sg, xr, xlr);
    ff_acc(v.z, v.w, sg, xi, xli);
    M[j * STRIDE] = v;
  }
  for (int j = P.nb; j < P.nd; ++j) {
    const float f = (float)((int)P.mult[j] - 2 * (int)digit_value(P, t_seg, j));  // small signed integer: exact
    float pr, er, pi, ei;
    ff_prod(xr, xlr, f, 0.0f, pr, er);
    ff_prod(xi, xli, f, 0.0f, pi, ei);
    float4 v = M[j * STRIDE];
    ff_acc(v.x, v.y, 1.0f, pr, er);
    ff_acc(v.z, v.w, 1.0f, pi, ei);
    M[j * STRIDE] = v;
  }
  if (P.fixed_digit) {
    float4 v = M[P.nd * STRIDE];
    ff_acc(v.x, v.y, 1.0f, xr, xlr);
    ff_acc(v.z, v.w, 1.0f, xi, xli);
    M[P.nd * STRIDE] = v;
  }
}

// One thread's part of a float-pair all-minors sweep (minors_walk's walk and
// bookkeeping).  DF: the nb x NF float-pair rows of D; fb: the factors' exponent
// biases for fx_to_ff; SS: this thread's exact sums (stride 128).
template <int NF, int STRIDE>
__device__ __forceinline__ void minors_walk_ff(const SweepProblem& P, const longlong2* __restrict__ D,
                                               const longlong2* __restrict__ base, const float4* __restrict__ DF,
                                               const int* __restrict__ fb, int64_t q, float4* M, longlong2* SS) {
  const int nd = P.nd + P.fixed_digit;
  for (int j = 0; j < nd; ++j) M[j * STRIDE] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  int64_t a, len;
  thread_range(P, q, a, len);
  if (len <= 0) return;
  const int nb = P.nb;
  const int low = nb < kSegLog ? nb : kSegLog;
  const bool weighted = P.nd > P.nb;
  uint64_t g, t_seg = (uint64_t)a;
  uint32_t parity;
  double w;
  ffc S[NF];
  decode_code_ff<NF>(P, D, base, fb, (uint64_t)a, SS, S, g, parity, w);
  uint64_t g_int = g;  // the code whose exact sums SS holds
  float wh = __double2float_rn(w), wl = __double2float_rn(w - (double)wh);
  ffc R = {0.0f, 0.0f, 0.0f, 0.0f};
  const uint64_t end = (uint64_t)(a + len);
  for (uint64_t t = (uint64_t)a;;) {
    {  // this code's product into the running total
      ffc p = S[0];
#pragma unroll
      for (int f = 1; f < NF; ++f) p = ff_cmul_lazy(p, S[f]);
      const float sg = parity ? -1.0f : 1.0f;
      ff_add_lazy(R.rh, R.rl, sg, p.rh, p.rl);
      ff_add_lazy(R.ih, R.il, sg, p.ih, p.il);
    }
    const uint64_t tn = t + 1;
    if (tn >= end) break;
    const int i = __ffsll((long long)tn) - 1;
    bool flips = true;  // false: a multi-valued digit moves and the code is re-decoded
    uint32_t bit = 0;
    if (i < low) {
      bit = (uint32_t)(g >> i) & 1u;
      float xr = R.rh, xlr = R.rl, xi = R.ih, xli = R.il;
      if (weighted) {
        ff_mul(xr, xlr, wh, wl);
        ff_mul(xi, xli, wh, wl);
      }
      const float sg = bit ? -1.0f : 1.0f;
      float4 v = M[i * STRIDE];
      ff_add_lazy(v.x, v.y, sg, xr, xlr);
      ff_add_lazy(v.z, v.w, sg, xi, xli);
      M[i * STRIDE] = v;
    } else {
      settle_minors_ff<STRIDE>(P, M, R, wh, wl, g, t_seg);
      R = {0.0f, 0.0f, 0.0f, 0.0f};
      t_seg = tn;
      if (i < nb) bit = (uint32_t)(g >> i) & 1u;
      else flips = false;
    }
    if (flips) {
      g ^= 1ull << i;
      parity ^= 1u;
      if (((tn - (uint64_t)a) & (kFFResync - 1)) == 0) {
        resync_ff<NF>(D, fb, g, g_int, SS, S);
        g_int = g;
      } else {
        const float sg = bit ? -1.0f : 1.0f;  // r_i 0 -> 1 adds the row
        const float4* row = DF + (size_t)i * NF;
#pragma unroll
        for (int f = 0; f < NF; ++f) {
          if (f > 0 && (f & 7) == 0) load_fence();
          const float4 d = row[f];
          ff_add_lazy(S[f].rh, S[f].rl, sg, d.x, d.y);
          ff_add_lazy(S[f].ih, S[f].il, sg, d.z, d.w);
        }
      }
    } else {
      decode_code_ff<NF>(P, D, base, fb, tn, SS, S, g, parity, w);
      g_int = g;
      wh = __double2float_rn(w);
      wl = __double2float_rn(w - (double)wh);
    }
    t = tn;
  }
  settle_minors_ff<STRIDE>(P, M, R, wh, wl, g, t_seg);
}

// minors_sweep_kernel with float pairs (NF <= kFFMaxFactors).  The group sums
// are float-pair sums in the same fixed order; the partials are written as
// float pairs (float4: re hi, re lo, im hi, im lo) in the factors' scales (the
// problem's scale carries the rest).
template <int NF>
__global__ void __launch_bounds__(128, kFFMinBlocks<NF>) minors_sweep_ff_kernel(const SweepProblem* __restrict__ probs, int n_probs,
                                                              const longlong2* __restrict__ pool, int64_t total_threads,
                                                              double2* __restrict__ partials, int rows,
                                                              int64_t uniform_threads) {
  extern __shared__ float4 minors_ff_smem[];
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gt >= total_threads) return;
  const SweepProblem& P =
      probs[uniform_threads > 0 ? (int)(gt / uniform_threads) : find_problem(probs, n_probs, gt)];
  const int64_t q = gt - P.thread_begin;
  const int nd = P.nd + P.fixed_digit;
  float4* M = minors_ff_smem + threadIdx.x;
  // exact sums after the launch's rows of minors (the launch passes rows in blockDim-sized units)
  longlong2* SS = reinterpret_cast<longlong2*>(minors_ff_smem + (size_t)rows * 128) + threadIdx.x;
  const float4* DF = reinterpret_cast<const float4*>(pool + P.ff_off);
  const int* fb = reinterpret_cast<const int*>(DF + (size_t)P.nb * NF);
  minors_walk_ff<NF, 128>(P, pool + P.mat_off, pool + P.base_off, DF, fb, q, M, SS);
  const int G = P.group;
  if (G > 32) {
    // Groups of 64 or 128 threads: the planner allows them only when the launch's
    // threads fill whole blocks, so no thread of this block has exited.  Each warp
    // sums its lanes' minors (lane l: digit l, nd <= 32) into row l's first column
    // of the warp, then thread t of each group adds up digit t over its warps.
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    __syncwarp();
    if (lane < nd) {
      const float4* row = minors_ff_smem + lane * 128 + wp * 32;
      float rh = 0.0f, rl = 0.0f, ih = 0.0f, il = 0.0f;
      for (int i = 0; i < 32; ++i) {
        const float4 v = row[(i + lane) & 31];
        ff_acc(rh, rl, 1.0f, v.x, v.y);
        ff_acc(ih, il, 1.0f, v.z, v.w);
      }
      minors_ff_smem[lane * 128 + wp * 32] = make_float4(rh, rl, ih, il);
    }
    __syncthreads();
    const int tin = threadIdx.x & (G - 1), w0 = (threadIdx.x - tin) >> 5;
    if (tin < nd) {
      float rh = 0.0f, rl = 0.0f, ih = 0.0f, il = 0.0f;
      for (int wv = 0; wv < (G >> 5); ++wv) {
        const float4 v = minors_ff_smem[tin * 128 + (w0 + wv) * 32];
        ff_acc(rh, rl, 1.0f, v.x, v.y);
        ff_acc(ih, il, 1.0f, v.z, v.w);
      }
      reinterpret_cast<float4*>(partials)[P.part_off + (q / G) * nd + tin] = make_float4(rh, rl, ih, il);
    }
  } else if (G > 1) {
    const int lane = threadIdx.x & 31;
    const int64_t warp0 = gt - lane;
    const unsigned live = (warp0 + 32 <= total_threads) ? 0xffffffffu : ((1u << (total_threads - warp0)) - 1u);
    __syncwarp(live);
    const int gl = lane & (G - 1);
    const float4* grp = minors_ff_smem + (threadIdx.x - gl);
    float4* out = reinterpret_cast<float4*>(partials) + P.part_off + (q / G) * nd;
    for (int j = gl; j < nd; j += G) {
      float rh = 0.0f, rl = 0.0f, ih = 0.0f, il = 0.0f;
      for (int i = 0; i < G; ++i) {
        const float4 v = grp[j * 128 + ((i + gl) & (G - 1))];
        ff_acc(rh, rl, 1.0f, v.x, v.y);
        ff_acc(ih, il, 1.0f, v.z, v.w);
      }
      out[j] = make_float4(rh, rl, ih, il);
    }
  } else {
    float4* out = reinterpret_cast<float4*>(partials) + P.part_off + q * nd;
    for (int j = 0; j < nd; ++j) out[j] = M[j * 128];
  }
}

// Single permanents with float pairs: perm_sweep_kernel's walk with the
// float-pair machinery of the all-minors sweep (exact sums in shared memory,
// resynchronised every kFFPermResync codes, lazily renormalised sums).  The products
// stay renormalised: a single permanent of 26-30 particles cancels more than the
// sampler's minors, and this keeps it 2-5x closer to double-double (n = 28:
// ~1e-11) at no measurable cost.  The float-pair running sum is folded into an
// FP64 accumulator every kFFPermFold codes: a lazily summed float pair loses
// about 2^-48 of its magnitude per addition, so left to run over a thread's whole
// range its error grows with the codes per thread -- with 64 permanents sharing
// one launch (each thread walking ~64x more codes than a lone permanent) n = 30
// measured 5.9e-10 against double-double.
// Each thread writes its partial as a float pair (float4) in the factors' scales.
constexpr int kFFPermMaxFactors = 32;
constexpr uint64_t kFFPermFold = 64;
template <int NF>
constexpr int kFFPermMinBlocks = NF <= 12 ? 4 : (NF <= 20 ? 3 : 2);

template <int NF>
__global__ void __launch_bounds__(128, kFFPermMinBlocks<NF>) perm_sweep_ff_kernel(
    const SweepProblem* __restrict__ probs, int n_probs, const longlong2* __restrict__ pool, int64_t total_threads,
    double2* __restrict__ partials) {
  extern __shared__ longlong2 perm_ff_smem[];
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gt >= total_threads) return;
  const SweepProblem& P = probs[find_problem(probs, n_probs, gt)];
  const int64_t q = gt - P.thread_begin;
  int64_t a, len;
  thread_range(P, q, a, len);
  double tr = 0.0, ti = 0.0;  // weighted total of the finished segments
  if (len > 0) {
    const longlong2* D = pool + P.mat_off;
    const longlong2* base = pool + P.base_off;
    const float4* DF = reinterpret_cast<const float4*>(pool + P.ff_off);
    const int* fb = reinterpret_cast<const int*>(DF + (size_t)P.nb * NF);
    longlong2* SS = perm_ff_smem + threadIdx.x;
    const int nb = P.nb;
    ffc S[NF];
    uint64_t g;
    uint32_t parity;
    double w;
    decode_code_ff<NF>(P, D, base, fb, (uint64_t)a, SS, S, g, parity, w);
    uint64_t g_int = g;
    ffc A = {0.0f, 0.0f, 0.0f, 0.0f};  // signed sum of products since the last fold
    double sr = 0.0, si = 0.0;         // this segment's folded sum
    const uint64_t end = (uint64_t)(a + len);
    for (uint64_t t = (uint64_t)a;;) {
      {
        ffc p = S[0];
#pragma unroll
        for (int f = 1; f < NF; ++f) p = ff_cmul(p, S[f]);
        const float sg = parity ? -1.0f : 1.0f;
        ff_add_lazy(A.rh, A.rl, sg, p.rh, p.rl);
        ff_add_lazy(A.ih, A.il, sg, p.ih, p.il);
      }
      const uint64_t tn = t + 1;
      if (tn >= end) break;
      const int i = __ffsll((long long)tn) - 1;
      if (i < nb) {
        const uint32_t bit = (uint32_t)(g >> i) & 1u;
        g ^= 1ull << i;
        parity ^= 1u;
        if (((tn - (uint64_t)a) & (kFFPermResync - 1)) == 0) {
          resync_ff<NF>(D, fb, g, g_int, SS, S);
          g_int = g;
          if (((tn - (uint64_t)a) & (kFFPermFold - 1)) == 0) {
            sr += ff_to_double(A.rh, A.rl);
            si += ff_to_double(A.ih, A.il);
            A = {0.0f, 0.0f, 0.0f, 0.0f};
          }
        } else {
          const float sg = bit ? -1.0f : 1.0f;
          const float4* row = DF + (size_t)i * NF;
#pragma unroll
          for (int f = 0; f < NF; ++f) {
            if (f > 0 && (f & 7) == 0) load_fence();
            const float4 d = row[f];
            ff_add_lazy(S[f].rh, S[f].rl, sg, d.x, d.y);
            ff_add_lazy(S[f].ih, S[f].il, sg, d.z, d.w);
          }
        }
      } else {  // a multi-valued digit moves: settle the segment with its weight, re-decode
        sr += ff_to_double(A.rh, A.rl);
        si += ff_to_double(A.ih, A.il);
        tr = fma(w, sr, tr);
        ti = fma(w, si, ti);
        A = {0.0f, 0.0f, 0.0f, 0.0f};
        sr = si = 0.0;
        decode_code_ff<NF>(P, D, base, fb, tn, SS, S, g, parity, w);
        g_int = g;
      }
      t = tn;
    }
    sr += ff_to_double(A.rh, A.rl);
    si += ff_to_double(A.ih, A.il);
    tr = fma(w, sr, tr);
    ti = fma(w, si, ti);
  }
  float4 o;
  double_to_ff(tr, o.x, o.y);
  double_to_ff(ti, o.z, o.w);
  reinterpret_cast<float4*>(partials)[P.part_off + q] = o;
}

// Gradient sweep (Glynn / Chin-Huh kind).  With s_f the factor sums and
// w_b = mult_b - 2 r_b the weight of digit b, d perm / d U[mode f][mode b] is
// scale * sum over the copies f of the mode of
//     G_{b,f} = sum_r sign(r) prod C(mult, r) w_b(r) L_f(r),  L_f = prod_{f' != f} s_f'
// (the derivative of the Chin-Huh sum; mult_b * copies(f) * minor once summed).
// Per code the leave-one-out products come from a prefix array (shared memory)
// and a running suffix, with the factors converted from the fixed-point sums in
// each pass, and sign * L_f is added to a running total R_f (shared memory).
// w_b only changes when digit b flips, so G is settled at flips:
// G_{b,.} += (w_b(before) - w_b(after)) * R_. , and at the end of each segment
// G_{b,.} += w_b * R_. for every digit.  A halved (fixed) digit has w = 1.
// The permanent itself is accumulated alongside (one fused product per code).
// Per-thread G lives in global scratch: (nd + fixed) x NF complex, row = digit,
// lane-interleaved within each group of 32 threads; each warp sums its lanes'
// rows at the end and leaves one group partial.
// Gradient ranges start at multiples of 2^kGradAlign codes (thread_range_aligned):
// the six lowest binary digits, which make 98% of the flips, then flip in step
// across a warp and their rows are updated in whole lines.
constexpr int kGradAlign = 6;

template <int NF>
__global__ void __launch_bounds__(64) grad_sweep_kernel(const SweepProblem* __restrict__ probs, int n_probs,
                                                        const longlong2* __restrict__ pool, int64_t total_threads,
                                                        double2* __restrict__ gpart, double2* __restrict__ ppart) {
  extern __shared__ double2 grad_smem[];
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gt >= total_threads) return;
  const SweepProblem& P = probs[find_problem(probs, n_probs, gt)];
  const int64_t q = gt - P.thread_begin;
  const int nd = P.nd, ndt = P.nd + P.fixed_digit;
  double2* R = grad_smem + threadIdx.x;             // running sign * L_f, R[f * 64]
  double2* Pp = grad_smem + NF * 64 + threadIdx.x;  // prefix products, Pp[f * 64]
  // Per-thread gradient slices are interleaved by lane within each group of 32
  // threads ([group][row][factor][lane]) so a warp's row updates coalesce.
  double2* G = gpart + P.part_off + (q >> 5) * (int64_t)(ndt * NF) * 32 + (q & 31);
  uint64_t touched = 0;  // rows of G written so far (the first write of a row stores, later ones add)
  double totr = 0.0, toti = 0.0;  // weighted permanent over finished segments
  int64_t a, len;
  thread_range_aligned(P, q, P.nb < kGradAlign ? P.nb : kGradAlign, a, len);
  const longlong2* D = pool + P.mat_off;
  const longlong2* base = pool + P.base_off;
  const int bias = 1023 + 63 - P.fx;
  const int nb = P.nb;
  const uint64_t end = (uint64_t)(a + len);
  // One walk over the thread's codes; a change of a multi-valued digit (every
  // 2^nb codes) settles the segment and re-decodes inside the loop, so the lanes
  // of a warp stay in step.
  if (len > 0) {
    long long sr[NF], si[NF];
    uint64_t g, seg = (uint64_t)a;
    uint32_t parity;
    double w;
    decode_code<NF>(P, D, base, seg, sr, si, g, parity, w);
#pragma unroll
    for (int f = 0; f < NF; ++f) R[f * 64] = make_double2(0.0, 0.0);
    double permr = 0.0, permi = 0.0;
    for (uint64_t t = seg; t < end; ++t) {
      // ---- this code: leave-one-out products into R, the full product into perm ----
      const uint32_t neg = parity << 31;
      if (NF == 1) {
        double2 v = R[0];
        v.x += xor_sign(1.0, neg);
        R[0] = v;
        permr += xor_sign(fx_to_double(sr[0], bias), neg);
        permi += xor_sign(fx_to_double(si[0], bias), neg);
      } else {
        // The factors are converted from the fixed-point sums twice (prefix and
        // suffix pass): integer work, cheaper than staging them in shared memory.
        double2 pv = make_double2(fx_to_double(sr[0], bias), fx_to_double(si[0], bias));
        Pp[0] = pv;
#pragma unroll
        for (int f = 1; f < NF - 1; ++f) {
          const double2 bv = make_double2(fx_to_double(sr[f], bias), fx_to_double(si[f], bias));
          const double t_re = fma(pv.x, bv.x, -(pv.y * bv.y));
          const double t_im = fma(pv.x, bv.y, pv.y * bv.x);
          pv = make_double2(t_re, t_im);
          Pp[f * 64] = pv;
        }
        load_fence();
        double2 qv = make_double2(fx_to_double(sr[NF - 1], bias), fx_to_double(si[NF - 1], bias));
        const double pnr = xor_sign(pv.x, neg), pni = xor_sign(pv.y, neg);
        permr = fma(pnr, qv.x, permr);
        permr = fma(-pni, qv.y, permr);
        permi = fma(pnr, qv.y, permi);
        permi = fma(pni, qv.x, permi);
        {
          double2 v = R[(NF - 1) * 64];
          v.x += pnr;
          v.y += pni;
          R[(NF - 1) * 64] = v;
        }
#pragma unroll
        for (int f = NF - 2; f >= 1; --f) {
          const double2 Pv = Pp[(f - 1) * 64];
          const double lr = xor_sign(Pv.x, neg), li = xor_sign(Pv.y, neg);
          double2 v = R[f * 64];
          v.x = fma(lr, qv.x, v.x);
          v.x = fma(-li, qv.y, v.x);
          v.y = fma(lr, qv.y, v.y);
          v.y = fma(li, qv.x, v.y);
          R[f * 64] = v;
          const double2 bv = make_double2(fx_to_double(sr[f], bias), fx_to_double(si[f], bias));
          const double nqr = fma(qv.x, bv.x, -(qv.y * bv.y));
          const double nqi = fma(qv.x, bv.y, qv.y * bv.x);
          qv = make_double2(nqr, nqi);
        }
        double2 v = R[0];
        v.x += xor_sign(qv.x, neg);
        v.y += xor_sign(qv.y, neg);
        R[0] = v;
        load_fence();
      }
      const uint64_t tn = t + 1;
      const bool last = (tn >= end);
      const int i = __ffsll((long long)tn) - 1;
      if (!last && i < nb) {
        // ---- a binary digit flips: its weight goes 1 - 2 bit -> 2 bit - 1 ----
        const uint32_t bit = (uint32_t)(g >> i) & 1u;
        const double cc = (bit ? -2.0 : 2.0) * w;
        double2* Gi = G + (size_t)i * NF * 32;
        if ((touched >> i) & 1ull) {
#pragma unroll
          for (int f = 0; f < NF; ++f) {
            if (f > 0 && (f & 7) == 0) load_fence();
            const double2 r = R[f * 64];
            double2 gv = Gi[f * 32];
            gv.x = fma(cc, r.x, gv.x);
            gv.y = fma(cc, r.y, gv.y);
            Gi[f * 32] = gv;
          }
        } else {
          touched |= 1ull << i;
#pragma unroll
          for (int f = 0; f < NF; ++f) {
            const double2 r = R[f * 64];
            Gi[f * 32] = make_double2(cc * r.x, cc * r.y);
          }
        }
        g ^= 1ull << i;
        flip_binary<NF>(D, i, bit, sr, si);
        parity ^= 1u;
      } else {
        // ---- end of a segment (or of the range): every digit receives its
        // current weight times R ----
        for (int bd = 0; bd < ndt; ++bd) {
          double wb;
          if (bd < nb) wb = ((g >> bd) & 1ull) ? -1.0 : 1.0;
          else if (bd < nd) wb = (double)P.mult[bd] - 2.0 * (double)digit_value(P, seg, bd);
          else wb = 1.0;
          wb *= w;
          double2* Gb = G + (size_t)bd * NF * 32;
          if ((touched >> bd) & 1ull) {
            for (int f = 0; f < NF; ++f) {
              const double2 r = R[f * 64];
              double2 gv = Gb[f * 32];
              gv.x = fma(wb, r.x, gv.x);
              gv.y = fma(wb, r.y, gv.y);
              Gb[f * 32] = gv;
            }
          } else {
            touched |= 1ull << bd;
            for (int f = 0; f < NF; ++f) {
              const double2 r = R[f * 64];
              Gb[f * 32] = make_double2(wb * r.x, wb * r.y);
            }
          }
        }
        totr = fma(w, permr, totr);
        toti = fma(w, permi, toti);
        permr = 0.0;
        permi = 0.0;
        if (!last) {
          for (int f = 0; f < NF; ++f) R[f * 64] = make_double2(0.0, 0.0);
          seg = tn;
          decode_code<NF>(P, D, base, tn, sr, si, g, parity, w);
        }
      }
    }
  }
  // Warp reduction of the 32 lanes' slices (the lane-interleaved layout makes
  // every read coalesced); lane e % 32 stores entry e of the group's partial.
  // Every lane of a warp belongs to the same sweep (thread counts are multiples of 32).
  const int ne = ndt * NF;
  const int lane = (int)(q & 31);
  double2* W = gpart + P.part_off + (q >> 5) * (int64_t)ne * 32;  // the group's slices, reused for the result
  for (int e = 0; e < ne; ++e) {
    const int bd = e / NF;
    double2 v = ((touched >> bd) & 1ull) ? G[(size_t)e * 32] : make_double2(0.0, 0.0);
    v.x = warp_sum(v.x);
    v.y = warp_sum(v.y);
    __syncwarp();
    if (lane == (e & 31)) W[e] = v;  // entry e of the group, compact at the start of its slices
    __syncwarp();
  }
  totr = warp_sum(totr);
  toti = warp_sum(toti);
  if (lane == 0) ppart[gt >> 5] = make_double2(totr, toti);
}

constexpr size_t kMinorsSmem = (size_t)kMaxMinorDigits * 128 * sizeof(double2);
constexpr size_t kGradSmem = (size_t)(2 * kMaxFactors) * 64 * sizeof(double2);

template <int NF>
cudaError_t sweep_launch_t(SweepOp op, const SweepLaunch& L, cudaStream_t st) {
  if (op == SweepOp::kGrad) {
    grad_sweep_kernel<NF><<<L.grid, 64, (size_t)(2 * NF) * 64 * sizeof(double2), st>>>(
        L.probs, L.n_probs, L.pool, L.total_threads, L.partials, L.partials2);
    return cudaGetLastError();
  }
  if (op == SweepOp::kMinorsFF) {
    if constexpr (NF <= kFFMaxFactors) {
      const int rows = (L.rows >= 1 && L.rows <= kMaxMinorDigits) ? L.rows : kMaxMinorDigits;
      minors_sweep_ff_kernel<NF><<<L.grid, 128, (size_t)(rows + NF) * 128 * sizeof(float4), st>>>(
          L.probs, L.n_probs, L.pool, L.total_threads, L.partials, rows, L.uniform_threads);
      return cudaGetLastError();
    } else {
      return cudaErrorInvalidValue;
    }
  }
  if (op == SweepOp::kPermFF) {
    perm_sweep_ff_kernel<NF><<<L.grid, 128, (size_t)NF * 128 * sizeof(longlong2), st>>>(
        L.probs, L.n_probs, L.pool, L.total_threads, L.partials);
    return cudaGetLastError();
  }
  if (op == SweepOp::kPerm) {
    perm_sweep_kernel<NF><<<L.grid, 128, 0, st>>>(L.probs, L.n_probs, L.pool, L.total_threads, L.partials);
  } else {  // shared memory: the launch's rows of minors per thread, 128 threads per block
    const int rows = (L.rows >= 1 && L.rows <= kMaxMinorDigits) ? L.rows : kMaxMinorDigits;
    minors_sweep_kernel<NF><<<L.grid, 128, (size_t)rows * 128 * sizeof(double2), st>>>(
        L.probs, L.n_probs, L.pool, L.total_threads, L.partials, L.uniform_threads);
  }
  return cudaGetLastError();
}

template <int NF>
cudaError_t grad_occupancy_t(int* blocks_per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, grad_sweep_kernel<NF>, 64,
                                                       (size_t)(2 * NF) * 64 * sizeof(double2));
}

// minors_blocks_per_sm[r] (r = 1..kMaxMinorDigits): blocks per SM with r rows of
// minors per thread in shared memory; ff_blocks_per_sm[r] the same for the
// float-pair kernel (left at 0 above kFFMaxFactors).
template <int NF>
cudaError_t sweep_prepare_t(int* perm_blocks_per_sm, int* minors_blocks_per_sm, int* ff_blocks_per_sm,
                            int* perm_ff_blocks_per_sm) {
  cudaError_t e = cudaFuncSetAttribute(minors_sweep_kernel<NF>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kMinorsSmem);
  if (e != cudaSuccess) return e;
  if constexpr (NF <= kFFMaxFactors) {
    e = cudaFuncSetAttribute(minors_sweep_ff_kernel<NF>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)((size_t)(kMaxMinorDigits + NF) * 128 * sizeof(float4)));
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(minors_sweep_ff_kernel<NF>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return e;
    for (int r = 1; r <= kMaxMinorDigits; ++r) {
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(ff_blocks_per_sm + r, minors_sweep_ff_kernel<NF>, 128,
                                                        (size_t)(r + NF) * 128 * sizeof(float4));
      if (e != cudaSuccess) return e;
    }
  } else {
    for (int r = 0; r <= kMaxMinorDigits; ++r) ff_blocks_per_sm[r] = 0;
  }
  e = cudaFuncSetAttribute(grad_sweep_kernel<NF>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGradSmem);
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(perm_blocks_per_sm, perm_sweep_kernel<NF>, 128, 0);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(perm_sweep_ff_kernel<NF>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)((size_t)NF * 128 * sizeof(longlong2)));
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(perm_sweep_ff_kernel<NF>, cudaFuncAttributePreferredSharedMemoryCarveout,
                           (int)cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(perm_ff_blocks_per_sm, perm_sweep_ff_kernel<NF>, 128,
                                                    (size_t)NF * 128 * sizeof(longlong2));
  if (e != cudaSuccess) return e;
  for (int r = 1; r <= kMaxMinorDigits; ++r) {
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(minors_blocks_per_sm + r, minors_sweep_kernel<NF>, 128,
                                                      (size_t)r * 128 * sizeof(double2));
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace boss

// Defines the dispatcher of one contiguous NF range [LO, LO + 7].
#define BOSS_SWEEP_RANGE(NAME, LO)                                                                       \
  namespace boss {                                                                                       \
  cudaError_t NAME##_launch(int nf, SweepOp op, const SweepLaunch& L, cudaStream_t st) {                 \
    switch (nf - (LO)) {                                                                                 \
      case 0: return sweep_launch_t<(LO) + 0>(op, L, st);                                                \
      case 1: return sweep_launch_t<(LO) + 1>(op, L, st);                                                \
      case 2: return sweep_launch_t<(LO) + 2>(op, L, st);                                                \
      case 3: return sweep_launch_t<(LO) + 3>(op, L, st);                                                \
      case 4: return sweep_launch_t<(LO) + 4>(op, L, st);                                                \
      case 5: return sweep_launch_t<(LO) + 5>(op, L, st);                                                \
      case 6: return sweep_launch_t<(LO) + 6>(op, L, st);                                                \
      case 7: return sweep_launch_t<(LO) + 7>(op, L, st);                                                \
      default: return cudaErrorInvalidValue;                                                             \
    }                                                                                                    \
  }                                                                                                      \
  cudaError_t NAME##_grad_occupancy(int nf, int* occ) {                                                  \
    switch (nf - (LO)) {                                                                                 \
      case 0: return grad_occupancy_t<(LO) + 0>(occ);                                                    \
      case 1: return grad_occupancy_t<(LO) + 1>(occ);                                                    \
      case 2: return grad_occupancy_t<(LO) + 2>(occ);                                                    \
      case 3: return grad_occupancy_t<(LO) + 3>(occ);                                                    \
      case 4: return grad_occupancy_t<(LO) + 4>(occ);                                                    \
      case 5: return grad_occupancy_t<(LO) + 5>(occ);                                                    \
      case 6: return grad_occupancy_t<(LO) + 6>(occ);                                                    \
      case 7: return grad_occupancy_t<(LO) + 7>(occ);                                                    \
      default: return cudaErrorInvalidValue;                                                             \
    }                                                                                                    \
  }                                                                                                      \
  cudaError_t NAME##_prepare(int* perm_occ, int* minors_occ, int* ff_occ, int* pff_occ) {                 \
    cudaError_t e;                                                                                       \
    for (int k = 0; k < 8; ++k) perm_occ[k] = 1;                                                         \
    for (int k = 0; k < 8; ++k) pff_occ[k] = 1;                                                          \
    for (int k = 0; k < 8 * 33; ++k) minors_occ[k] = 1;                                                  \
    for (int k = 0; k < 8 * 33; ++k) ff_occ[k] = 0;                                                      \
    if ((e = sweep_prepare_t<(LO) + 0>(perm_occ + 0, minors_occ + 0 * 33, ff_occ + 0 * 33, pff_occ + 0)) != cudaSuccess) return e;     \
    if ((e = sweep_prepare_t<(LO) + 1>(perm_occ + 1, minors_occ + 1 * 33, ff_occ + 1 * 33, pff_occ + 1)) != cudaSuccess) return e;     \
    if ((e = sweep_prepare_t<(LO) + 2>(perm_occ + 2, minors_occ + 2 * 33, ff_occ + 2 * 33, pff_occ + 2)) != cudaSuccess) return e;     \
    if ((e = sweep_prepare_t<(LO) + 3>(perm_occ + 3, minors_occ + 3 * 33, ff_occ + 3 * 33, pff_occ + 3)) != cudaSuccess) return e;     \
    if ((e = sweep_prepare_t<(LO) + 4>(perm_occ + 4, minors_occ + 4 * 33, ff_occ + 4 * 33, pff_occ + 4)) != cudaSuccess) return e;     \
    if ((e = sweep_prepare_t<(LO) + 5>(perm_occ + 5, minors_occ + 5 * 33, ff_occ + 5 * 33, pff_occ + 5)) != cudaSuccess) return e;     \
    if ((e = sweep_prepare_t<(LO) + 6>(perm_occ + 6, minors_occ + 6 * 33, ff_occ + 6 * 33, pff_occ + 6)) != cudaSuccess) return e;     \
    return sweep_prepare_t<(LO) + 7>(perm_occ + 7, minors_occ + 7 * 33, ff_occ + 7 * 33, pff_occ + 7);              \
  }                                                                                                      \
  }
