// boss_sweep.cuh -- device-side building blocks of the permanent sweeps.
//
// Every permanent in theboss's hot path is a signed, binomially weighted sum over
// the codes r of a reflected mixed-radix Gray ("Guan") code of
//     prod_l ( base_l + sgn * sum_i r_i * D_il ) ^ pw_l
// where i runs over the iterated side's distinct modes ("digits", multiplicity
// mult_i, r_i in [0, mult_i]) and l over the product side's distinct modes
// ("columns", power pw_l):
//   * Ryser   (ryser_permanent_calculator.py:45-64): base = 0, sgn = +1, D = U,
//               sign (-1)^(n + |r|);
//   * Glynn / Chin-Huh (chin_huh_permanent_calculator.py:38-59,
//     glynn_gray_permanent_calculator.py:41-84): base_l = sum_i mult_i U_il,
//               sgn = -1, D = 2U, sign (-1)^|r|, scale 2^-n.
// The weight is prod_i C(mult_i, r_i) (bs_permanent_calculator_base.py:151-164).
//
// GPU layout of one sweep: the digits are ordered binary-first (mult 1), then
// multi-valued.  The code range is cut into chunks of 2^c codes that only move
// the lowest c (binary) digits, so inside a chunk the flip sequence is the
// binary-reflected Gray code (step t flips digit ctz(t)) for every thread at
// once, the multi-valued digits and the binomial weight are constant, and each
// thread decodes its chunk's start code in closed form.  A warp owns 32
// consecutive chunks (one per lane) = one "work item"; sums stay in registers,
// the delta rows are warp-broadcast loads.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace boss {

constexpr int kMaxDigits = 64;      // distinct modes on the iterated side
constexpr int kMaxCols = 32;        // distinct modes on the product side
constexpr int kMaxMinorDigits = 32; // digits of an all-minors sweep
constexpr int kMaxChunkLog = 20;

enum SweepKind : int32_t { kRyser = 0, kGlynn = 1 };

// One sweep (one permanent, or one all-minors problem), built on the host or by
// the sampler's device-side planner.  Plain old data; lives in device memory.
struct SweepPlan {
  int32_t nd;        // digits (iterated side), binary ones first
  int32_t nb;        // number of leading binary digits
  int32_t c;         // log2(codes per chunk); c <= nb
  int32_t nc;        // product columns (0 < nc <= kMaxCols)
  int32_t kind;      // SweepKind
  int32_t parity0;   // sign parity of the r = 0 code
  int32_t has_base;  // Glynn/Chin-Huh: base sums present at base_off
  int32_t all_pow1;  // every column power is 1
  int64_t n_chunks;  // total codes >> c
  int64_t item_off;  // first work item of this sweep in the flat item space
  int64_t n_items;   // ceil(n_chunks / 32)
  int64_t mat_off;   // delta rows D: nd x nc complex, row-major, at pool + mat_off
  int64_t base_off;  // nc complex base sums (has_base)
  int64_t part_off;  // partial-result slot: perms use 1 complex / item, minors nd / item
  int64_t code_off;  // first code of this segment (a sweep may be cut into segments)
  int32_t out_idx;   // result this segment contributes to
  int32_t reserved;
  double scale;      // final real scale
  uint8_t mult[kMaxDigits];
  uint8_t pw[kMaxCols];
};

// ---------------------------------------------------------------------------
// FP64 helpers.  The GB300 FP64 pipe issues ~2 lanes/clk/SM, 1/64 of FP32, so
// everything that is not FP64 arithmetic (sign handling, index math, loads) is
// kept on the integer / load pipes.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double xor_sign(double x, uint32_t neg_mask) {
  // neg_mask is 0 or 0x80000000: flips the sign bit with one integer LOP.
  return __hiloint2double(__double2hiint(x) ^ (int)neg_mask, __double2loint(x));
}

__device__ __forceinline__ void cmul_acc(double& pr, double& pi, double br, double bi) {
  // (pr + i pi) *= (br + i bi): 2 DMUL + 2 DFMA.
  const double t_re = fma(pr, br, -(pi * bi));
  const double t_im = fma(pr, bi, pi * br);
  pr = t_re;
  pi = t_im;
}

__device__ __forceinline__ double binom_small(int n, int k) {
  // C(n, k) for n <= 255; exact in double for the multiplicities a sweep allows.
  double r = 1.0;
  for (int i = 1; i <= k; ++i) r = r * (double)(n - k + i) / (double)i;
  return r;
}

// Decodes the start code of a chunk (code number t0, low c bits zero) into the
// sweep state: starting sums, the sign parity, the binomial weight of the
// multi-valued digits, and the Gray bits of the low c digits.  The digit value
// is the closed form of the reflected mixed-radix code: digit i of code t is d_i
// (the plain mixed-radix digit) when the number of completed cycles of digits
// 0..i is even and mult_i - d_i otherwise; for binary digits that is
// bit_i(t) ^ bit_(i+1)(t).
template <int NC>
__device__ __forceinline__ void decode_chunk_start(const SweepPlan& P, const double2* __restrict__ D,
                                                   const double2* __restrict__ base, uint64_t t0,
                                                   double (&sr)[NC], double (&si)[NC], uint32_t& parity,
                                                   double& weight, uint32_t& gray_low) {
  const int nc = P.nc;
#pragma unroll
  for (int l = 0; l < NC; ++l) {
    if (l < nc) {
      if (P.has_base) {
        const double2 b = base[l];
        sr[l] = b.x;
        si[l] = b.y;
      } else {
        sr[l] = 0.0;
        si[l] = 0.0;
      }
    } else {
      sr[l] = 0.0;
      si[l] = 0.0;
    }
  }
  parity = (uint32_t)P.parity0;
  weight = 1.0;
  // Ryser adds r_i * D_i, Glynn subtracts it.
  const uint32_t sub_mask = (P.kind == kGlynn) ? 0x80000000u : 0u;
  for (int i = 0; i < P.nb; ++i) {
    const uint32_t r = (uint32_t)(((t0 >> i) ^ (t0 >> (i + 1))) & 1ull);
    if (r) {
      parity ^= 1u;
      const double2* row = D + (size_t)i * nc;
#pragma unroll
      for (int l = 0; l < NC; ++l) {
        if (l < nc) {
          const double2 d = row[l];
          sr[l] += xor_sign(d.x, sub_mask);
          si[l] += xor_sign(d.y, sub_mask);
        }
      }
    }
  }
  uint64_t th = t0 >> P.nb;
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
      const double coef = (P.kind == kGlynn) ? -(double)r : (double)r;
      const double2* row = D + (size_t)i * nc;
#pragma unroll
      for (int l = 0; l < NC; ++l) {
        if (l < nc) {
          const double2 d = row[l];
          sr[l] = fma(coef, d.x, sr[l]);
          si[l] = fma(coef, d.y, si[l]);
        }
      }
    }
  }
  const int c = P.c;
  gray_low = (c > 0) ? (uint32_t)((t0 >> c) & 1ull) << (c - 1) : 0u;
}

// prod_l s_l^pw_l.  nc >= 1.
template <int NC>
__device__ __forceinline__ void column_product(const SweepPlan& P, const double (&sr)[NC], const double (&si)[NC],
                                               double& pr, double& pi) {
  const int nc = P.nc;
  pr = sr[0];
  pi = si[0];
  if (P.all_pow1) {
#pragma unroll
    for (int l = 1; l < NC; ++l)
      if (l < nc) cmul_acc(pr, pi, sr[l], si[l]);
  } else {
    for (int q = 1; q < P.pw[0]; ++q) cmul_acc(pr, pi, sr[0], si[0]);
#pragma unroll
    for (int l = 1; l < NC; ++l) {
      if (l < nc) {
        const int p = P.pw[l];
        for (int q = 0; q < p; ++q) cmul_acc(pr, pi, sr[l], si[l]);
      }
    }
  }
}

// Moves digit i (a low, binary digit) from r_i = bit to 1 - bit.
template <int NC>
__device__ __forceinline__ void flip_digit(const SweepPlan& P, const double2* __restrict__ D, int i, uint32_t bit,
                                           double (&sr)[NC], double (&si)[NC]) {
  // Ryser: sums += (bit ? -D_i : +D_i).  Glynn: sums += (bit ? +D_i : -D_i).
  const uint32_t neg = ((bit ^ (uint32_t)(P.kind == kGlynn)) & 1u) ? 0x80000000u : 0u;
  const int nc = P.nc;
  const double2* row = D + (size_t)i * nc;
#pragma unroll
  for (int l = 0; l < NC; ++l) {
    if (l < nc) {
      const double2 d = row[l];
      sr[l] += xor_sign(d.x, neg);
      si[l] += xor_sign(d.y, neg);
    }
  }
}

__device__ __forceinline__ double warp_sum(double v) {
  // Fixed butterfly order: every lane ends with the same, run-to-run identical sum.
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

}  // namespace boss
