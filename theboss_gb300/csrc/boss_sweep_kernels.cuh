// boss_sweep_kernels.cuh -- the sweep kernels, templated on the number of product
// factors NF so that the row sums live in registers with no padding.  Explicit
// instantiations are spread over boss_sweep_nf*.cu so they compile in parallel.
#pragma once
#include "boss_internal.h"

namespace boss {

// One permanent per sweep problem; every thread writes one complex partial.
template <int NF>
__global__ void __launch_bounds__(128) perm_sweep_kernel(const SweepProblem* __restrict__ probs, int n_probs,
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
    accumulate_product<NF>(sr, si, bias, parity << 31, ar, ai);
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
      accumulate_product<NF>(sr, si, bias, parity << 31, ar, ai);
    }
    tr = fma(w, ar, tr);
    ti = fma(w, ai, ti);
  }
  partials[P.part_off + q] = make_double2(tr, ti);
}

// Closes the current segment of an all-minors sweep: every digit whose value is
// constant over the segment receives R times its weight
// (S_j - r_j) / S_j * prod C(S_l, r_l)
// (bs_cc_ryser_submatrices_permanent_calculator.py:96-119); binary digits get R
// when r_j = 0, which also closes the run the flip bookkeeping left open.
__device__ __forceinline__ void settle_minors(const SweepProblem& P, double2* M, double Rr, double Ri, double w,
                                             uint64_t g, uint64_t t_seg) {
  const double wr = w * Rr, wi = w * Ri;
  for (int j = 0; j < P.nb; ++j) {
    if (((g >> j) & 1ull) == 0ull) {
      double2 v = M[j * 128];
      v.x += wr;
      v.y += wi;
      M[j * 128] = v;
    }
  }
  for (int j = P.nb; j < P.nd; ++j) {
    const uint32_t r = digit_value(P, t_seg, j);
    const uint32_t mu = P.mult[j];
    if (r < mu) {
      const double f = (double)(mu - r) / (double)mu;
      double2 v = M[j * 128];
      v.x = fma(wr, f, v.x);
      v.y = fma(wi, f, v.y);
      M[j * 128] = v;
    }
  }
}

// All-minors sweep (C&C-B).  For a binary digit i the minor receives every code
// with r_i = 0.  A running signed total R of the products is kept and a minor is
// touched only when its digit flips: 0 -> 1 ends a run of r_i = 0 codes
// (minor += R), 1 -> 0 starts one (minor -= R).  Segments of 2^16 codes (and
// every change of a multi-valued digit) are closed by settle_minors and R
// restarts from zero.  Per-thread minors live in shared memory (digit-major,
// 128-thread stride); every thread writes nd complex partials.
template <int NF>
__global__ void __launch_bounds__(128) minors_sweep_kernel(const SweepProblem* __restrict__ probs, int n_probs,
                                                           const longlong2* __restrict__ pool, int64_t total_threads,
                                                           double2* __restrict__ partials) {
  extern __shared__ double2 minors_smem[];
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gt >= total_threads) return;
  const SweepProblem& P = probs[find_problem(probs, n_probs, gt)];
  const int64_t q = gt - P.thread_begin;
  const int nd = P.nd;
  double2* M = minors_smem + threadIdx.x;
  for (int j = 0; j < nd; ++j) M[j * 128] = make_double2(0.0, 0.0);
  int64_t a, len;
  thread_range(P, q, a, len);
  if (len > 0) {
    const longlong2* D = pool + P.mat_off;
    const longlong2* base = pool + P.base_off;
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
    accumulate_product<NF>(sr, si, bias, parity << 31, Rr, Ri);
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
        double2 v = M[i * 128];
        v.x += xor_sign(vr, bit << 31);
        v.y += xor_sign(vi, bit << 31);
        M[i * 128] = v;
        g ^= 1ull << i;
        flip_binary<NF>(D, i, bit, sr, si);
        parity ^= 1u;
      } else {
        settle_minors(P, M, Rr, Ri, w, g, t_seg);
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
      accumulate_product<NF>(sr, si, bias, parity << 31, Rr, Ri);
    }
    settle_minors(P, M, Rr, Ri, w, g, t_seg);
  }
  double2* out = partials + P.part_off + q * nd;
  for (int j = 0; j < nd; ++j) out[j] = M[j * 128];
}

constexpr size_t kMinorsSmem = (size_t)kMaxMinorDigits * 128 * sizeof(double2);

template <int NF>
cudaError_t sweep_launch_t(SweepOp op, const SweepLaunch& L, cudaStream_t st) {
  if (op == SweepOp::kPerm) {
    perm_sweep_kernel<NF><<<L.grid, 128, 0, st>>>(L.probs, L.n_probs, L.pool, L.total_threads, L.partials);
  } else {
    minors_sweep_kernel<NF><<<L.grid, 128, kMinorsSmem, st>>>(L.probs, L.n_probs, L.pool, L.total_threads,
                                                              L.partials);
  }
  return cudaGetLastError();
}

template <int NF>
cudaError_t sweep_prepare_t(int* perm_blocks_per_sm, int* minors_blocks_per_sm) {
  cudaError_t e = cudaFuncSetAttribute(minors_sweep_kernel<NF>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kMinorsSmem);
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(perm_blocks_per_sm, perm_sweep_kernel<NF>, 128, 0);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(minors_blocks_per_sm, minors_sweep_kernel<NF>, 128,
                                                       kMinorsSmem);
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
  cudaError_t NAME##_prepare(int* perm_occ, int* minors_occ) {                                           \
    cudaError_t e;                                                                                       \
    for (int k = 0; k < 8; ++k) perm_occ[k] = minors_occ[k] = 1;                                         \
    if ((e = sweep_prepare_t<(LO) + 0>(perm_occ + 0, minors_occ + 0)) != cudaSuccess) return e;          \
    if ((e = sweep_prepare_t<(LO) + 1>(perm_occ + 1, minors_occ + 1)) != cudaSuccess) return e;          \
    if ((e = sweep_prepare_t<(LO) + 2>(perm_occ + 2, minors_occ + 2)) != cudaSuccess) return e;          \
    if ((e = sweep_prepare_t<(LO) + 3>(perm_occ + 3, minors_occ + 3)) != cudaSuccess) return e;          \
    if ((e = sweep_prepare_t<(LO) + 4>(perm_occ + 4, minors_occ + 4)) != cudaSuccess) return e;          \
    if ((e = sweep_prepare_t<(LO) + 5>(perm_occ + 5, minors_occ + 5)) != cudaSuccess) return e;          \
    if ((e = sweep_prepare_t<(LO) + 6>(perm_occ + 6, minors_occ + 6)) != cudaSuccess) return e;          \
    return sweep_prepare_t<(LO) + 7>(perm_occ + 7, minors_occ + 7);                                      \
  }                                                                                                      \
  }
